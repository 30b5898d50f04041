"""The device-resident multiply service (hg_svc_*) on the GPU.

Every product the service runs must equal the same product computed alone
by hg_mul_device / hg_sqr_device, limb for limb, whether it ran alone in the
service or in a mix submitted from several threads while other batches were
on the device.  Admission must respect the per-slot workspace.
"""

import threading
import time

import numpy as np
import pytest

from hypergeometrica_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def _dev(a):
    import torch

    return torch.from_numpy(np.ascontiguousarray(a).view(np.int64)).cuda()


def _host(t):
    return t.cpu().numpy().view(np.uint64)


def _full(n):
    import torch

    return torch.full((n,), -1, dtype=torch.int64, device="cuda")


def _items(count, seed, lo_bits=0, hi_bits=13):
    sx = W.log_uniform_sizes(seed, count, lo_bits, hi_bits)
    sy = W.log_uniform_sizes(seed + 1, count, lo_bits, hi_bits)
    items = []
    for k in range(count):
        x = _dev(W.limbs(1000 * seed + 2 * k, int(sx[k])))
        sq = k % 9 == 4
        y = None if sq else _dev(W.limbs(1000 * seed + 2 * k + 1, int(sy[k])))
        nout = (2 * x.numel() if sq else x.numel() + y.numel()) + (3 if k % 4 == 1 else 0)
        items.append((x, y, _full(nout)))
    _sync()
    return items


def _sync():
    """The service's streams do not wait for torch's: inputs must be complete."""
    import torch

    torch.cuda.synchronize()


def _footprint(x, y):
    """Workspace bytes of one product: one or two operands x 3 primes x N words."""
    size = 2 * x.numel() if y is None else x.numel() + y.numel()
    n = 1 << max(0, (size - 1).bit_length())
    return (1 if y is None else 2) * 3 * n * 8


def _alone(items):
    from hypergeometrica_gb300 import device as D

    want = []
    for x, y, out in items:
        o = _full(out.numel())
        if y is None:
            D.sqr(x, o)
        else:
            D.mul(x, y, o)
        want.append(o)
    D.sync()
    _sync()
    return [_host(o) for o in want]


def test_service_matches_single_products(hg):
    from hypergeometrica_gb300 import device as D

    items = _items(300, 3)
    want = _alone(items)
    with D.Service(workspace_bytes=256 << 20, slots=2) as svc:
        tickets = svc.submit(items)
        svc.wait_all(timeout=120)
        for t in tickets:
            assert svc.status(t) == 1
        st = svc.stats()
    for k, (_, _, out) in enumerate(items):
        assert np.array_equal(_host(out), want[k]), k
    assert st["completed"] == 300 and st["failed"] == 0
    assert st["p50_us"] > 0 and st["p99_us"] >= st["p50_us"]
    assert st["peak_batch_workspace_bytes"] <= st["slot_workspace_bytes"]


def test_same_alone_and_in_the_mix(hg):
    """Products run alone in the service, then again in a mix that three
    threads submit at staggered times while earlier batches are running."""
    from hypergeometrica_gb300 import device as D

    big = _items(6, 11, 14, 15)  # transform 2^15..2^16
    small = _items(400, 12, 0, 10)
    mid = _items(60, 13, 10, 13)
    groups = [big, small, mid]
    want = [_alone(g) for g in groups]
    with D.Service(workspace_bytes=64 << 20, slots=2, max_batch=64) as svc:
        # alone: one product at a time
        for g in groups:
            for x, y, out in g[:3]:
                (t,) = svc.submit([(x, y, out)])
                svc.wait(t, timeout=60)
        for gi, g in enumerate(groups):
            for k, (_, _, out) in enumerate(g[:3]):
                assert np.array_equal(_host(out), want[gi][k]), (gi, k)
        for g in groups:
            for _, _, out in g:
                out.fill_(-1)
        _sync()
        svc.stats(reset=True)
        errors = []

        def client(g, delay, chunk):
            try:
                time.sleep(delay)
                for s in range(0, len(g), chunk):
                    svc.submit(g[s: s + chunk])
                    time.sleep(0.0005)
            except Exception as e:  # surfaced below
                errors.append(e)

        th = [threading.Thread(target=client, args=(g, d, c))
              for g, d, c in ((big, 0.0, 2), (small, 0.001, 25), (mid, 0.002, 7))]
        for t in th:
            t.start()
        for t in th:
            t.join()
        assert not errors, errors
        svc.wait_all(timeout=120)
        st = svc.stats()
    for gi, g in enumerate(groups):
        for k, (_, _, out) in enumerate(g):
            assert np.array_equal(_host(out), want[gi][k]), (gi, k)
    n = sum(len(g) for g in groups)
    assert st["completed"] >= n and st["latency_samples"] == n
    assert st["batches"] >= 2
    assert st["peak_batch_products"] <= 64


def test_admission_by_workspace(hg):
    from hypergeometrica_gb300 import device as D
    from hypergeometrica_gb300._lib import HG_ERR_ARG, HGError

    # 2 slots x 4 MiB: a 2^17-point product (6 MiB of residues) does not fit
    with D.Service(workspace_bytes=8 << 20, slots=2) as svc:
        x = _dev(W.limbs(5, 70000))
        y = _dev(W.limbs(6, 60000))
        with pytest.raises(HGError) as e:
            svc.submit([(x, y, _full(130000))])
        assert e.value.code == HG_ERR_ARG and "workspace" in str(e.value)
        # 2^13-point products (384 KiB each): at most 10 per 4 MiB slot
        items = _items(64, 21, 11, 12)
        want = _alone(items)
        svc.submit(items)
        svc.wait_all(timeout=60)
        st = svc.stats()
        assert st["peak_batch_workspace_bytes"] <= st["slot_workspace_bytes"]
        total = sum(_footprint(x, y) for x, y, _ in items)
        assert st["batches"] >= -(-total // st["slot_workspace_bytes"])
    for k, (_, _, out) in enumerate(items):
        assert np.array_equal(_host(out), want[k]), k


def test_records_submission_and_shutdown_guard(hg):
    import ctypes

    from hypergeometrica_gb300 import _lib
    from hypergeometrica_gb300 import device as D

    items = _items(40, 31, 0, 8)
    want = _alone(items)
    rec = D.product_records([x.data_ptr() for x, _, _ in items], [x.numel() for x, _, _ in items],
                            [0 if y is None else y.data_ptr() for _, y, _ in items],
                            [0 if y is None else y.numel() for _, y, _ in items],
                            [o.data_ptr() for _, _, o in items], [o.numel() for _, _, o in items])
    svc = D.Service(workspace_bytes=32 << 20, slots=1)
    try:
        tickets = svc.submit_records(rec)
        svc.wait(tickets[-1], timeout=60)
        svc.wait_all(timeout=60)
        assert _lib.load().hg_shutdown() == _lib.HG_ERR_ARG  # refused while a service is open
        buf = ctypes.create_string_buffer(256)
        _lib.load().hg_last_error(buf, 256)
        assert b"service" in buf.value
    finally:
        svc.close()
    for k, (_, _, out) in enumerate(items):
        assert np.array_equal(_host(out), want[k]), k


def test_bounded_waits_time_out_then_finish(hg):
    """hg_svc_wait and hg_svc_wait_all give up with HG_ERR_TIMEOUT when their
    limit runs out before the products finish; the products still finish,
    and a later wait without a limit returns them complete and exact.  The
    limit runs out on the host: nothing on the GPU is made to wait."""
    from hypergeometrica_gb300 import device as D
    from hypergeometrica_gb300._lib import HG_ERR_TIMEOUT, HGError

    n = 1 << 22
    items = []
    for k in range(3):
        x = _dev(W.limbs(600 + 2 * k, n))
        y = _dev(W.limbs(601 + 2 * k, n))
        items.append((x, y, _full(2 * n)))
    _sync()
    want = _alone(items)
    for _, _, out in items:
        out.fill_(-1)
    _sync()
    # one 2^23-point product at a time per slot: several milliseconds each
    with D.Service(workspace_bytes=2 * 420 << 20, slots=1, max_batch=1) as svc:
        tickets = svc.submit(items)
        with pytest.raises(HGError) as e:
            svc.wait(tickets[-1], timeout=1e-6)
        assert e.value.code == HG_ERR_TIMEOUT and "not finished" in str(e.value)
        with pytest.raises(HGError) as e:
            svc.wait_all(timeout=1e-6)
        assert e.value.code == HG_ERR_TIMEOUT
        assert svc.status(tickets[-1]) == 0  # still pending or running
        svc.wait(tickets[-1])
        svc.wait_all(timeout=120)
        assert all(svc.status(t) == 1 for t in tickets)
        st = svc.stats()
    assert st["completed"] == 3 and st["failed"] == 0
    for k, (_, _, out) in enumerate(items):
        assert np.array_equal(_host(out), want[k]), k
