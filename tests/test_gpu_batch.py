"""Batched products (hg_batch_*, hg_mul_batch_device) on the GPU.

Each product of a batch must equal the same product computed alone (and the
oracle's, on a sample), whatever schedule the autotuner picks, and a batch
captured in a CUDA graph must give the same limbs on every replay.
"""

import numpy as np
import pytest

from hypergeometrica_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def _dev(a):
    import torch

    return torch.from_numpy(np.ascontiguousarray(a).view(np.int64)).cuda()


def _host(t):
    return t.cpu().numpy().view(np.uint64)


def _make(count, seed, lo_bits=6, hi_bits=14, squares=True, extra_out=0):
    """Operands with sizes log-uniform in [2^lo, 2^hi] (seeded)."""
    import torch

    sx = W.log_uniform_sizes(seed, count, lo_bits, hi_bits)
    sy = W.log_uniform_sizes(seed + 1, count, lo_bits, hi_bits)
    items, host = [], []
    for k in range(count):
        x = W.limbs(10 * seed + 2 * k, int(sx[k]))
        sq = squares and k % 7 == 3
        y = None if sq else W.limbs(10 * seed + 2 * k + 1, int(sy[k]))
        nout = (2 * len(x) if sq else len(x) + len(y)) + (extra_out if k % 5 == 0 else 0)
        out = torch.full((nout,), -1, dtype=torch.int64, device="cuda")
        items.append((_dev(x), None if y is None else _dev(y), out))
        host.append((x, y))
    return items, host


def _single(hg, x, y, nout):
    """The same product alone through the single-product device entry points."""
    import torch

    from hypergeometrica_gb300 import device as D

    out = torch.empty(nout, dtype=torch.int64, device="cuda")
    if y is None:
        D.sqr(_dev(x), out)
    else:
        D.mul(_dev(x), _dev(y), out)
    D.sync()
    return _host(out)


def test_batch_matches_single_products(hg, oracle):
    from hypergeometrica_gb300 import device as D

    items, host = _make(300, 5, extra_out=37)
    D.mul_batch(items)
    D.sync()
    for k, ((x, y), it) in enumerate(zip(host, items)):
        got = _host(it[2])
        assert np.array_equal(got, _single(hg, x, y, len(got))), k
        if k % 25 == 0:
            ref = oracle.mpz_square(x) if y is None else oracle.mpz_mul_ntt(x, y)
            m = min(len(ref), len(got))
            assert np.array_equal(got[:m], ref[:m]) and not got[m:].any() and not ref[m:].any(), k


def test_batch_autotuned_and_graph_replay(hg):
    import torch

    from hypergeometrica_gb300 import device as D

    items, host = _make(400, 9)
    D.mul_batch(items)
    D.sync()
    want = [_host(it[2]).copy() for it in items]
    for it in items:
        it[2].fill_(-1)
    b = D.Batch(items, autotune=True)
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        b.run(s)
    s.synchronize()
    D.sync()
    for k, it in enumerate(items):
        assert np.array_equal(_host(it[2]), want[k]), k
    # capture the steady-state launch sequence and replay it twice
    for it in items:
        it[2].fill_(-1)
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=s):
        b.run(s)
    for _ in range(2):
        for it in items:
            it[2].fill_(-1)
        g.replay()
        torch.cuda.synchronize()
        D.sync()
        for k, it in enumerate(items):
            assert np.array_equal(_host(it[2]), want[k]), k
    b.close()


def test_batch_edge_products(hg):
    import torch

    from hypergeometrica_gb300 import device as D

    items = []
    ones = W.limbs(0, 5000, "ones")
    # empty operand, 1x1, all-ones (longest carries), square, sizes around 4096
    specs = [(0, 7), (1, 1), (5000, 5000), (4096, None), (2049, 2047), (3, 4093), (7, 1)]
    for nx, ny in specs:
        x = ones[:nx] if nx else np.zeros(0, dtype=np.uint64)
        y = None if ny is None else W.limbs(ny, ny, "uniform")
        nout = max(1, (2 * nx if y is None else nx + ny)) + 3
        xt = _dev(x) if nx else torch.zeros(1, dtype=torch.int64, device="cuda")
        items.append((xt, None if y is None else _dev(y), torch.full((nout,), -1, dtype=torch.int64, device="cuda"),
                      nx, None if y is None else ny))
    D.mul_batch(items)
    D.sync()
    for (nx, ny), it in zip(specs, items):
        got = _host(it[2])
        x = ones[:nx]
        xi = int.from_bytes(x.astype("<u8").tobytes(), "little") if nx else 0
        if ny is None:
            want = xi * xi
        else:
            yv = W.limbs(ny, ny, "uniform")
            want = xi * int.from_bytes(yv.astype("<u8").tobytes(), "little")
        assert int.from_bytes(got.astype("<u8").tobytes(), "little") == want, (nx, ny)


def test_batch_all_ones_carries(hg):
    """(2^(64n) - 1)(2^(64m) - 1): runs of zero limbs that only a carry
    rippling through whole 4096-limb tiles produces, in products that share a
    batch with uniform ones (the carry's second launch stops at each
    product's first tile)."""
    import torch

    from hypergeometrica_gb300 import device as D

    ones = W.limbs(0, 20000, "ones")
    specs = [(5000, 5000), (9000, 4000), (12000, None), (20000, 13000), (3000, 2500)]
    items, want = [], []
    for k, (nx, ny) in enumerate(specs):
        x = ones[:nx]
        y = None if ny is None else (ones[:ny] if k != 4 else W.limbs(77, ny, "uniform"))
        nout = (2 * nx if y is None else nx + ny) + 2
        items.append((_dev(x), None if y is None else _dev(y), torch.full((nout,), -1, dtype=torch.int64,
                                                                          device="cuda")))
        xi = int.from_bytes(x.astype("<u8").tobytes(), "little")
        yi = xi if y is None else int.from_bytes(y.astype("<u8").tobytes(), "little")
        want.append(xi * yi)
    D.mul_batch(items)
    D.sync()
    for k, it in enumerate(items):
        got = int.from_bytes(_host(it[2]).astype("<u8").tobytes(), "little")
        assert got == want[k], specs[k]
        assert _single(hg, _host(it[0]), None if it[1] is None else _host(it[1]), it[2].numel()).tobytes() == \
            _host(it[2]).tobytes(), specs[k]


def test_graph_capture_before_any_warm_run(hg):
    """A batch captured into a CUDA graph on its first run, for a transform
    length (2^16) no earlier test in this file builds inter-pass tables for,
    replays bit-identically to the single product computed afterwards."""
    import torch

    from hypergeometrica_gb300 import device as D

    nx, ny = 5 * 4096 + 17, 3 * 4096 + 5
    x = _dev(W.limbs(901, nx))
    y = _dev(W.limbs(902, ny))
    out = torch.full((nx + ny,), -1, dtype=torch.int64, device="cuda")
    b = D.Batch([(x, y, out)], autotune=False)
    s = torch.cuda.Stream()
    g = torch.cuda.CUDAGraph()
    torch.cuda.synchronize()
    with torch.cuda.graph(g, stream=s):
        b.run(s)
    got = []
    for _ in range(2):
        out.fill_(-1)
        g.replay()
        torch.cuda.synchronize()
        got.append(out.clone())
    want = torch.full((nx + ny,), -1, dtype=torch.int64, device="cuda")
    D.mul(x, y, want)
    D.sync()
    assert torch.equal(got[0], want) and torch.equal(got[1], want)


@pytest.mark.parametrize("seed,count,lo,hi", [(21, 500, 0, 14), (22, 40, 10, 16), (23, 6, 14, 17), (24, 2, 20, 20)])
def test_persistent_launch_matches_per_pass(hg, seed, count, lo, hi):
    """The whole batch as one persistent launch (a work list of group, pass
    and tile items) gives the same limbs as the per-pass schedule and as the
    products computed alone: transform lengths from 2^1 (the in-register
    transforms) to 2^21, squares, result
    tails past the product, and an empty operand; 2^21-point products run
    two strided passes each way."""
    import torch

    from hypergeometrica_gb300 import device as D

    items, host = _make(count, seed, lo_bits=lo, hi_bits=hi, extra_out=9)
    zx = torch.zeros(1, dtype=torch.int64, device="cuda")
    items.append((zx, _dev(W.limbs(3, 5)), torch.full((8,), -1, dtype=torch.int64, device="cuda"), 0, 5))
    host.append((np.zeros(0, dtype=np.uint64), W.limbs(3, 5)))
    outs = {}
    for sched in ("per_pass", "persistent"):
        for it in items:
            it[2].fill_(-1)
        b = D.Batch(items, autotune=False, schedule=sched)
        kind, launches = b.schedule()
        assert kind == sched
        if sched == "persistent":
            assert launches == 1
        for _ in range(2):  # a second run reuses the work list and the counters
            b.run()
            D.sync()
        outs[sched] = [_host(it[2]).copy() for it in items]
        b.close()
    for k in range(len(items)):
        assert np.array_equal(outs["persistent"][k], outs["per_pass"][k]), k
    for k in range(0, len(items), max(1, len(items) // 40)):
        x, y = host[k]
        if len(x) == 0:
            assert not outs["persistent"][k].any()
            continue
        assert np.array_equal(outs["persistent"][k], _single(hg, x, y, len(outs["persistent"][k]))), k


def test_persistent_launch_in_a_graph(hg):
    """The persistent launch captured in a CUDA graph replays bit-identically."""
    import torch

    from hypergeometrica_gb300 import device as D

    items, _ = _make(200, 31, lo_bits=4, hi_bits=14)
    b = D.Batch(items, autotune=False, schedule="persistent")
    b.run()
    D.sync()
    want = [_host(it[2]).copy() for it in items]
    s = torch.cuda.Stream()
    g = torch.cuda.CUDAGraph()
    torch.cuda.synchronize()
    with torch.cuda.graph(g, stream=s):
        b.run(s)
    for _ in range(3):
        for it in items:
            it[2].fill_(-1)
        g.replay()
        torch.cuda.synchronize()
        D.sync()
        for k, it in enumerate(items):
            assert np.array_equal(_host(it[2]), want[k]), k
    b.close()
