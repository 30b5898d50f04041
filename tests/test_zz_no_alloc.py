"""hg_mul_device_noalloc on the GPU: the product on the library's fixed
scratch array equals hg_mul_device's (hg_sqr_device's for squares).

The results are integers, so the tolerance is exact equality, limb for limb.
Every case runs the allocation-free call twice in a row (the second call
reuses the scratch the first one left behind).  The file name sorts last so
that the suite runs it after every other GPU test; it also passes alone.
"""

import numpy as np
import pytest

from hypergeometrica_gb300 import workloads as W

pytestmark = pytest.mark.gpu

# (nx, ny or None for a square, extra output limbs past the product)
CASES = [
    (3, 5, 0),  # transform 2^3: the tiny in-register kernel
    (100, 28, 0),  # 2^7, one contiguous pass
    (2048, 2048, 9),  # 2^12, the largest single-pass length, zero tail
    (3000, 2500, 0),  # 2^13, strided + contiguous
    (9000, 7000, 0),  # 2^14
    (20000, None, 3),  # square, 2^16
    (40000, 25536, 0),  # 2^16, the largest accepted product
]


def _dev(a):
    import torch

    return torch.from_numpy(np.ascontiguousarray(a).view(np.int64)).cuda()


def _host(t):
    return t.cpu().numpy().view(np.uint64)


def _full(n):
    import torch

    return torch.full((n,), -1, dtype=torch.int64, device="cuda")


@pytest.mark.parametrize("nx,ny,extra", CASES)
def test_noalloc_matches_mul_device(hg, nx, ny, extra):
    from hypergeometrica_gb300 import device as D

    x = _dev(W.limbs(7 * nx + 1, nx))
    y = None if ny is None else _dev(W.limbs(7 * nx + 2, ny))
    nout = (2 * nx if ny is None else nx + ny) + extra
    want = _full(nout)
    if y is None:
        D.sqr(x, want)
    else:
        D.mul(x, y, want)
    D.sync()
    ref = _host(want)
    for call in range(2):
        got = _full(nout)
        D.mul_noalloc(x, y, got)
        D.sync()
        assert np.array_equal(_host(got), ref), f"call {call}"


def test_noalloc_matches_oracle_small(hg, oracle):
    from hypergeometrica_gb300 import device as D

    a, b = W.limbs(11, 700), W.limbs(12, 300)
    ref = oracle.mpz_mul_ntt(a, b)[:1000]
    for call in range(2):
        got = _full(1000)
        D.mul_noalloc(_dev(a), _dev(b), got)
        D.sync()
        assert np.array_equal(_host(got), ref), f"call {call}"


def test_noalloc_zero_operand(hg):
    from hypergeometrica_gb300 import device as D

    x = _dev(W.limbs(3, 50))
    got = _full(50)
    D.mul_noalloc(x, x, got, ny=0)  # a non-null y of length 0 (null y means a square)
    D.sync()
    assert not _host(got).any()


def test_noalloc_rejects_oversize_and_short_output(hg):
    from hypergeometrica_gb300 import device as D
    from hypergeometrica_gb300._lib import HG_ERR_ARG, HGError

    x = _dev(W.limbs(5, 40000))
    y = _dev(W.limbs(6, D.NOALLOC_MAX_LIMBS - 40000 + 1))
    out = _full(D.NOALLOC_MAX_LIMBS + 1)
    with pytest.raises(HGError) as e:
        D.mul_noalloc(x, y, out)
    assert e.value.code == HG_ERR_ARG and "65536" in str(e.value)
    D.sync()
    assert (_host(out) == np.uint64(2**64 - 1)).all()  # nothing was enqueued
    with pytest.raises(HGError) as e:
        D.mul_noalloc(x, x, _full(100))
    assert e.value.code == HG_ERR_ARG


def test_noalloc_leaves_device_memory_alone(hg):
    """After the first call's setup, further calls change no device memory
    accounting: no workspace growth, no allocation."""
    import torch

    from hypergeometrica_gb300 import device as D

    x = _dev(W.limbs(21, 33000))
    y = _dev(W.limbs(22, 32536))
    outs = [_full(65536) for _ in range(3)]
    D.mul_noalloc(x, y, outs[0])
    D.sync()
    free0, _ = torch.cuda.mem_get_info()
    D.mul_noalloc(x, y, outs[1])
    D.mul_noalloc(x, y, outs[2])
    D.sync()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0
    assert np.array_equal(_host(outs[1]), _host(outs[0]))
    assert np.array_equal(_host(outs[2]), _host(outs[0]))
