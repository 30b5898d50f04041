"""Unbalanced products run in chunks (GPU): the long operand is cut into
chunks multiplied by one shared spectrum of the short operand, and the chunk
products are added during the reconstruction.  The result must be the same
integer as mpz-*/ntt's single transform (src/ntt-multiply.lisp:174-254):
bit-exact against the oracle, against the batch path (which always runs one
transform per product) and, at full size, modulo independent primes.
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


def _plan(nx, ny):
    from hypergeometrica_gb300 import _lib

    return _lib.chunk_plan(nx, ny)


def _last_chunk_of_one(ny, start):
    """An nx whose chunk plan leaves exactly one limb in the last chunk."""
    nx = start
    for _ in range(20):
        L, c, k = _plan(nx, ny)
        want = (k - 1) * c + 1
        if want == nx:
            return nx
        nx = want if want > c else nx + c
    pytest.fail("no plan with a one-limb last chunk found")


CASES = [
    (5000, 9), (9, 5000), (3000, 7), (65536, 64), (64, 65536),
    (200003, 1000), (1000, 200003), ((1 << 18) + 3, 3001), ((1 << 18) + 3, 1 << 10), (1 << 18, 37),
]


@pytest.mark.parametrize("nx,ny", CASES)
@pytest.mark.parametrize("dist", ["uniform", "ones", "sparse"])
def test_chunked_products_vs_oracle(hg, oracle, nx, ny, dist):
    assert _plan(nx, ny) is not None, (nx, ny)
    x = W.limbs(4000 + nx, nx, dist)
    y = W.limbs(5000 + ny, ny, dist)
    got = hg.mpz_mul_ntt(hg.MPZ(1, x), hg.MPZ(1, y)).storage
    assert np.array_equal(got, oracle.mpz_mul_ntt(x, y)), (nx, ny, dist, _plan(nx, ny))


@pytest.mark.parametrize("ny", [1000, 3001])
def test_one_limb_last_chunk(hg, oracle, ny):
    nx = _last_chunk_of_one(ny, 150000)
    for dist in ("uniform", "ones"):
        x = W.limbs(nx, nx, dist)
        y = W.limbs(ny, ny, dist)
        got = hg.mpz_mul_ntt(hg.MPZ(1, x), hg.MPZ(1, y)).storage
        assert np.array_equal(got, oracle.mpz_mul_ntt(x, y)), (nx, ny, dist, _plan(nx, ny))


def test_chunked_equals_single_transform(hg):
    """The chunked device product equals the batch path's single transform."""
    import torch

    from hypergeometrica_gb300 import _lib
    from hypergeometrica_gb300 import device as D

    for nx, ny in ((1 << 22, 1 << 12), (1 << 21, 77777), (5 << 18, 1 << 17)):
        assert _plan(nx, ny) is not None
        tx, ty = _dev(W.limbs(nx, nx)), _dev(W.limbs(ny + 1, ny))
        a = torch.full((nx + ny + 64,), -1, dtype=torch.int64, device="cuda")
        b = torch.full((nx + ny + 64,), -1, dtype=torch.int64, device="cuda")
        D.mul(tx, ty, a)        # chunked, with a zeroed tail past nx + ny
        D.mul_batch([(tx, ty, b)])  # one transform
        D.sync()
        assert torch.equal(a, b), (nx, ny)
        assert not a[nx + ny:].any()
        c = torch.full((nx + ny,), -1, dtype=torch.int64, device="cuda")
        D.mul(ty, tx, c)        # operands swapped
        D.sync()
        assert torch.equal(c, a[: nx + ny]), (nx, ny)
        d = torch.full((nx + ny,), -1, dtype=torch.int64, device="cuda")
        _lib.set_chunking(False)
        try:
            D.mul(tx, ty, d)    # the reference's one transform through hg_mul_device
            D.sync()
        finally:
            _lib.set_chunking(True)
        assert torch.equal(d, a[: nx + ny]), (nx, ny)


def test_chunked_host_paths(hg, oracle):
    """hg_mul on pageable and pinned host buffers, both operand orders, with
    nout past the product (zeroed)."""
    import torch

    from hypergeometrica_gb300 import _lib

    lib = _lib.load()
    nx, ny = (1 << 20) + 12345, 3001
    assert _plan(nx, ny) is not None
    x = W.limbs(31, nx)
    y = W.limbs(32, ny)
    ref = oracle.mpz_mul_ntt(x, y)[: nx + ny]
    nout = nx + ny + 100
    for a, b in ((x, y), (y, x)):
        out = np.full(nout, 7, dtype=np.uint64)
        _lib.check(lib.hg_mul(a.ctypes.data, len(a), b.ctypes.data, len(b), out.ctypes.data, nout))
        assert np.array_equal(out[: len(ref)], ref) and not out[len(ref):].any()
        ha = torch.from_numpy(a.view(np.int64)).pin_memory()
        hb = torch.from_numpy(b.view(np.int64)).pin_memory()
        hout = torch.full((nout,), -1, dtype=torch.int64).pin_memory()
        _lib.check(lib.hg_mul(ha.data_ptr(), len(a), hb.data_ptr(), len(b), hout.data_ptr(), nout))
        got = hout.numpy().view(np.uint64)
        assert np.array_equal(got[: len(ref)], ref) and not got[len(ref):].any()


def test_chunked_mpz_dispatch(hg, oracle):
    """mpz-* routes an unbalanced pair above the schoolboy threshold to the
    chunked product; signs follow the reference's dispatch."""
    x = W.limbs(41, 70000, "uniform")
    y = W.limbs(42, 300, "uniform")
    for sa, sb in ((1, -1), (-1, -1)):
        got = hg.mpz_mul(hg.MPZ(sa, y), hg.MPZ(sb, x), threshold=100)
        mag, s = oracle.mpz_mul(y, sa, x, sb, False, 100)
        assert got.sign == s and np.array_equal(got.storage, mag)

