"""Parity of the CUDA path with the oracle, through the C ABI (GPU).

Bit-exact comparisons: spectra against ntt-forward / ntt-reverse, products
against the oracle's mpz-*/ntt / mpz-square storage, the mpz-* dispatch
against the oracle's, and, at sizes the oracle cannot finish quickly,
size-independent properties (residues modulo independent primes, squaring
versus multiplication).
"""

import numpy as np
import pytest

from conftest import h2i
from hypergeometrica_gb300 import workloads as W
from hypergeometrica_gb300.mpz import digits_from_int, int_from_digits

pytestmark = pytest.mark.gpu


def _torch():
    import torch

    return torch


def _dev(a):
    torch = _torch()
    return torch.from_numpy(np.ascontiguousarray(a).view(np.int64)).cuda()


def _host(t):
    return t.cpu().numpy().view(np.uint64)


def test_spectra_fixtures(hg, golden):
    from hypergeometrica_gb300 import device as D

    for case in golden["ntt"]:
        v = np.array(h2i(case["input"]), dtype=np.uint64)
        t = _dev(v)
        D.ntt_forward(t, case["mod"])
        D.sync()
        assert [int(x) for x in _host(t)] == h2i(case["forward"]), (case["lgn"], case["mod"])
        D.ntt_reverse(t, case["mod"])
        D.sync()
        assert np.array_equal(_host(t), v)


@pytest.mark.parametrize("lg", [3, 4, 5, 11, 12, 13, 14, 16, 17, 20])
def test_spectra_vs_oracle(hg, oracle, lg):
    from hypergeometrica_gb300 import device as D

    for i, m in enumerate(oracle.moduli()):
        v = W.splitmix64(lg * 7 + i, 1 << lg) % np.uint64(m)
        t = _dev(v)
        D.ntt_forward(t, i)
        D.sync()
        fwd = oracle.ntt_forward(v, i)
        assert np.array_equal(_host(t), fwd), (lg, i)
        # ntt-reverse on the bit-reversed spectrum gives back the input
        D.ntt_reverse(t, i)
        D.sync()
        assert np.array_equal(_host(t), v)
        # and matches the oracle's ntt-reverse on an arbitrary input
        w = W.splitmix64(lg * 13 + i, 1 << lg) % np.uint64(m)
        t = _dev(w)
        D.ntt_reverse(t, i)
        D.sync()
        assert np.array_equal(_host(t), oracle.ntt_reverse(w, i)), (lg, i)


def test_product_fixtures(hg, golden):
    for case in golden["products"]:
        x = hg.MPZ(1, np.array(h2i(case["x"]), dtype=np.uint64))
        if case["kind"] == "mul":
            y = hg.MPZ(1, np.array(h2i(case["y"]), dtype=np.uint64))
            got = hg.mpz_mul_ntt(x, y)
        else:
            got = hg.mpz_square(x)
        assert [int(v) for v in got.storage] == h2i(case["storage"]), case


SIZES = [
    (1, 1), (2, 1), (3, 3), (8, 8), (100, 101), (2048, 2048), (2049, 2047), (4096, 4096), (3000, 7),
    (1 << 15, 1 << 15), (65536, 64), (100000, 31000), (1 << 17, 1 << 17), (1 << 18, 5),
]


@pytest.mark.parametrize("nx,ny", SIZES)
@pytest.mark.parametrize("dist", ["uniform", "ones", "sparse"])
def test_products_vs_oracle(hg, oracle, nx, ny, dist):
    x = W.limbs(1000 + nx, nx, dist)
    y = W.limbs(2000 + ny, ny, dist)
    got = hg.mpz_mul_ntt(hg.MPZ(1, x), hg.MPZ(1, y)).storage
    assert np.array_equal(got, oracle.mpz_mul_ntt(x, y)), (nx, ny, dist)


@pytest.mark.parametrize("n", [1, 2, 5, 1000, 2048, 4097, 1 << 16, 1 << 17])
@pytest.mark.parametrize("dist", ["uniform", "ones"])
def test_squares_vs_oracle(hg, oracle, n, dist):
    x = W.limbs(3000 + n, n, dist)
    got = hg.mpz_square(hg.MPZ(1, x)).storage
    assert np.array_equal(got, oracle.mpz_square(x)), (n, dist)


_PW = {}


def _powers(q: int, n: int) -> np.ndarray:
    """(2^64)^i mod q for i < n (q < 2^31), built from two 4096-entry tables."""
    have = _PW.get(q)
    if have is not None and len(have) >= n:
        return have[:n]
    base = (1 << 64) % q
    blk = 4096
    lo = np.empty(blk, dtype=np.uint64)
    v = 1
    for i in range(blk):
        lo[i] = v
        v = v * base % q
    step, nb = v, (n + blk - 1) // blk
    hi = np.empty(nb, dtype=np.uint64)
    v = 1
    for i in range(nb):
        hi[i] = v
        v = v * step % q
    pw = (np.tile(lo, nb)[:n] * np.repeat(hi, blk)[:n]) % np.uint64(q)
    _PW[q] = pw
    return pw


def _residue(a: np.ndarray, q: int) -> int:
    """a (little-endian 64-bit limbs) mod q for q < 2^31, in O(len(a)) numpy."""
    if len(a) == 0:
        return 0
    r = (a % np.uint64(q)) * _powers(q, len(a)) % np.uint64(q)
    return int(r.sum(dtype=np.uint64) % np.uint64(q))


PRIMES = [2147483647, 2147483629, 2147483587, 2147483579]


@pytest.mark.parametrize("nx,ny,dist", [
    (1 << 20, 1 << 20, "uniform"), (1 << 22, 1 << 22, "uniform"), (1 << 24, 1 << 24, "uniform"),
    (1 << 24, 1 << 16, "uniform"), (1 << 24, 1 << 16, "ones"), (1 << 24, 1 << 16, "sparse"),
    (1 << 25, 1 << 20, "uniform"), (1 << 20, 1 << 6, "ones"), (1 << 20, 1 << 6, "sparse"),
])
def test_large_products_residue_checks(hg, nx, ny, dist):
    """At full size: the product agrees with x*y modulo four independent
    31-bit primes, and its top limbs vanish past nx+ny."""
    x = W.limbs(77, nx, dist)
    y = W.limbs(78, ny, dist)
    got = hg.mpz_mul_ntt(hg.MPZ(1, x), hg.MPZ(1, y)).storage
    assert not got[nx + ny:].any()
    for q in PRIMES:
        assert _residue(got, q) == _residue(x, q) * _residue(y, q) % q, q


def test_full_size_product_equals_gmp(hg):
    """A 2^22 x 2^22-limb product equals GMP's mpz_mul limb for limb (a
    third-party exact product; skipped where libgmp is missing)."""
    import gmp

    if not gmp.available():
        pytest.skip("libgmp not installed")
    n = 1 << 22
    x = W.limbs(61, n, "uniform")
    y = W.limbs(62, n, "uniform")
    got = hg.mpz_mul_ntt(hg.MPZ(1, x), hg.MPZ(1, y)).storage
    assert np.array_equal(got[: 2 * n], gmp.mul(x, y))


def test_large_ones_product_exact(hg):
    """(2^(64n) - 1)^2 = 2^(128n) - 2^(64n+1) + 1: known limbs, longest carries."""
    n = 1 << 23
    x = W.limbs(0, n, "ones")
    got = hg.mpz_square(hg.MPZ(1, x)).storage
    want = np.zeros(len(got), dtype=np.uint64)
    want[0] = 1
    want[n] = np.uint64(2**64 - 2)
    want[n + 1: 2 * n] = np.uint64(2**64 - 1)
    assert np.array_equal(got, want)


def test_square_equals_multiply_large(hg):
    n = 1 << 22
    x = W.limbs(5, n, "uniform")
    a = hg.mpz_square(hg.MPZ(1, x)).storage
    b = hg.mpz_mul_ntt(hg.MPZ(1, x), hg.MPZ(1, x.copy())).storage
    assert np.array_equal(a, b)


def test_mpz_dispatch_vs_oracle(hg, oracle):
    rng = np.random.default_rng(11)
    for trial in range(12):
        na = int(rng.integers(1, 400))
        nb = int(rng.integers(1, 400))
        a = W.limbs(trial, na, "uniform")
        b = W.limbs(trial + 50, nb, "uniform")
        sa, sb = int(rng.choice([1, -1])), int(rng.choice([1, -1]))
        for thr in (1 << 40, 0, 100):
            got = hg.mpz_mul(hg.MPZ(sa, a), hg.MPZ(sb, b), threshold=thr)
            mag, s = oracle.mpz_mul(a, sa, b, sb, False, thr)
            assert got.sign == s and np.array_equal(got.storage, mag)
        x = hg.MPZ(sa, a)
        got = hg.mpz_mul(x, x, threshold=0)
        mag, s = oracle.mpz_mul(a, sa, a, sa, True, 0)
        assert got.sign == s and np.array_equal(got.storage, mag)


@pytest.mark.parametrize("n", [2, 7, 64, 100, 101, 160])
def test_mpz_dispatch_same_object_threshold(hg, oracle, n):
    """(eq x y) below the threshold goes to schoolboy, not to mpz-square: the
    threshold test comes first in mpz-* (src/multiply.lisp:37-44).  The
    schoolboy storage (1 + 2n digits before optimize-mpz) and mpz-square's
    (a power of two) both trim to the same magnitude, so the branch is
    checked through the C ABI's dispatch as well, whose result size is the
    trimmed size either way, and through the storage the host mirror
    returns."""
    import ctypes

    from hypergeometrica_gb300 import _lib

    a = W.limbs(500 + n, n, "uniform")
    for thr in (100, 1 << 40, 0):
        x = hg.MPZ(-1, a.copy())
        got = hg.mpz_mul(x, x, threshold=thr)
        mag, s = oracle.mpz_mul(a, -1, a, -1, True, thr)
        assert got.sign == s == 1 and np.array_equal(got.storage, mag), (n, thr)
        out = np.zeros(2 * n + 1 if n <= thr else int(_lib.load().hg_ntt_length(n, n)), dtype=np.uint64)
        nres, sres = ctypes.c_size_t(0), ctypes.c_int(0)
        _lib.check(_lib.load().hg_mpz_mul(a.ctypes.data, n, -1, a.ctypes.data, n, -1, 1, thr, out.ctypes.data,
                                          len(out), ctypes.byref(nres), ctypes.byref(sres)))
        assert sres.value == 1 and np.array_equal(out[: nres.value], mag), (n, thr)


def test_mpz_dispatch_branch_taken(hg, monkeypatch):
    """Which branch mpz-* takes for (eq x y): schoolboy when size <= the
    threshold, mpz-square above it (src/multiply.lisp:37-44)."""
    from hypergeometrica_gb300 import mpz as M

    taken = []
    real_school, real_square = M.multiply_storage_schoolboy, M.mpz_square
    monkeypatch.setattr(M, "multiply_storage_schoolboy",
                        lambda *a: taken.append("schoolboy") or real_school(*a))
    monkeypatch.setattr(M, "mpz_square", lambda *a: taken.append("square") or real_square(*a))
    for n, thr, want in ((100, 100, "schoolboy"), (101, 100, "square"), (5, 4, "square"), (5, 5, "schoolboy")):
        taken.clear()
        x = hg.MPZ(1, W.limbs(900 + n, n, "uniform"))
        r = M.mpz_mul(x, x, threshold=thr)
        assert taken == [want], (n, thr, taken)
        assert r.to_int() == x.to_int() ** 2


def test_small_paths_vs_oracle(hg, oracle):
    x = W.limbs(1, 5000, "uniform")
    y = W.limbs(2, 100, "uniform")
    assert np.array_equal(hg.multiply_storage_schoolboy(x, 5000, y, 100), oracle.mul_schoolboy(x, y))
    z = W.limbs(3, 20000, "ones")
    for d in (2, 0xFFFFFFFFFFFFFFFF, 987654321987654321):
        got = hg.mpz_multiply_by_digit(d, hg.MPZ(1, z)).storage
        assert np.array_equal(got, oracle.mul_by_digit(z, d))


def test_mpz_mult_simple(hg):
    # test-mpz-mult-simple (tests/mpz.lisp:25-30)
    k = 1 << 128
    n = hg.MPZ.from_int(k)
    assert hg.mpz_mul(n, n).to_int() == k * k
    for thr in (0, 100):
        assert hg.mpz_mul(n, n, threshold=thr).to_int() == k * k


def test_plus_minus_times_randomly(hg):
    # test-mpz-plus-minus-times-randomly (tests/mpz.lisp:32-47), products only
    rng = np.random.default_rng(3)
    for _ in range(10):
        a = int.from_bytes(rng.bytes(42), "little") - (1 << 335)
        b = int.from_bytes(rng.bytes(42), "little") - (1 << 335)
        za, zb = hg.MPZ.from_int(a), hg.MPZ.from_int(b)
        assert hg.mpz_square(za).to_int() == a * a
        assert hg.mpz_mul(za, zb, threshold=1 << 62).to_int() == a * b
        assert hg.mpz_mul(za, zb, threshold=0).to_int() == a * b


def test_device_api_matches_host(hg):
    from hypergeometrica_gb300 import device as D

    torch = _torch()
    x = W.limbs(8, 300000, "uniform")
    y = W.limbs(9, 200001, "uniform")
    host = hg.mpz_mul_ntt(hg.MPZ(1, x), hg.MPZ(1, y)).storage
    tx, ty = _dev(x), _dev(y)
    out = torch.empty(len(host), dtype=torch.int64, device="cuda")
    D.mul(tx, ty, out)
    D.sync()
    assert np.array_equal(_host(out), host)
    sq = torch.empty(1 << 20, dtype=torch.int64, device="cuda")
    D.sqr(tx, sq)
    D.sync()
    assert np.array_equal(_host(sq), hg.mpz_square(hg.MPZ(1, x)).storage)


def test_host_api_pinned_buffers(hg):
    """Pinned host buffers are read and written in place by the kernels;
    the result equals the staged (pageable) path's."""
    import torch

    from hypergeometrica_gb300 import _lib

    lib = _lib.load()
    for nx, ny in ((1 << 20, 3 * (1 << 18) + 5), (5000, 4000), (3, 2)):
        x = W.limbs(21 + nx, nx)
        y = W.limbs(22 + ny, ny)
        ref = hg.mpz_mul_ntt(hg.MPZ(1, x), hg.MPZ(1, y)).storage
        hx = torch.from_numpy(x.view(np.int64)).pin_memory()
        hy = torch.from_numpy(y.view(np.int64)).pin_memory()
        hout = torch.full((len(ref),), -1, dtype=torch.int64).pin_memory()
        _lib.check(lib.hg_mul(hx.data_ptr(), nx, hy.data_ptr(), ny, hout.data_ptr(), len(ref)))
        assert np.array_equal(hout.numpy().view(np.uint64), ref)
        sq = torch.full((int(lib.hg_ntt_length(nx, nx)),), -1, dtype=torch.int64).pin_memory()
        _lib.check(lib.hg_sqr(hx.data_ptr(), nx, sq.data_ptr(), sq.numel()))
        assert np.array_equal(sq.numpy().view(np.uint64), hg.mpz_square(hg.MPZ(1, x)).storage)


def test_error_behaviour(hg):
    import ctypes

    from hypergeometrica_gb300 import _lib

    lib = _lib.load()
    a = np.ones(10, dtype=np.uint64)
    out = np.zeros(15, dtype=np.uint64)
    rc = lib.hg_mul(a.ctypes.data, 10, a.ctypes.data, 10, out.ctypes.data, 15)
    assert rc == _lib.HG_ERR_ARG and "cannot hold" in _lib.last_error()
    bad = (ctypes.c_uint64 * 3)(3, 5, 7)
    assert lib.hg_init(bad, 3, -1) == _lib.HG_ERR_NOT_INIT
    # zero operands give zero without touching the transform
    out[:] = 7
    assert lib.hg_mul(a.ctypes.data, 0, a.ctypes.data, 10, out.ctypes.data, 15) == 0
    assert not out.any()
    x = hg.MPZ.from_int(0)
    assert hg.mpz_mul(x, hg.MPZ.from_int(5)).to_int() == 0
    assert int_from_digits(digits_from_int(0)) == 0


def test_unaligned_device_arrays(hg, oracle):
    """Arrays at an 8-byte offset from a 16-byte boundary (a slice one limb
    into a tensor) cannot be staged by TMA; those passes run with per-thread
    loads and stores and give the same limbs and spectra."""
    from hypergeometrica_gb300 import device as D

    torch = _torch()
    nx, ny = 300001, 200003
    x = W.limbs(31, nx)
    y = W.limbs(32, ny)
    want = hg.mpz_mul_ntt(hg.MPZ(1, x), hg.MPZ(1, y)).storage
    bx = torch.zeros(nx + 1, dtype=torch.int64, device="cuda")
    by = torch.zeros(ny + 1, dtype=torch.int64, device="cuda")
    bx[1:] = _dev(x)
    by[1:] = _dev(y)
    bo = torch.full((len(want) + 1,), -1, dtype=torch.int64, device="cuda")
    tx, ty, out = bx[1:], by[1:], bo[1:]
    assert tx.data_ptr() % 16 == 8 and out.data_ptr() % 16 == 8
    D.mul(tx, ty, out)
    D.sync()
    assert np.array_equal(_host(out), want)
    for lg in (13, 17):
        v = W.splitmix64(lg + 90, 1 << lg) % np.uint64(oracle.moduli()[2])
        buf = torch.zeros((1 << lg) + 1, dtype=torch.int64, device="cuda")
        buf[1:] = _dev(v)
        t = buf[1:]
        D.ntt_forward(t, 2)
        D.sync()
        assert np.array_equal(_host(t), oracle.ntt_forward(v, 2)), lg
        D.ntt_reverse(t, 2)
        D.sync()
        assert np.array_equal(_host(t), v), lg
