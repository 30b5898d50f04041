"""Property tests of the C oracle against exact integer arithmetic (CPU only),
modelled on the reference's suite (tests/mpz.lisp, tests/ntt.lisp,
tests/arithmetic.lisp, tests/multiplication.lisp)."""


import numpy as np
import pytest

from hypergeometrica_gb300 import workloads as W
from hypergeometrica_gb300.mpz import digits_from_int, int_from_digits


def _int(a):
    return int_from_digits(a)


@pytest.mark.parametrize("nx,ny,dist", [
    (101, 101, "uniform"), (1000, 333, "uniform"), (4096, 4096, "uniform"), (3000, 1, "uniform"),
    (500, 500, "ones"), (2048, 17, "ones"), (2000, 1500, "sparse"),
])
def test_ntt_product_exact(oracle, nx, ny, dist):
    x = W.limbs(11 + nx, nx, dist)
    y = W.limbs(29 + ny, ny, dist)
    got = oracle.mpz_mul_ntt(x, y)
    assert len(got) == oracle.hg_len(nx, ny)
    assert _int(got) == _int(x) * _int(y)


@pytest.mark.parametrize("n,dist", [(1, "uniform"), (77, "uniform"), (2048, "uniform"), (1000, "ones")])
def test_square_exact(oracle, n, dist):
    x = W.limbs(5 + n, n, dist)
    assert _int(oracle.mpz_square(x)) == _int(x) ** 2


def test_small_paths_exact(oracle):
    x = W.limbs(1, 300, "uniform")
    y = W.limbs(2, 100, "uniform")
    assert _int(oracle.mul_schoolboy(x, y)) == _int(x) * _int(y)
    for d in (2, 3, 0xFFFFFFFFFFFFFFFF, 12345678901234567):
        assert _int(oracle.mul_by_digit(x, d)) == _int(x) * d


def test_mpz_dispatch_randomly(oracle):
    # test-mpz-plus-minus-times-randomly (tests/mpz.lisp:32-47): signed
    # ~333-bit operands through schoolboy (threshold infinite), NTT
    # (threshold 0) and squaring.
    rng = np.random.default_rng(7)
    for _ in range(10):
        a = int(rng.integers(0, 2**62)) ** 5 * (-1) ** int(rng.integers(0, 2))
        b = int(rng.integers(0, 2**62)) ** 5 * (-1) ** int(rng.integers(0, 2))
        da, db = digits_from_int(a), digits_from_int(b)
        sa, sb = (1 if a >= 0 else -1), (1 if b >= 0 else -1)
        for thr in (2**62, 0, 100):
            mag, s = oracle.mpz_mul(da, sa, db, sb, False, thr)
            assert s * _int(mag) == a * b
        mag, s = oracle.mpz_mul(da, sa, da, sa, True, 0)
        assert s * _int(mag) == a * a


def test_mpz_mult_simple(oracle):
    # test-mpz-mult-simple (tests/mpz.lisp:25-30): (2^128)^2
    d = digits_from_int(1 << 128)
    mag, s = oracle.mpz_mul(d, 1, d, 1, True, 100)
    assert s == 1 and _int(mag) == 1 << 256


def test_inversion_property(oracle):
    # test-inversion-properties (tests/ntt.lisp:121-131) at N = 2^6 and larger
    for lg in (6, 12):
        for i, m in enumerate(oracle.moduli()):
            v = W.splitmix64(lg * 10 + i, 1 << lg) % np.uint64(m)
            assert np.array_equal(oracle.ntt_reverse(oracle.ntt_forward(v, i), i), v)


def test_ntt_matches_direct_dft(oracle):
    # test-ntt-from-various-definitions (tests/ntt.lisp:133-155) at N = 2^8
    n = 256
    L = oracle.lib()
    s = oracle.scheme()
    for i, m in enumerate(oracle.moduli()):
        v = [int(x) for x in W.splitmix64(900 + i, n) % np.uint64(m)]
        w = L.hgo_scheme_root(s, 8, i, 0, 0)
        direct = [sum(pow(w, j * k, m) * v[j] for j in range(n)) % m for k in range(n)]
        fwd = oracle.bit_reverse_permute(oracle.ntt_forward(np.array(v, dtype=np.uint64), i))
        assert [int(x) for x in fwd] == direct


def test_m_mul_fast_random(oracle):
    # test-m*/fast (tests/multiplication.lisp:9-18), 20k pairs per modulus
    L = oracle.lib()
    minv = [0xA655C4392D7B73A5, 0xBC52640BC52640BA, 0xFA232CF252138ABB]
    for i, m in enumerate(oracle.moduli()):
        a = W.splitmix64(31 + i, 20000) % np.uint64(m)
        b = W.splitmix64(71 + i, 20000) % np.uint64(m)
        for x, y in zip(a.tolist(), b.tolist()):
            assert L.hgo_m_mul_fast(x, y, m, minv[i]) == x * y % m


def test_parallel_tasks_same_result(oracle):
    x = W.limbs(3, 5000, "uniform")
    y = W.limbs(4, 4000, "uniform")
    oracle.set_threads(1)
    a = oracle.mpz_mul_ntt(x, y)
    oracle.set_threads(6)
    try:
        b = oracle.mpz_mul_ntt(x, y)
    finally:
        oracle.set_threads(1)
    assert np.array_equal(a, b)


def test_oracle_against_gmp(oracle):
    """Cross-check with GMP's mpz_mul (a third-party exact product), when the
    GMP runtime is installed (oracle/gmp.py)."""
    import gmp

    if not gmp.available():
        pytest.skip("libgmp not installed")
    nx = ny = 1 << 15
    x = W.limbs(100, nx, "uniform")
    y = W.limbs(101, ny, "uniform")
    got = oracle.mpz_mul_ntt(x, y)
    assert np.array_equal(got[: nx + ny], gmp.mul(x, y))


def test_gmp_powers_against_python():
    """The GMP power binding (oracle/gmp.py) that the 9^(9^9) GPU check
    compares with: exact against Python's integers on small powers."""
    import gmp

    from hypergeometrica_gb300.mpz import int_from_digits

    if not gmp.available():
        pytest.skip("libgmp not installed")
    for base, exp in ((9, 9**5), (3, 1000), (2**32 - 5, 77), (7, 1), (2, 64), (5, 0)):
        assert int_from_digits(gmp.ui_pow_ui(base, exp)) == base**exp
