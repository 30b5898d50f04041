"""Every benchmark configuration compared limb for limb with an exact product (GPU).

  single product  2^16 x 2^16 limbs against the oracle's mpz-*/ntt storage
                  (src/ntt-multiply.lisp:174-254), seeds 1 and 2;
  balanced sweep  a*b and a^2 with |a| = |b| in {2^18, 2^20, 2^22, 2^24, 2^26}
                  against GMP's mpz_mul (a^2 passes one operand twice), seeds
                  11 and 12, the bench's own operands;
  unbalanced      2^24 x 2^16, 2^25 x 2^20 and 2^20 x 2^6 limbs in uniform,
                  all-ones and 1%-sparse limbs against GMP, seeds 13 and 14,
                  both as the library runs them (in chunks) and as the
                  reference's one transform of the least power of two
                  >= nx + ny points (chunking off).

GMP's products are exact and unique, so equality with them is equality with
the reference's ntt-multiply on the same operands.  They are computed on host
threads (ctypes releases the interpreter lock inside mpz_mul), all submitted
when the first case of this file asks for one, so that they run while the
GPU works on the earlier cases.
"""

import concurrent.futures as cf
import os

import numpy as np
import pytest

from hypergeometrica_gb300 import workloads as W

pytestmark = pytest.mark.gpu

BALANCED = (18, 20, 22, 24, 26)
UNBALANCED = ((24, 16), (25, 20), (20, 6))
DISTS = ("uniform", "ones", "sparse")


def _jobs():
    jobs = {}
    for k in BALANCED:
        n = 1 << k
        jobs[("mul", k)] = ("mul", (11, n, "uniform"), (12, n, "uniform"))
        jobs[("sqr", k)] = ("sqr", (11, n, "uniform"), None)
    for ka, kb in UNBALANCED:
        for dist in DISTS:
            jobs[("unb", ka, kb, dist)] = ("mul", (13, 1 << ka, dist), (14, 1 << kb, dist))
    return jobs


def _gmp_product(kind, xs, ys):
    import gmp

    x = W.limbs(*xs)
    if kind == "sqr":
        return gmp.sqr(x)
    return gmp.mul(x, W.limbs(*ys))


@pytest.fixture(scope="module")
def exact():
    """Futures of GMP's products of every case, largest first."""
    import gmp

    if not gmp.available():
        pytest.skip("libgmp not installed")
    jobs = _jobs()
    order = sorted(jobs, key=lambda key: -(jobs[key][1][1] * (jobs[key][2][1] if jobs[key][2] else jobs[key][1][1])))
    ex = cf.ThreadPoolExecutor(max_workers=max(2, min(len(jobs), (os.cpu_count() or 2) - 1)))
    futs = {key: ex.submit(_gmp_product, *jobs[key]) for key in order}
    yield futs
    ex.shutdown(wait=True, cancel_futures=True)


def test_single_product_2e16_vs_oracle(hg, oracle):
    """The single-product configuration: 2^16 x 2^16 limbs (transform 2^17)
    against the oracle's mpz-*/ntt storage, every limb."""
    n = 1 << 16
    x, y = W.limbs(1, n), W.limbs(2, n)
    got = hg.mpz_mul_ntt(hg.MPZ(1, x), hg.MPZ(1, y)).storage
    assert len(got) == 1 << 17
    assert np.array_equal(got, oracle.mpz_mul_ntt(x, y))


@pytest.mark.parametrize("k", BALANCED)
@pytest.mark.parametrize("kind", ["mul", "sqr"])
def test_balanced_sweep_vs_gmp(hg, exact, kind, k):
    n = 1 << k
    x = W.limbs(11, n)
    if kind == "mul":
        got = hg.mpz_mul_ntt(hg.MPZ(1, x), hg.MPZ(1, W.limbs(12, n))).storage
    else:
        got = hg.mpz_square(hg.MPZ(1, x)).storage
    assert len(got) == 2 * n
    want = exact[(kind, k)].result()
    assert np.array_equal(got, want), (kind, k, int(np.flatnonzero(got != want)[0]))


@pytest.mark.parametrize("ka,kb", UNBALANCED)
@pytest.mark.parametrize("dist", DISTS)
def test_unbalanced_vs_gmp(hg, exact, ka, kb, dist):
    from hypergeometrica_gb300 import _lib

    na, nb = 1 << ka, 1 << kb
    x, y = W.limbs(13, na, dist), W.limbs(14, nb, dist)
    chunked = hg.mpz_mul_ntt(hg.MPZ(1, x), hg.MPZ(1, y)).storage
    _lib.set_chunking(False)
    try:
        one = hg.mpz_mul_ntt(hg.MPZ(1, x), hg.MPZ(1, y)).storage
    finally:
        _lib.set_chunking(True)
    want = exact[("unb", ka, kb, dist)].result()
    assert not chunked[na + nb:].any() and not one[na + nb:].any()
    assert np.array_equal(chunked[: na + nb], want), (ka, kb, dist, "chunked")
    assert np.array_equal(one[: na + nb], want), (ka, kb, dist, "one transform")
