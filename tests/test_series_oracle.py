"""The binary-splitting oracle and the host-side tree logic (CPU only).

The oracle's Chudnovsky series is pinned by an independent pi (Machin's
formula); its closed-form residues by the recursion itself; the driver's
level-by-level tree by the reference's recursive split.
"""

import numpy as np
import pytest

import series_oracle as O


@pytest.mark.parametrize("prec", [1, 2, 10, 57, 400, 3000])
def test_chudnovsky_reproduces_machin_pi(prec):
    # compute-pi/chudnovsky returns floor(10^prec * pi / 10)
    assert O.compute_pi_chudnovsky(prec) == O.pi_machin(prec - 1)


SERIES = {
    "chudnovsky": O.chudnovsky_series(),
    "e": O.e_series(),
    "exp(-2/7)": O.exp_series("-2/7"),
    "ramanujan": O.ramanujan_series(),
    "catalan": O.catalan_series(),
    "apery": O.apery_series(),
}


@pytest.mark.parametrize("name", sorted(SERIES))
@pytest.mark.parametrize("lo,hi", [(0, 1), (0, 2), (0, 9), (4, 77)])
def test_residues_match_recursion(name, lo, hi):
    s = SERIES[name]
    P, Q, B, R = O.binary_split(s, lo, hi)
    for m in ((1 << 61) - 1, 2305843009213693921, 998244353):
        assert O.residues(s, lo, hi, m) == (P % m, Q % m, B % m, R % m)


def _ref_nodes(lo, hi, acc):
    acc.append((lo, hi))
    if hi - lo > 1:
        m = (lo + hi) // 2
        _ref_nodes(lo, m, acc)
        _ref_nodes(m, hi, acc)


@pytest.mark.parametrize("lo,hi", [(0, 1), (0, 2), (0, 3), (0, 7), (5, 40), (0, 1000), (3, 12345)])
def test_tree_is_the_reference_recursion(lo, hi):
    from hypergeometrica_gb300 import series as S

    L, H, left, right, height = S._tree(lo, hi)
    acc = []
    _ref_nodes(lo, hi, acc)
    assert sorted(zip(L.tolist(), H.tolist())) == sorted(acc)
    for i in range(L.size):
        span = int(H[i] - L[i])
        assert height[i] == (span - 1).bit_length()
        if left[i] >= 0:
            m = (L[i] + H[i]) // 2
            assert (L[left[i]], H[left[i]], L[right[i]], H[right[i]]) == (L[i], m, m, H[i])
            assert height[i] == max(height[left[i]], height[right[i]]) + 1


def test_pack_round_trip():
    from hypergeometrica_gb300 import series as S
    from hypergeometrica_gb300.mpz import int_from_digits

    vals = [0, 1, -5, 2**64 - 1, -(2**64), 3**200, -(7**90)]
    sg, limbs, sz, w = S._pack(vals)
    for v, s_, row, n in zip(vals, sg, limbs, sz):
        mag = int_from_digits(row[:n])
        assert (mag if s_ > 0 else -mag) == v
        assert n == (abs(v).bit_length() + 63) // 64


def test_series_definitions_agree_with_oracle():
    """The package's series (the GPU driver's input) equal the oracle's."""
    from hypergeometrica_gb300 import series as S

    pkg = {
        "chudnovsky": S.make_chudnovsky_series(),
        "e": S.make_e_series(),
        "exp(-2/7)": S.make_exp_series("-2/7"),
        "ramanujan": S.make_ramanujan_series(),
        "catalan": S.make_catalan_series(),
        "apery": S.make_apery_series(),
    }
    for name, s in pkg.items():
        a, b, p, q = SERIES[name]
        for n in range(0, 40):
            assert (s.a(n), s.b(n), s.p(n), s.q(n)) == (a(n), b(n), p(n), q(n)), (name, n)


def test_chudnovsky_terms():
    from hypergeometrica_gb300 import series as S

    # num-terms of mpd-pi (src/pi.lisp:53-56)
    import math

    for b in (10, 100, 1000, 1 << 16, 1 << 22, 1 << 26):
        assert S.chudnovsky_terms(b) == 2 + math.floor((b + 64) / math.log2(151931373056000))
    assert np.isclose(S.CHUD_BITS_PER_TERM, 47.1104, atol=1e-3)
