"""The MPD / mpd-pi oracle (CPU only).

Pinned by an independent pi (Machin's formula): mpd-pi's result must lie
within 2^-b of pi/10, the reference's acceptance test (tests/pi.lisp:7-48).
The single-float steps are checked against numpy's IEEE float32.
"""

import math

import numpy as np
import pytest

import mpd_oracle as M
import series_oracle as S


@pytest.mark.parametrize("bits", [10, 64, 100, 500, 1000, 3000])
def test_mpd_pi_within_2_to_minus_b(bits):
    x = M.mpd_pi(bits)
    # |x - pi/10| <= 2^-bits, compared through enough decimal digits
    d = bits * 30103 // 100000 + 10
    err = abs(M.digits_of(x, d) - S.pi_machin(d - 1))
    assert err <= 1 + (10 ** d >> bits)


def test_single_float_steps_match_ieee_float32():
    rng = np.random.default_rng(3)
    for n in list(range(1, 3000)) + [int(v) for v in rng.integers(1, 2**63, 2000)] + [2**64 - 1, 2**40 + 1]:
        assert M.int_to_single(n) == float(np.float32(n)) or n > 2**53  # float32(n) is exact rounding below 2^53
        s = M.single_sqrt_of_int(n)
        if n < 2**24:
            assert s == float(np.sqrt(np.float32(n)))
        q = M.cl_round_int_by_single(2**64, s)
        assert q == int(np.float32(2.0**64) / np.float32(s))


def test_int_to_single_ties_to_even():
    # 2^24 + 1 lies halfway between 2^24 and 2^24 + 2: ties to even
    assert M.int_to_single(2**24 + 1) == 2.0**24
    assert M.int_to_single(2**24 + 3) == 2.0**24 + 4
    assert M.int_to_single(3 * 2**100 + 2**76) == float(3 * 2**100)  # exactly half an ulp, even stays
    assert M.int_to_single(2**127 * 3 // 2) == 1.5 * 2.0**127


def test_cl_round_ties_to_even():
    assert M.cl_round_ratio(5, 2) == 2 and M.cl_round_ratio(7, 2) == 4 and M.cl_round_ratio(2**64, 3) == 6148914691236517205


def test_reciprocal_and_inv_sqrt_converge():
    for v in (3, 7, 10005, 2**70 + 12345):
        x = M.mpd_reciprocal(M.integer_mpd(v), 500)
        assert abs(M.digits_of(x, 140) - 10**140 // v) <= 1
        y = M.mpd_inv_sqrt(M.integer_mpd(v), 500)
        z = M.digits_of(y, 140)
        assert abs(z * z * v - 10**280) <= 2 * z * v + 10**141
