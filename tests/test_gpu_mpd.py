"""MPD arithmetic and mpd-pi on the GPU (mpd.py) against the oracle.

mpd_pi follows the reference exactly (no truncation), so its result must be
bit-identical to the oracle's: the same mantissa integer and exponent.  At
2^16 bits, where the oracle on Python integers would take minutes, the GPU
result is checked against an independent pi to 2^-b.  The truncated variant
is not the reference's mantissa; it must agree with pi/10 to the bits asked.
"""

import hashlib
import json
import os

import numpy as np
import pytest

import mpd_oracle as M
import series_oracle as O
from conftest import ROOT

pytestmark = pytest.mark.gpu


def _mpd_pi_fixtures():
    with open(os.path.join(ROOT, "tests", "golden", "mpd_pi.json")) as f:
        return json.load(f)["fixtures"]


def _pair(x):
    return x.to_pair()


@pytest.mark.parametrize("bits", [10, 100, 1000, 3000, 10000])
def test_mpd_pi_bit_identical(hg, bits):
    from hypergeometrica_gb300 import mpd as G

    got = G.mpd_pi(bits)
    want = M.mpd_pi(bits)
    assert _pair(got) == (want.m, want.e)


@pytest.mark.parametrize("fx", _mpd_pi_fixtures(), ids=lambda f: f"{f['bits']}bits")
def test_mpd_pi_bit_identical_golden(hg, fx):
    """Untruncated mpd-pi at up to 2^18 bits against the oracle's result
    (tests/golden/make_mpd_pi_golden.py): exponent, sign, length, end limbs
    and SHA-256 of the mantissa's little-endian limbs."""
    from hypergeometrica_gb300 import mpd as G

    got = G.mpd_pi(fx["bits"])
    mant = got.mantissa
    limbs = np.trim_zeros(mant.t[: mant.size].cpu().numpy().view(np.uint64), "b")
    assert got.exponent == fx["exponent"]
    assert mant.sign == fx["sign"] and limbs.size == fx["limbs"]
    assert hex(int(limbs[0])) == fx["low_limb"] and hex(int(limbs[-1])) == fx["high_limb"]
    assert hashlib.sha256(limbs.tobytes()).hexdigest() == fx["sha256"]


def test_reciprocal_and_inv_sqrt_bit_identical(hg):
    from hypergeometrica_gb300 import mpd as G
    from hypergeometrica_gb300.series import DeviceInt

    rng = np.random.default_rng(9)
    for k in range(8):
        m = int.from_bytes(rng.bytes(8 * int(rng.integers(1, 6))), "little") | 1
        sign = -1 if k % 3 == 1 else 1
        e = int(rng.integers(-30, 30))
        bits = int(rng.choice([64, 300, 1000]))
        a_g = G.MPD(DeviceInt.from_int(sign * m), e)
        a_o = M.MPD(sign * m, e)
        r = G.mpd_reciprocal(a_g, bits)
        ro = M.mpd_reciprocal(a_o, bits)
        assert _pair(r) == (ro.m, ro.e), k
        if sign > 0:
            s = G.mpd_sqrt(a_g, bits)
            so = M.mpd_sqrt(a_o, bits)
            assert _pair(s) == (so.m, so.e), k


def test_mpd_pi_2e16_bits_accuracy(hg):
    from hypergeometrica_gb300 import mpd as G

    bits = 1 << 16
    x = G.mpd_pi(bits)
    d = bits * 30103 // 100000
    assert abs(x.digits(d) - O.pi_machin(d - 1)) <= 1 + (10 ** d >> bits)


@pytest.mark.parametrize("bits", [1000, 10000, 1 << 16])
def test_truncated_variant_accuracy(hg, bits):
    from hypergeometrica_gb300 import mpd as G

    x = G.mpd_pi_truncated(bits)
    d = bits * 30103 // 100000
    assert abs(x.digits(d) - O.pi_machin(d - 1)) <= 1 + (10 ** d >> bits)
    assert x.mantissa.size <= -(-(bits + 64) // 64) + 2


def test_truncated_variant_2e20_bits_consistent(hg):
    """At 2^20 bits (too large for an independent pi here): the truncated
    result agrees with a run at 2^20 + 4096 bits to 2^20 bits, and with the
    reference-exact 2^16-bit result to 2^16 bits."""
    from hypergeometrica_gb300 import mpd as G

    bits = 1 << 20
    a = G.mpd_pi_truncated(bits)
    b = G.mpd_pi_truncated(bits + 4096)
    ma, ea = a.to_pair()
    mb, eb = b.to_pair()
    # both as floor(2^bits * value)
    fa = ma >> (-64 * ea - bits) if -64 * ea > bits else ma << (bits + 64 * ea)
    fb = mb >> (-64 * eb - bits) if -64 * eb > bits else mb << (bits + 64 * eb)
    assert abs(fa - fb) <= 2
    x = G.mpd_pi(1 << 16)
    mx, ex = x.to_pair()
    fx = mx >> (-64 * ex - (1 << 16))
    assert abs((fa >> (bits - (1 << 16))) - fx) <= 2
