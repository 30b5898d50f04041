"""Oracle for the reference's dyadic floats and mpd-pi (TEST INFRASTRUCTURE).

A CPU restatement, on Python integers, of src/mpd.lisp, src/mpd-reciprocal.lisp,
src/mpd-sqrt.lisp and mpd-pi (src/pi.lisp:53-74).  Only tests/,
__graft_entry__.smoke() and bench.py's CPU leg may use it, as the checker.

An MPD is mantissa * 2^(64 * exponent) (mpd.lisp:7-12); every operation of
the reference depends only on the mantissa's value (mpz-size is the length
without high zero limbs, src/vec.lisp:218-229), so (mantissa, exponent) pairs
of Python integers reproduce it exactly.  The two float steps are restated
bit for bit:

  estimate-reciprocal (mpd-reciprocal.lisp:7-25): (round $base msb) on two
      integers, CL round = nearest, ties to even, on the exact rational;
  estimate-inv-sqrt (mpd-sqrt.lisp:7-38): (sqrt msb) of an integer is an IEEE
      single-float (the integer rounded to single, then a correctly rounded
      single sqrt); (round $base <single>) converts $base to single, divides
      in single precision and rounds the single result to an integer.

Pinned by series_oracle.pi_machin: mpd_pi(b) must lie within 2^-b of pi/10,
the reference's own acceptance test (tests/pi.lisp:7-48).
"""

from __future__ import annotations

import math
import struct

import series_oracle

BASE = 1 << 64


def mpz_size(m: int) -> int:
    return (abs(m).bit_length() + 63) // 64


class MPD:
    __slots__ = ("m", "e")

    def __init__(self, m: int, e: int):
        self.m, self.e = int(m), int(e)

    def __eq__(self, o):
        return isinstance(o, MPD) and (self.m, self.e) == (o.m, o.e)

    def __repr__(self):
        return f"MPD({mpz_size(self.m)} limbs, e={self.e})"


def integer_mpd(n):
    return MPD(n, 0)


def mpd_oom(x: MPD):
    """(values oom zero?) (mpd.lisp:23-39)."""
    if x.m == 0:
        return 0, True
    return min(0, mpz_size(x.m) + x.e), False


def mpd_mul(a: MPD, b: MPD) -> MPD:
    return MPD(a.m * b.m, a.e + b.e)


def mpd_add(a: MPD, b: MPD) -> MPD:
    lo = min(a.e, b.e)
    return MPD((a.m << (64 * (a.e - lo))) + (b.m << (64 * (b.e - lo))), lo)


def mpd_negate(a: MPD) -> MPD:
    return MPD(-a.m, a.e)


def mpd_sub(a: MPD, b: MPD) -> MPD:
    return mpd_add(a, mpd_negate(b))


def mpd_half(a: MPD) -> MPD:
    """mpd-half! (mpd.lisp:77-81): times $base/2, exponent - 1."""
    return MPD(a.m * (BASE // 2), a.e - 1)


def cl_round_ratio(n: int, d: int) -> int:
    """CL (round n d) on integers: nearest, ties to even."""
    q, r = divmod(n, d)
    if 2 * r > d or (2 * r == d and q % 2 == 1):
        q += 1
    return q


def _f32(x: float) -> float:
    return struct.unpack("<f", struct.pack("<f", x))[0]


def int_to_single(n: int) -> float:
    """An integer rounded to the nearest IEEE single (ties to even)."""
    if n == 0:
        return 0.0
    if n.bit_length() <= 24:
        return float(n)
    shift = n.bit_length() - 24
    q, r = divmod(n, 1 << shift)
    half = 1 << (shift - 1)
    if r > half or (r == half and q % 2 == 1):
        q += 1
    return _f32(float(q) * 2.0 ** shift)


def single_sqrt_of_int(n: int) -> float:
    """(sqrt n) for an integer n: single-float."""
    x = int_to_single(n)
    # a correctly rounded single sqrt: the double sqrt rounded to single is
    # correctly rounded (doubles carry more than 2 * 24 + 2 bits)
    return _f32(math.sqrt(x))


def cl_round_int_by_single(n: int, s: float) -> int:
    """(round n s): n to single, single division, round the single to an integer."""
    x = int_to_single(n)
    qf = _f32(x / s)  # the double quotient of two singles, rounded once to single
    return cl_round_ratio(*float(qf).as_integer_ratio())


def _msb(m: int) -> int:
    s = mpz_size(m)
    return abs(m) >> (64 * (s - 1))


def estimate_reciprocal(a: MPD) -> MPD:
    assert a.m != 0
    size = mpz_size(a.m)
    est = cl_round_ratio(BASE, _msb(a.m))
    if a.m < 0:
        est = -est
    return MPD(est, -a.e - size)


def mpd_reciprocal(a: MPD, bits: int) -> MPD:
    digits = max(1, -(-bits // 64))
    x = estimate_reciprocal(a)
    while True:
        h = mpd_sub(integer_mpd(1), mpd_mul(a, x))
        zeros, zero = mpd_oom(h)
        zeros = -zeros
        if zero or zeros >= digits:
            return x
        x = mpd_add(x, mpd_mul(x, h))


def estimate_inv_sqrt(a: MPD) -> MPD:
    assert a.m >= 0
    size = mpz_size(a.m)
    msb = _msb(a.m)
    dexp = -1 - size - a.e
    if dexp % 2:
        est = cl_round_int_by_single(BASE, single_sqrt_of_int(BASE * msb))
        dexp += 1
    else:
        est = cl_round_int_by_single(BASE, single_sqrt_of_int(msb))
    return MPD(est, dexp // 2)


def mpd_inv_sqrt(a: MPD, bits: int) -> MPD:
    digits = max(1, -(-bits // 64))
    x = estimate_inv_sqrt(a)
    while True:
        h = mpd_sub(integer_mpd(1), mpd_mul(a, mpd_mul(x, x)))
        zeros, zero = mpd_oom(h)
        zeros = -zeros
        if zero or zeros >= digits:
            return x
        x = mpd_half(mpd_add(mpd_add(x, x), mpd_mul(x, h)))


def mpd_sqrt(a: MPD, bits: int) -> MPD:
    return mpd_mul(a, mpd_inv_sqrt(a, bits))


CHUD_BITS_PER_TERM = math.log(151931373056000) / math.log(2.0)


def mpd_pi(prec_bits: int) -> MPD:
    """mpd-pi (src/pi.lisp:53-74): pi/10, untruncated."""
    guard = prec_bits + 64
    num_terms = 2 + math.floor(guard / CHUD_BITS_PER_TERM)
    p, q, b, r = series_oracle.binary_split(series_oracle.chudnovsky_series(), 0, num_terms)
    final = mpd_sqrt(integer_mpd(10005), guard)
    final = mpd_mul(final, mpd_reciprocal(MPD(r, 0), guard))
    return mpd_mul(final, MPD(b * q, 0))


def digits_of(x: MPD, digits: int) -> int:
    """floor(10^digits * x)."""
    if x.e >= 0:
        return (x.m << (64 * x.e)) * 10 ** digits
    return (x.m * 10 ** digits) >> (-64 * x.e)
