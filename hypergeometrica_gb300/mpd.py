"""Dyadic floats (MPD) and mpd-pi with the mantissas on the GPU.

Mirrors the reference (paths relative to its source tree):

  MPD                      mpd (src/mpd.lisp:7-12): mantissa * $base^exponent,
                           $base = 2^64; the mantissa is a DeviceInt.
  mpz_mpd, integer_mpd     (:14-17, :44-45)
  mpd_oom                  (:23-39)
  mpd_mul, mpd_add,        mpd-*, mpd-+, mpd--, mpd-negate, mpd-half!
  mpd_sub, mpd_negate,     (:72-102)
  mpd_half
  mpd_truncate             mpd-truncate! (:53-70)
  estimate_reciprocal,     src/mpd-reciprocal.lisp:7-73
  mpd_reciprocal
  estimate_inv_sqrt,       src/mpd-sqrt.lisp:7-90
  mpd_inv_sqrt, mpd_sqrt
  mpd_pi                   src/pi.lisp:53-74: pi/10 to prec_bits bits.

mpd_pi follows the reference exactly: its Newton iterations never truncate,
so the result's mantissa grows with the square of the precision (about
7.8 million limbs at 2^16 bits); the value is bit-identical to the
reference's.  mpd_pi_truncated is NOT the reference's result: it keeps each
Newton iterate to the working precision (the mpd-truncate! that
src/pi.lisp:72 leaves commented out), which is what makes 2^22 to 2^26 bits
feasible; its value agrees with pi/10 to the requested bits.

Products run through the device-resident multiply service when one is given
(series.multiply), sums through hg_add_batch_device; the two float seeds
(estimate-reciprocal's (round $base msb) and estimate-inv-sqrt's single-float
sqrt) are computed on the host exactly as SBCL computes them.
"""

from __future__ import annotations

import math
import struct

import numpy as np

from . import series as S
from .series import DeviceInt

BASE = 1 << 64


class MPD:
    __slots__ = ("mantissa", "exponent")

    def __init__(self, mantissa: DeviceInt, exponent: int):
        self.mantissa = mantissa
        self.exponent = int(exponent)

    def to_pair(self):
        """(mantissa as a Python int, exponent)."""
        return self.mantissa.to_int(), self.exponent

    def digits(self, n: int) -> int:
        """floor(10^n * value)."""
        m, e = self.to_pair()
        return (m << (64 * e)) * 10 ** n if e >= 0 else (m * 10 ** n) >> (-64 * e)


def mpz_mpd(x: DeviceInt) -> MPD:
    return MPD(x, 0)


def integer_mpd(n: int) -> MPD:
    return MPD(DeviceInt.from_int(n), 0)


def mpd_oom(x: MPD):
    if x.mantissa.size == 0:
        return 0, True
    return min(0, x.mantissa.size + x.exponent), False


def _shift(x: DeviceInt, limbs: int) -> DeviceInt:
    """x * 2^(64 limbs) (mpz-left-shift by whole digits, src/mpz-ram.lisp:310-332)."""
    import torch

    if limbs == 0 or x.size == 0:
        return x
    t = torch.zeros(limbs + x.size, dtype=torch.int64, device="cuda")
    t[limbs:] = x.t[: x.size]
    return DeviceInt(x.sign, t, x.size + limbs)


def mpz_add(x: DeviceInt, y: DeviceInt) -> DeviceInt:
    """mpz-+ (src/mpz-ram.lisp:292-306)."""
    import torch

    if x.size == 0:
        return y
    if y.size == 0:
        return x
    nout = max(x.size, y.size) + 1
    out = torch.empty(nout, dtype=torch.int64, device="cuda")
    rec = np.array([[x.ptr(), x.size, y.ptr(), y.size, out.data_ptr(), nout,
                     np.int64(x.sign).view(np.uint64), np.int64(y.sign).view(np.uint64)]], dtype=np.uint64)
    (sign, size), = S._sum_records(rec)
    return DeviceInt(int(sign), out, int(size))


def mpd_mul(a: MPD, b: MPD, service=None) -> MPD:
    return MPD(S.multiply(a.mantissa, b.mantissa, service), a.exponent + b.exponent)


def mpd_add(a: MPD, b: MPD) -> MPD:
    lo = min(a.exponent, b.exponent)
    return MPD(mpz_add(_shift(a.mantissa, a.exponent - lo), _shift(b.mantissa, b.exponent - lo)), lo)


def mpd_negate(a: MPD) -> MPD:
    m = a.mantissa
    return MPD(DeviceInt(-m.sign, m.t, m.size), a.exponent)


def mpd_sub(a: MPD, b: MPD) -> MPD:
    return mpd_add(a, mpd_negate(b))


def mpd_half(a: MPD, service=None) -> MPD:
    """mpd-half!: mantissa times $base/2, exponent - 1."""
    return MPD(S.multiply(a.mantissa, DeviceInt.from_int(BASE // 2), service), a.exponent - 1)


def mpd_truncate(a: MPD, limbs: int) -> MPD:
    """mpd-truncate! to at least `limbs` digits: drop the low digits beyond."""
    m = a.mantissa
    if limbs >= m.size:
        return a
    d = m.size - limbs
    return MPD(DeviceInt(m.sign, m.t[d: m.size], limbs), a.exponent + d)


# ---- the float seeds, as SBCL computes them --------------------------------


def _cl_round_ratio(n: int, d: int) -> int:
    """CL (round n d) on integers: nearest, ties to even."""
    q, r = divmod(n, d)
    if 2 * r > d or (2 * r == d and q % 2 == 1):
        q += 1
    return q


def _f32(x: float) -> float:
    return struct.unpack("<f", struct.pack("<f", x))[0]


def _int_to_single(n: int) -> float:
    if n.bit_length() <= 24:
        return float(n)
    shift = n.bit_length() - 24
    q, r = divmod(n, 1 << shift)
    half = 1 << (shift - 1)
    if r > half or (r == half and q % 2 == 1):
        q += 1
    return _f32(float(q) * 2.0 ** shift)


def _round_int_by_single(n: int, s: float) -> int:
    return _cl_round_ratio(*float(_f32(_int_to_single(n) / s)).as_integer_ratio())


def _msb(x: DeviceInt) -> int:
    return int(x.t[x.size - 1].item()) & (BASE - 1)


def estimate_reciprocal(a: MPD) -> MPD:
    m = a.mantissa
    if m.size == 0:
        raise ZeroDivisionError("reciprocal of zero")
    est = _cl_round_ratio(BASE, _msb(m))
    return MPD(DeviceInt.from_int(-est if m.sign < 0 else est), -a.exponent - m.size)


def mpd_reciprocal(a: MPD, bits: int, service=None, truncate: bool = False) -> MPD:
    """Newton on f(x) = 1/x - a: x <- x + x h, h = 1 - a x.  With truncate,
    each step works at twice the previous step's precision (a, x and h kept
    to it), up to the requested digits plus two."""
    digits = max(1, -(-bits // 64))
    x = estimate_reciprocal(a)
    one = integer_mpd(1)
    prec = 2
    while True:
        at = mpd_truncate(a, prec + 2) if truncate else a
        h = mpd_sub(one, mpd_mul(at, x, service))
        zeros, zero = mpd_oom(h)
        if (zero or -zeros >= digits) and (not truncate or prec >= digits + 2):
            return x
        if truncate:
            h = mpd_truncate(h, prec + 2)
        x = mpd_add(x, mpd_mul(x, h, service))
        if truncate:
            prec = min(2 * prec, digits + 2)
            x = mpd_truncate(x, prec + 2)


def estimate_inv_sqrt(a: MPD) -> MPD:
    m = a.mantissa
    if m.sign < 0 and m.size:
        raise ValueError("inverse square root of a negative number")
    size, msb = m.size, _msb(m)
    dexp = -1 - size - a.exponent
    if dexp % 2:
        est = _round_int_by_single(BASE, _f32(math.sqrt(_int_to_single(BASE * msb))))
        dexp += 1
    else:
        est = _round_int_by_single(BASE, _f32(math.sqrt(_int_to_single(msb))))
    return MPD(DeviceInt.from_int(est), dexp // 2)


def mpd_inv_sqrt(a: MPD, bits: int, service=None, truncate: bool = False) -> MPD:
    """Newton on f(x) = 1/x^2 - a: x <- (2x + x h) / 2, h = 1 - a x^2.  With
    truncate, precision doubles step by step as in mpd_reciprocal."""
    digits = max(1, -(-bits // 64))
    x = estimate_inv_sqrt(a)
    one = integer_mpd(1)
    prec = 2
    while True:
        at = mpd_truncate(a, prec + 2) if truncate else a
        xx = mpd_mul(x, x, service)
        if truncate:
            xx = mpd_truncate(xx, prec + 2)
        h = mpd_sub(one, mpd_mul(at, xx, service))
        zeros, zero = mpd_oom(h)
        if (zero or -zeros >= digits) and (not truncate or prec >= digits + 2):
            return x
        if truncate:
            h = mpd_truncate(h, prec + 2)
        x = mpd_half(mpd_add(mpd_add(x, x), mpd_mul(x, h, service)), service)
        if truncate:
            prec = min(2 * prec, digits + 2)
            x = mpd_truncate(x, prec + 2)


def mpd_sqrt(a: MPD, bits: int, service=None, truncate: bool = False) -> MPD:
    return mpd_mul(a, mpd_inv_sqrt(a, bits, service, truncate), service)


def mpd_pi(prec_bits: int, service=None, timings: dict | None = None) -> MPD:
    """mpd-pi (src/pi.lisp:53-74): pi/10, bit-identical to the reference's."""
    return _pi(prec_bits, service, False, timings)


def mpd_pi_truncated(prec_bits: int, service=None, timings: dict | None = None) -> MPD:
    """pi/10 to prec_bits bits with each Newton iterate truncated to the working
    precision: not the reference's (untruncated) mantissa."""
    return _pi(prec_bits, service, True, timings)


def _pi(prec_bits, service, truncate, timings):
    import time

    import torch

    t = {} if timings is None else timings
    guard = prec_bits + 64
    num_terms = S.chudnovsky_terms(prec_bits)
    t0 = time.perf_counter()
    comp = S.binary_split(S.make_chudnovsky_series(), 0, num_terms, service)
    torch.cuda.synchronize()
    t["split_s"] = time.perf_counter() - t0
    t0 = time.perf_counter()
    final = mpd_sqrt(integer_mpd(10005), guard, service, truncate)
    t["sqrt_s"] = time.perf_counter() - t0
    t0 = time.perf_counter()
    num = mpz_mpd(S.partial_numerator(comp))
    if truncate:  # 1/R to the working precision needs only R's top digits
        num = mpd_truncate(num, -(-guard // 64) + 2)
    recip = mpd_reciprocal(num, guard, service, truncate)
    if truncate:
        final = mpd_truncate(final, -(-guard // 64) + 2)
    final = mpd_mul(final, recip, service)
    t["recip_s"] = time.perf_counter() - t0
    t0 = time.perf_counter()
    final = mpd_mul(final, mpz_mpd(S.partial_denominator(comp, service)), service)
    if truncate:
        final = mpd_truncate(final, -(-guard // 64) + 2)
    torch.cuda.synchronize()
    t["final_s"] = time.perf_counter() - t0
    t["terms"] = num_terms
    return final
