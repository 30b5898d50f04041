"""Oracle for binary splitting and the Chudnovsky constant (TEST INFRASTRUCTURE).

A CPU restatement, on Python integers, of the reference's series code.  Only
tests/, __graft_entry__.smoke() and bench.py's CPU leg may use it, as the
checker; the library never calls it.

  binary_split       binary-split, binary-split-base-case=1 and combine
                     (src/binary-splitting.lisp:102-133), recursing exactly as
                     the reference does (split at floor((lower+upper)/2)).
  *_series           make-e-series, make-exp-series, make-ramanujan-series,
                     make-catalan-series, make-apery-series
                     (src/binary-splitting.lisp:147-231) and
                     make-chudnovsky-series (src/pi.lisp:24-43), each as a
                     tuple of functions (a, b, p, q).
  compute_pi_chudnovsky  compute-pi/chudnovsky (src/pi.lisp:45-51).
  residues           P, Q, B, R of [lower, upper) modulo a prime from their
                     closed forms in O(upper - lower): a size-independent check.

Pinned by pi_machin below: an independent computation of pi (Machin's
formula) that the restated Chudnovsky series must reproduce digit for digit.
"""

from __future__ import annotations

import math
import sys
from fractions import Fraction

sys.setrecursionlimit(10000)


def _one(n):
    return 1


def e_series():
    return (_one, _one, _one, lambda n: 1 if n == 0 else n)


def exp_series(x):
    x = Fraction(x)
    num, den = x.numerator, x.denominator
    return (_one, _one, lambda n: 1 if n == 0 else num, lambda n: 1 if n == 0 else n * den)


def ramanujan_series():
    # p(n) = (2n - 1)(4n - 3)(4n - 1), q(n) = n^3 396^4 / 8 (src/binary-splitting.lisp:174-193)
    return (lambda n: 1103 + 26390 * n, _one,
            lambda n: 1 if n == 0 else (2 * n - 1) * (4 * n - 3) * (4 * n - 1),
            lambda n: 1 if n == 0 else n ** 3 * (396 ** 4 // 8))


def catalan_series():
    return (_one, lambda n: 2 * n + 1, lambda n: 1 if n == 0 else n, lambda n: 1 if n == 0 else 4 * n + 2)


def apery_series():
    return (lambda n: 205 * n * n + 250 * n + 77, lambda n: 2,
            lambda n: 1 if n == 0 else -(n ** 5), lambda n: 32 * (2 * n + 1) ** 5)


def chudnovsky_series():
    # pi/10: a(n) = 10 (13591409 + 545140134 n), b = 8 * 640320 / 12,
    # p(n) = -(6n - 5)(2n - 1)(6n - 1), q(n) = n^3 640320^3 / 24 (src/pi.lisp:24-43)
    return (lambda n: 10 * (13591409 + 545140134 * n), lambda n: 8 * 640320 // 12,
            lambda n: 1 if n == 0 else -(6 * n - 5) * (2 * n - 1) * (6 * n - 1),
            lambda n: 1 if n == 0 else n ** 3 * (640320 ** 3 // 24))


def binary_split(series, lower, upper):
    """(P, Q, B, R) of [lower, upper)."""
    a, b, p, q = series
    if upper - lower == 1:
        pk = p(lower)
        return (pk, q(lower), b(lower), pk * a(lower))
    m = (lower + upper) // 2
    pl, ql, bl, rl = binary_split(series, lower, m)
    pr, qr, br, rr = binary_split(series, m, upper)
    return (pl * pr, ql * qr, bl * br, br * (qr * rl) + bl * (pl * rr))


def compute_pi_chudnovsky(prec):
    """floor(10^prec * pi / 10) by compute-pi/chudnovsky (src/pi.lisp:45-51)."""
    num_terms = math.floor(2 + prec / math.log10(151931373056000))
    sqrt_c = math.isqrt(10005 * 100 ** prec)
    p, q, b, r = binary_split(chudnovsky_series(), 0, num_terms)
    return (sqrt_c * (b * q)) // r


def pi_machin(digits):
    """floor(10^digits * pi), independently: pi = 16 atan(1/5) - 4 atan(1/239)."""
    guard = 20
    scale = 10 ** (digits + guard)

    def atan_inv(x):
        total, term, k, x2 = 0, scale // x, 0, x * x
        while term:
            total += term // (2 * k + 1) if k % 2 == 0 else -(term // (2 * k + 1))
            term //= x2
            k += 1
        return total

    return (16 * atan_inv(5) - 4 * atan_inv(239)) // 10 ** guard


def residues(series, lower, upper, m):
    """(P, Q, B, R) of [lower, upper) modulo m from the closed forms
    P = prod p(k), Q = prod q(k), B = prod b(k),
    R = sum_k a(k) p(lower)..p(k) q(k+1)..q(upper-1) prod_{j != k} b(j),
    which the combine recurrence unrolls to."""
    a, b, p, q = series
    ks = range(lower, upper)
    pv = [p(k) % m for k in ks]
    qv = [q(k) % m for k in ks]
    bv = [b(k) % m for k in ks]
    av = [a(k) % m for k in ks]
    n = len(pv)
    pre_p = [1] * (n + 1)
    pre_b = [1] * (n + 1)
    for i in range(n):
        pre_p[i + 1] = pre_p[i] * pv[i] % m
        pre_b[i + 1] = pre_b[i] * bv[i] % m
    suf_q = [1] * (n + 1)
    suf_b = [1] * (n + 1)
    for i in range(n - 1, -1, -1):
        suf_q[i] = suf_q[i + 1] * qv[i] % m
        suf_b[i] = suf_b[i + 1] * bv[i] % m
    r = 0
    for i in range(n):
        r = (r + av[i] * pre_p[i + 1] % m * suf_q[i + 1] % m * (pre_b[i] * suf_b[i + 1] % m)) % m
    return pre_p[n], suf_q[0], pre_b[n], r
