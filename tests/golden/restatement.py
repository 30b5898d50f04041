"""Pure-Python restatement of hypergeometrica's multiplication path.

Test infrastructure only.  It is written independently of the C oracle
(oracle/hg_oracle.c) so that the two can pin each other, and it is small and
slow on purpose: Python integers stand in for the reference's SBCL bignums,
so every line can be read against the Common Lisp it restates (paths relative
to the hypergeometrica source tree).
"""

from __future__ import annotations

MODULUS_BITS = 63  # +modulus-bits+ (src/modular-arithmetic.lisp:12)
LG_MODULUS = MODULUS_BITS - 1  # +lg-modulus+ (:14)
BASE = 1 << 64  # $base (src/digit.lisp:12-13)
MASK64 = BASE - 1


# ---------------------------------------------------------------- digit.lisp
def mul128(x, y):
    """mul128 (src/digit.lisp:84-90): (lo, hi) of x*y."""
    r = x * y
    return r & MASK64, r >> 64


def div128(lo, hi, d):
    """div128 (src/digit.lisp:95-99): (quotient, remainder), truncating."""
    n = (hi << 64) | lo
    return n // d, n % d


def add128(alo, ahi, blo, bhi):
    """add128 (src/digit.lisp:104-114)."""
    s = alo + blo + (ahi + bhi) * BASE
    return s & MASK64, (s >> 64) & MASK64


def sub128(alo, ahi, blo, bhi):
    """sub128 (src/digit.lisp:116-131), two's complement modulo 2^128."""
    s = (alo - blo) + BASE * (ahi - bhi)
    s &= (1 << 128) - 1
    return s & MASK64, s >> 64


# ---------------------------------------------------- modular-arithmetic.lisp
def m_sub(a, b, m):
    """m- (src/modular-arithmetic.lisp:25-35)."""
    return (m - b) + a if a < b else a - b


def m_add(a, b, m):
    """m+ (src/modular-arithmetic.lisp:37-48)."""
    return a if b == 0 else m_sub(a, m - b, m)


def m_mul(a, b, m):
    """m* (src/modular-arithmetic.lisp:81-88)."""
    return (a * b) % m


def inv_mod(x, m):
    """inv-mod (src/modular-arithmetic.lisp:90-99)."""

    def egcd(x, b, a, u):
        while x != 0:
            q, r = divmod(b, x)
            x, b, a, u = r, x, u, a - u * q
        if b != 1:
            raise ArithmeticError(f"{x} is not invertible in Z/{m}Z")
        return a % m

    return egcd(x % m, m, 0, 1)


def expt_mod(a, n, m):
    """expt-mod / expt-mod/safe (src/modular-arithmetic.lisp:118-159)."""
    if n < 0:
        a, n = inv_mod(a, m), -n
    return pow(a, n, m)


def mod128_fast(lo, hi, m, m_inv):
    """mod128/fast (src/modular-arithmetic.lisp:167-188)."""
    a1 = ((hi & ((1 << LG_MODULUS) - 1)) << (64 - LG_MODULUS)) | (lo >> LG_MODULUS)
    q = mul128(a1, m_inv)[1]
    slo, shi = mul128(q, m)
    lo, hi = sub128(lo, hi, slo, shi)
    lo, hi = sub128(lo, hi, (2 * m) & MASK64, 0)
    lo, hi = add128(lo, hi, m & (hi >> 1), 0)
    return (lo + (m & hi)) & MASK64


def m_mul_fast(a, b, m, m_inv):
    """m*/fast (src/modular-arithmetic.lisp:190-202)."""
    lo, hi = mul128(a, b)
    return mod128_fast(lo, hi, m, m_inv)


def calc_b_inv(b, m):
    """calc-b-inv (src/modular-arithmetic.lisp:207-208)."""
    return div128(0, b, m)[0]


def m_mul_fast2(b, b_inv, a, m):
    """m*/fast2 (src/modular-arithmetic.lisp:211-231)."""
    q = mul128(a, b_inv)[1]
    r = ((a * b) - (q * m)) & MASK64
    if r >= m:
        r -= m
    return r


def garner(moduli, values):
    """garner (src/modular-arithmetic.lisp:235-267): mixed-radix digits."""
    k = len(moduli)
    x = list(values)
    for i in range(k):
        for j in range(i):
            r = inv_mod(moduli[j], moduli[i])
            x[i] = m_mul(r, m_sub(x[i], x[j] % moduli[i], moduli[i]), moduli[i])
    return x


def reconstruct_from_garner(moduli, mixed):
    """reconstruct-from-garner (src/modular-arithmetic.lisp:279-287)."""
    ans, prod = mixed[0], 1
    for i in range(1, len(moduli)):
        prod *= moduli[i - 1]
        ans += prod * mixed[i]
    return ans


# ------------------------------------------------------------- moduli.lisp
def primep(n):
    """primep (src/moduli.lisp:23-45) with fixed bases (exact below 3.3e24)."""
    if n == 1:
        return False
    if n < 4:
        return True
    if n % 2 == 0:
        return False
    d, s = n - 1, 0
    while d % 2 == 0:
        d //= 2
        s += 1
    for a in (2, 3, 5, 7, 11, 13, 17, 19, 23, 29, 31, 37, 41):
        if a % n == 0:
            continue
        x = pow(a, d, n)
        if x == 1 or x == n - 1:
            continue
        for _ in range(s - 1):
            x = x * x % n
            if x == n - 1:
                break
        else:
            return False
    return True


def next_prime(n):
    """next-prime (src/moduli.lisp:47-53)."""
    i = n if n % 2 else n - 1
    i += 2
    while not primep(i):
        i += 2
    return i


def next_power_of_two(n):
    """next-power-of-two (src/math-utilities.lisp:12-16)."""
    return n.bit_length() - 1 if n > 0 and n & (n - 1) == 0 else n.bit_length()


def factor_out(n, f):
    """factor-out (src/moduli.lisp:12-18)."""
    p = 0
    while n % f == 0:
        n //= f
        p += 1
    return n, p


def find_suitable_moduli(transform_length, count=1):
    """find-suitable-moduli (src/moduli.lisp:109-124)."""
    min_power = next_power_of_two(transform_length)
    step = 1 << min_power
    out, pm1 = [], step
    while count > 0:
        p = pm1 + 1
        if primep(p) and factor_out(p - 1, 2)[1] >= min_power:
            out.append(p)
            count -= 1
        pm1 += step
    return out


def factorize(n):
    """factorize (src/moduli.lisp:64-77)."""
    if primep(n):
        return [(n, 1)]
    out, f = [], 2
    while n != 1:
        n2, p = factor_out(n, f)
        if p:
            out.append((f, p))
            n = n2
        f = next_prime(f)
    return out


def find_finite_field_generator(m):
    """find-finite-field-generator (src/moduli.lisp:164-179)."""
    powers = [(m - 1) // f for f, _ in factorize(m - 1)]
    p = 2
    while any(pow(p, e, m) == 1 for e in powers):
        p = next_prime(p)
    return p


def find_primitive_root(n, m):
    """find-primitive-root (src/moduli.lisp:181-191)."""
    g = find_finite_field_generator(m)
    assert (m - 1) % n == 0
    return pow(g, (m - 1) // n, m)


def default_moduli():
    """default-moduli (src/moduli.lisp:257-264), restricted to the 63-bit ones
    the reference keeps (i*2^55+1 with 128 <= i < 256)."""
    ms = [(i << 55) + 1 for i in range(1, 256)]
    ms = [m for m in ms if m.bit_length() == MODULUS_BITS and primep(m)]
    return sorted(set(ms), reverse=True)


class Scheme:
    """make-modular-scheme (src/moduli.lisp:302-353), built lazily: the full
    roots table is (56 x k x 56 x 2); entries are computed on demand."""

    def __init__(self, moduli):
        self.moduli = sorted(moduli, reverse=True)
        self.max_trans = min(factor_out(m - 1, 2)[1] for m in self.moduli)
        self.lg_modulus = min(m.bit_length() - 1 for m in self.moduli)
        self.inverses = [(1 << (64 + self.lg_modulus)) // m for m in self.moduli]
        self._gen = {}

    def _g(self, i):
        if i not in self._gen:
            self._gen[i] = find_finite_field_generator(self.moduli[i])
        return self._gen[i]

    def root(self, power, i, k, which, inverse=False):
        m = self.moduli[i]
        w = pow(self._g(i), (m - 1) >> power, m)
        if inverse:
            w = inv_mod(w, m)
        wk = pow(w, 1 << k, m)  # expt-mod/2^n
        return wk if which == 0 else calc_b_inv(wk, m)

    def inv_length(self, power, i, which):
        m = self.moduli[i]
        v = inv_mod(1 << power, m)
        return v if which == 0 else calc_b_inv(v, m)


# ------------------------------------------- number-theoretic-transform.lisp
def lg(n):
    return n.bit_length() - 1


def ntt_forward(a, scheme, mod_num):
    """ntt-forward (src/number-theoretic-transform.lisp:40-90), in place."""
    m, mi = scheme.moduli[mod_num], scheme.inverses[mod_num]
    n = len(a)
    ln = lg(n)
    for lsubn in range(ln, 1, -1):
        subn = 1 << lsubn
        half = subn // 2
        dw = scheme.root(ln, mod_num, ln - lsubn, 0)
        dwi = scheme.root(ln, mod_num, ln - lsubn, 1)
        wj = 1
        for j in range(half):
            for r in range(0, n - subn + 1, subn):
                p, q = r + j, r + j + half
                u, v = a[p], a[q]
                a[p] = m_add(u, v, m)
                a[q] = m_mul_fast(wj, m_sub(u, v, m), m, mi)
            wj = m_mul_fast2(dw, dwi, wj, m)
    if ln > 0:
        for r in range(0, n, 2):
            u, v = a[r], a[r + 1]
            a[r], a[r + 1] = m_add(u, v, m), m_sub(u, v, m)
    return a


def ntt_reverse(a, scheme, mod_num):
    """ntt-reverse (src/number-theoretic-transform.lisp:93-143), in place."""
    m, mi = scheme.moduli[mod_num], scheme.inverses[mod_num]
    n = len(a)
    ldn = lg(n)
    invn, invni = scheme.inv_length(ldn, mod_num, 0), scheme.inv_length(ldn, mod_num, 1)
    if ldn > 0:
        for r in range(0, n, 2):
            u, v = a[r], a[r + 1]
            a[r], a[r + 1] = (m_mul_fast2(invn, invni, m_add(u, v, m), m),
                              m_mul_fast2(invn, invni, m_sub(u, v, m), m))
    for ldm in range(2, ldn + 1):
        subn = 1 << ldm
        half = subn // 2
        dw = scheme.root(ldn, mod_num, ldn - ldm, 0, inverse=True)
        dwi = scheme.root(ldn, mod_num, ldn - ldm, 1, inverse=True)
        wj = 1
        for j in range(half):
            for r in range(0, n - subn + 1, subn):
                p, q = r + j, r + j + half
                u = a[p]
                v = m_mul_fast(wj, a[q], m, mi)
                a[p], a[q] = m_add(u, v, m), m_sub(u, v, m)
            wj = m_mul_fast2(dw, dwi, wj, m)
    return a


def bit_reverse_permute(a):
    """bit-reversed-permute-vec! (src/strandh-elster-reversal.lisp:198-206)."""
    n = len(a)
    bits = max(0, (n - 1).bit_length())
    out = list(a)
    for i in range(n):
        r = int(format(i, f"0{bits}b")[::-1], 2) if bits else 0
        out[r] = a[i]
    return out


# Definitions used by the reference's own NTT tests (tests/ntt.lisp:12-89).
def ntt_forward_direct(v, m, w):
    n = len(v)
    return [sum(pow(w, j * k, m) * v[j] for j in range(n)) % m for k in range(n)]


def ntt_reverse_direct(v, m, w):
    n = len(v)
    wi = inv_mod(w, m)
    ninv = inv_mod(n, m)
    return [sum(pow(wi, j * k, m) * v[j] for j in range(n)) % m * ninv % m for k in range(n)]


# ----------------------------------------------------- ntt-multiply.lisp etc
def least_power_of_two_ge(n):
    """least-power-of-two->= (src/math-utilities.lisp:18-22)."""
    return n if n > 0 and n & (n - 1) == 0 else 1 << n.bit_length()


def mpz_size(digits):
    """mpz-size = vec-digit-length* (src/vec.lisp:218-229)."""
    n = len(digits)
    while n and digits[n - 1] == 0:
        n -= 1
    return n


def num_moduli_needed_for_bits(scheme, bits):
    """num-moduli-needed-for-bits (src/moduli.lisp:356-372)."""
    needed = 0
    while bits > 0:
        if needed == len(scheme.moduli):
            raise ArithmeticError("scheme does not support enough moduli")
        bits -= scheme.moduli[needed].bit_length()
        needed += 1
    return needed


def add_big_digit(big, storage, i):
    """add-big-digit (src/ntt-multiply.lisp:10-51) as integer addition."""
    while big:
        if i >= len(storage):
            raise ArithmeticError(f"Trying to add {big} at index {i}")
        s = storage[i] + (big & MASK64)
        storage[i] = s & MASK64
        big = (big >> 64) + (s >> 64)
        i += 1


def _crt(ntts, scheme, k, result, length):
    """The CRT block (src/ntt-multiply.lisp:242-253)."""
    moduli = scheme.moduli[:k]
    composite = 1
    for m in moduli:
        composite *= m
    complements = [composite // m for m in moduli]
    inverses = [inv_mod(c, m) for c, m in zip(complements, moduli)]
    factors = [c * v for c, v in zip(complements, inverses)]
    for i in range(length):
        d = sum(f * a[i] for a, f in zip(ntts, factors))
        add_big_digit(d % composite, result, i)


def mpz_mul_ntt(x, y, scheme):
    """mpz-*/ntt (src/ntt-multiply.lisp:174-254) on digit lists; returns the
    transform-length storage of the magnitude."""
    nx, ny = mpz_size(x), mpz_size(y)
    length = least_power_of_two_ge(nx + ny)
    bound_bits = (length * (BASE - 1) ** 2).bit_length()
    k = num_moduli_needed_for_bits(scheme, bound_bits)
    wx = [[d % m for d in x[:nx]] + [0] * (length - nx) for m in scheme.moduli]
    wy = [[d % m for d in y[:ny]] + [0] * (length - ny) for m in scheme.moduli]
    for i in range(k):
        ntt_forward(wx[i], scheme, i)
        ntt_forward(wy[i], scheme, i)
    for i in range(k):
        m, mi = scheme.moduli[i], scheme.inverses[i]
        wx[i] = [m_mul_fast(a, b, m, mi) for a, b in zip(wx[i], wy[i])]
    result = [0] * length
    for i in range(k):
        ntt_reverse(wx[i], scheme, i)
    _crt(wx[:k], scheme, k, result, length)
    return result


def mpz_square(x, scheme):
    """mpz-square (src/ntt-multiply.lisp:101-172)."""
    nx = mpz_size(x)
    length = least_power_of_two_ge(2 * nx)
    bound_bits = (length * (BASE - 1) ** 2).bit_length()
    k = num_moduli_needed_for_bits(scheme, bound_bits)
    w = [[d % m for d in x[:nx]] + [0] * (length - nx) for m in scheme.moduli]
    for i in range(k):
        ntt_forward(w[i], scheme, i)
    for i in range(k):
        m, mi = scheme.moduli[i], scheme.inverses[i]
        w[i] = [m_mul_fast(a, a, m, mi) for a in w[i]]
    for i in range(k):
        ntt_reverse(w[i], scheme, i)
    result = [0] * length
    _crt(w[:k], scheme, k, result, length)
    return result


def int_to_digits(n):
    """integer-mpz (src/mpz-ram.lisp:46-75) digits of |n|, little-endian."""
    n = abs(n)
    out = []
    while n:
        out.append(n & MASK64)
        n >>= 64
    return out


def digits_to_int(d):
    """mpz-integer (src/mpz-ram.lisp:38-44) of a magnitude."""
    return sum(v << (64 * i) for i, v in enumerate(d))
