"""Host-side mirror of hypergeometrica's MPZ multiplication interface.

Names, argument meaning and error behaviour follow the Common Lisp reference
(paths relative to the hypergeometrica source tree):

  MPZ                 mpz/ram: a sign in {1, -1} and a little-endian storage
                      of 64-bit digits that may carry high zeros
                      (src/mpz-ram.lisp:19-24).
  mpz_size            mpz-size: digits up to the last nonzero one (src/vec.lisp:218-229).
  mpz_mul             mpz-* on two mpz/ram (src/multiply.lisp:12-49).
  mpz_mul_ntt         mpz-*/ntt (src/ntt-multiply.lisp:174-254): storage of the
                      transform length, sign sx*sy.
  mpz_square          mpz-square (src/ntt-multiply.lisp:101-172): storage of the
                      transform length, sign +1.
  mpz_multiply_by_digit  mpz-multiply-by-digit! (src/mpz-ram.lisp:367-395).
  multiply_storage_schoolboy  %multiply-storage/schoolboy (src/mpz-ram.lisp:404-431).
  f_expt / mpz_expt   (src/multiply.lisp:51-79).

Every product runs on the GPU through libhg_gb300.so; failures raise HGError
where the reference signals a CL error.
"""

from __future__ import annotations

import ctypes

import numpy as np

from ._lib import check, load

NTT_MULTIPLY_THRESHOLD = 100  # *ntt-multiply-threshold* (src/multiply.lisp:9-10)
DIGIT_BITS = 64


def digits_from_int(n: int) -> np.ndarray:
    """Little-endian uint64 digits of |n| (integer-mpz, src/mpz-ram.lisp:46-75)."""
    n = abs(int(n))
    if n == 0:
        return np.zeros(0, dtype=np.uint64)
    nbytes = (n.bit_length() + 63) // 64 * 8
    return np.frombuffer(n.to_bytes(nbytes, "little"), dtype="<u8").astype(np.uint64)


def int_from_digits(d) -> int:
    """Magnitude of a digit array (mpz-integer, src/mpz-ram.lisp:38-44)."""
    a = np.ascontiguousarray(np.asarray(d, dtype=np.uint64))
    return int.from_bytes(a.astype("<u8").tobytes(), "little")


def _size(d: np.ndarray) -> int:
    nz = np.flatnonzero(d)
    return int(nz[-1]) + 1 if nz.size else 0


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(ctypes.c_void_p)


class MPZ:
    """mpz/ram (src/mpz-ram.lisp:19-24)."""

    __slots__ = ("sign", "storage")

    def __init__(self, sign: int, storage):
        if sign not in (1, -1):
            raise ValueError("sign must be 1 or -1")
        self.sign = sign
        self.storage = np.ascontiguousarray(np.asarray(storage, dtype=np.uint64))

    @classmethod
    def from_int(cls, n: int) -> "MPZ":
        """integer-mpz (src/mpz-ram.lisp:46-75)."""
        return cls(-1 if n < 0 else 1, digits_from_int(n))

    def to_int(self) -> int:
        """mpz-integer (src/mpz-ram.lisp:38-44)."""
        return self.sign * int_from_digits(self.storage)

    def size(self) -> int:
        return mpz_size(self)

    def __repr__(self) -> str:
        return f"<MPZ {mpz_bit_size(self)} bits{'*' if len(self.storage) == self.size() else ''}>"


def mpz_size(x: MPZ) -> int:
    """mpz-size (src/mpz-ram.lisp:77-78)."""
    return _size(x.storage)


def mpz_bit_size(x: MPZ) -> int:
    """mpz-bit-size (src/mpz-ram.lisp:106-113)."""
    s = mpz_size(x)
    if s == 0:
        return 0
    return 64 * (s - 1) + int(x.storage[s - 1]).bit_length() + (x.sign - 1) // 2


def optimize_mpz(x: MPZ) -> MPZ:
    """optimize-mpz (src/mpz-ram.lisp:83-92): drop high zero digits."""
    x.storage = x.storage[: mpz_size(x)].copy()
    return x


def least_power_of_two_ge(n: int) -> int:
    """least-power-of-two->= (src/math-utilities.lisp:18-22)."""
    return n if n > 0 and n & (n - 1) == 0 else 1 << n.bit_length()


def _mag(x: MPZ) -> np.ndarray:
    return np.ascontiguousarray(x.storage[: mpz_size(x)])


def mpz_mul_ntt(x: MPZ, y: MPZ) -> MPZ:
    """mpz-*/ntt (src/ntt-multiply.lisp:174-254)."""
    a, b = _mag(x), _mag(y)
    length = least_power_of_two_ge(len(a) + len(b))
    out = np.zeros(length, dtype=np.uint64)
    check(load().hg_mul(_ptr(a), len(a), _ptr(b), len(b), _ptr(out), length))
    return MPZ(x.sign * y.sign, out)


def mpz_square(x: MPZ) -> MPZ:
    """mpz-square (src/ntt-multiply.lisp:101-172)."""
    a = _mag(x)
    length = least_power_of_two_ge(2 * len(a))
    out = np.zeros(length, dtype=np.uint64)
    check(load().hg_sqr(_ptr(a), len(a), _ptr(out), length))
    return MPZ(1, out)


def mul_host_pipeline(items) -> None:
    """Many NTT products of host arrays in one pipelined call
    (hg_mul_host_pipeline): items are (x, y_or_None, out) uint64 arrays (or
    pinned torch tensors, via .data_ptr()); out receives |x| * |y| (|x|^2
    when y is None) and zeros to its end.  Outputs shared by products must be
    at least two apart in the list."""
    from ._lib import HgHostProduct

    arr = (HgHostProduct * len(items))()
    keep = []
    for k, (x, y, out) in enumerate(items):
        def addr(a):
            if a is None:
                return None
            if hasattr(a, "data_ptr"):
                return a.data_ptr()
            keep.append(a)
            return a.ctypes.data

        n = (lambda a: 0 if a is None else (a.numel() if hasattr(a, "numel") else len(a)))
        arr[k] = HgHostProduct(addr(x), n(x), addr(y), n(y), addr(out), n(out))
    check(load().hg_mul_host_pipeline(arr, len(items)))


def multiply_storage_schoolboy(a: np.ndarray, a_size: int, b: np.ndarray, b_size: int) -> np.ndarray:
    """%multiply-storage/schoolboy (src/mpz-ram.lisp:404-431): storage of
    1 + a_size + b_size digits."""
    a = np.ascontiguousarray(a[:a_size], dtype=np.uint64)
    b = np.ascontiguousarray(b[:b_size], dtype=np.uint64)
    out = np.zeros(1 + a_size + b_size, dtype=np.uint64)
    check(load().hg_mul_schoolboy(_ptr(a), a_size, _ptr(b), b_size, _ptr(out), len(out)))
    return out


def mpz_multiply_by_digit(d: int, x: MPZ) -> MPZ:
    """The by-digit branch of mpz-* (src/multiply.lisp:33-38): a fresh MPZ with
    a storage of size(x) + 2 holding x * d."""
    a = _mag(x)
    out = np.zeros(len(a) + 2, dtype=np.uint64)
    check(load().hg_mul_digit(_ptr(a), len(a), ctypes.c_uint64(d), _ptr(out), len(out)))
    return MPZ(x.sign, out)


def mpz_mul(x: MPZ, y: MPZ, threshold: int | None = None) -> MPZ:
    """mpz-* (src/multiply.lisp:12-49); `threshold` overrides
    *ntt-multiply-threshold* for this call."""
    thr = NTT_MULTIPLY_THRESHOLD if threshold is None else threshold
    same = x is y
    optimize_mpz(x)
    if not same:
        optimize_mpz(y)
    if mpz_size(x) < mpz_size(y):
        x, y = y, x
    nx, ny = mpz_size(x), mpz_size(y)
    if ny == 0:
        return MPZ(1, np.zeros(0, dtype=np.uint64))
    if ny == 1:
        d = int(y.storage[0])
        if d == 1:
            return x if y.sign == 1 else MPZ(-x.sign, x.storage.copy())
        r = mpz_multiply_by_digit(d, x)
        r.sign = x.sign * y.sign
        return optimize_mpz(r)
    if ny <= thr:
        return optimize_mpz(MPZ(x.sign * y.sign, multiply_storage_schoolboy(x.storage, nx, y.storage, ny)))
    if same:
        return optimize_mpz(mpz_square(x))
    return optimize_mpz(mpz_mul_ntt(x, y))


def f_expt(a, n: int, one, multiply):
    """f-expt (src/multiply.lisp:51-75): left-to-right binary powering."""
    if n < 0:
        raise ValueError("n must be non-negative")
    if n == 0:
        return one
    if n == 1:
        return a
    x = a
    for bit in range(n.bit_length() - 2, -1, -1):
        x = multiply(x, x)
        if (n >> bit) & 1:
            x = multiply(x, a)
    return x


def mpz_expt(a: MPZ, n: int) -> MPZ:
    """mpz-expt (src/multiply.lisp:77-79)."""
    return f_expt(a, n, MPZ.from_int(1), mpz_mul)


def scheme_moduli() -> list[int]:
    """The scheme's moduli, largest first (scheme-moduli of **scheme**)."""
    buf = (ctypes.c_uint64 * 8)()
    n = load().hg_scheme_moduli(buf, 8)
    return [int(buf[i]) for i in range(n)]


def init(device: int = -1) -> None:
    """hg_init with the reference's default moduli (src/moduli.lisp:257-264)."""
    m = scheme_moduli()
    arr = (ctypes.c_uint64 * len(m))(*m)
    check(load().hg_init(arr, len(m), device))
