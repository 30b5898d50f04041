"""GMP's mpz_mul and mpz_ui_pow_ui through ctypes: third-party exact
products and powers, for checking and timing beside the oracle.  Test infrastructure, like the rest of this
directory: tests and bench.py's CPU-baseline leg use it to compare against
or to time; nothing on the product path does.

GMP's runtime (libgmp.so.10) ships with gcc, so it is on both the build
machine and the GPU host; its headers are not, so the prototypes below are
declared by hand from the public GMP manual (mpz_init, mpz_clear,
mpz_import, mpz_export, mpz_mul, mpz_ui_pow_ui; __mpz_struct is {int alloc;
int size; limb pointer}).
"""

from __future__ import annotations

import ctypes
import ctypes.util

import numpy as np


class _MPZ(ctypes.Structure):
    _fields_ = [("alloc", ctypes.c_int), ("size", ctypes.c_int), ("d", ctypes.c_void_p)]


_lib = None


def _load():
    global _lib
    if _lib is None:
        name = ctypes.util.find_library("gmp")
        if not name:
            raise OSError("libgmp not found")
        g = ctypes.CDLL(name)
        P = ctypes.POINTER(_MPZ)
        for f in ("__gmpz_init", "__gmpz_clear"):
            getattr(g, f).argtypes = [P]
        g.__gmpz_import.argtypes = [P, ctypes.c_size_t, ctypes.c_int, ctypes.c_size_t, ctypes.c_int,
                                    ctypes.c_size_t, ctypes.c_void_p]
        g.__gmpz_export.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_size_t), ctypes.c_int,
                                    ctypes.c_size_t, ctypes.c_int, ctypes.c_size_t, P]
        g.__gmpz_export.restype = ctypes.c_void_p
        g.__gmpz_mul.argtypes = [P, P, P]
        g.__gmpz_ui_pow_ui.argtypes = [P, ctypes.c_ulong, ctypes.c_ulong]
        _lib = g
    return _lib


def available() -> bool:
    try:
        _load()
        return True
    except OSError:
        return False


def _from_limbs(g, a: np.ndarray) -> _MPZ:
    z = _MPZ()
    g.__gmpz_init(ctypes.byref(z))
    a = np.ascontiguousarray(a, dtype=np.uint64)
    if a.size:
        g.__gmpz_import(ctypes.byref(z), a.size, -1, 8, 0, 0, a.ctypes.data)
    return z


def mul(x: np.ndarray, y: np.ndarray, timer=None) -> np.ndarray:
    """x * y for little-endian uint64 limb arrays: len(x) + len(y) limbs.
    With `timer` (a list), the seconds spent in mpz_mul alone are appended."""
    import time

    g = _load()
    zx, zy, zr = _from_limbs(g, x), _from_limbs(g, y), _MPZ()
    g.__gmpz_init(ctypes.byref(zr))
    t = time.perf_counter()
    g.__gmpz_mul(ctypes.byref(zr), ctypes.byref(zx), ctypes.byref(zy))
    if timer is not None:
        timer.append(time.perf_counter() - t)
    out = np.zeros(len(x) + len(y) + 1, dtype=np.uint64)
    cnt = ctypes.c_size_t(0)
    g.__gmpz_export(out.ctypes.data, ctypes.byref(cnt), -1, 8, 0, 0, ctypes.byref(zr))
    for z in (zx, zy, zr):
        g.__gmpz_clear(ctypes.byref(z))
    return out[: len(x) + len(y)]


def sqr(x: np.ndarray, timer=None) -> np.ndarray:
    """x * x through mpz_mul with one operand passed twice (GMP then squares):
    2 len(x) limbs.  With `timer` (a list), the seconds spent in mpz_mul are
    appended."""
    import time

    g = _load()
    zx, zr = _from_limbs(g, x), _MPZ()
    g.__gmpz_init(ctypes.byref(zr))
    t = time.perf_counter()
    g.__gmpz_mul(ctypes.byref(zr), ctypes.byref(zx), ctypes.byref(zx))
    if timer is not None:
        timer.append(time.perf_counter() - t)
    out = _export(g, zr, 2 * len(x) + 1)
    for z in (zx, zr):
        g.__gmpz_clear(ctypes.byref(z))
    full = np.zeros(2 * len(x), dtype=np.uint64)
    full[: len(out)] = out
    return full


def _export(g, z: _MPZ, nlimbs: int) -> np.ndarray:
    out = np.zeros(nlimbs, dtype=np.uint64)
    cnt = ctypes.c_size_t(0)
    g.__gmpz_export(out.ctypes.data, ctypes.byref(cnt), -1, 8, 0, 0, ctypes.byref(z))
    return out[: cnt.value]


def ui_pow_ui(base: int, exp: int, timer=None) -> np.ndarray:
    """base ** exp as little-endian uint64 limbs, without high zero limbs.
    With `timer` (a list), the seconds spent in mpz_ui_pow_ui are appended."""
    import math
    import time

    g = _load()
    z = _MPZ()
    g.__gmpz_init(ctypes.byref(z))
    t = time.perf_counter()
    g.__gmpz_ui_pow_ui(ctypes.byref(z), base, exp)
    if timer is not None:
        timer.append(time.perf_counter() - t)
    bits = int(exp * math.log2(base)) + 2 if base > 1 else 1
    out = _export(g, z, bits // 64 + 2)
    g.__gmpz_clear(ctypes.byref(z))
    return out
