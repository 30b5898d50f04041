"""ctypes wrapper of the C oracle (oracle/hg_oracle.c).

TEST INFRASTRUCTURE ONLY.  tests/, __graft_entry__.smoke() and bench.py's CPU
baseline leg use this module as the checker or the timed CPU restatement of
the reference; the shipped package never imports it.

The oracle restates hypergeometrica's Common Lisp multiplication path
(src/ntt-multiply.lisp, src/number-theoretic-transform.lisp,
src/modular-arithmetic.lisp, src/moduli.lisp, src/multiply.lisp,
src/mpz-ram.lisp).  Parity of the restatement is pinned by the golden
fixtures in tests/golden (an independent Python restatement checked against
DFT definitions and exact integer products) and by the known answers the
reference embeds (src/moduli.lisp:213-231, logs/24apr21-999-ram.txt:199).
"""

from __future__ import annotations

import ctypes
import os
import subprocess
import threading

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libhg_oracle.so")

_u64 = ctypes.c_uint64
_sz = ctypes.c_size_t
_vp = ctypes.c_void_p
_lock = threading.Lock()
_lib = None

SIGNATURES = {
    "hgo_primep": (ctypes.c_int, [_u64]),
    "hgo_next_prime": (_u64, [_u64]),
    "hgo_m_add": (_u64, [_u64, _u64, _u64]),
    "hgo_m_sub": (_u64, [_u64, _u64, _u64]),
    "hgo_m_mul": (_u64, [_u64, _u64, _u64]),
    "hgo_inv_mod": (_u64, [_u64, _u64]),
    "hgo_expt_mod": (_u64, [_u64, _u64, _u64]),
    "hgo_mod128_fast": (_u64, [_u64, _u64, _u64, _u64]),
    "hgo_m_mul_fast": (_u64, [_u64, _u64, _u64, _u64]),
    "hgo_calc_b_inv": (_u64, [_u64, _u64]),
    "hgo_m_mul_fast2": (_u64, [_u64, _u64, _u64, _u64]),
    "hgo_find_suitable_moduli": (ctypes.c_int, [_u64, ctypes.c_int, _vp]),
    "hgo_find_generator": (_u64, [_u64]),
    "hgo_primitive_root": (_u64, [_u64, _u64]),
    "hgo_default_moduli": (ctypes.c_int, [_vp, ctypes.c_int]),
    "hgo_default_scheme": (_vp, []),
    "hgo_scheme_root": (_u64, [_vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int]),
    "hgo_scheme_inv_root": (_u64, [_vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int]),
    "hgo_scheme_inv_length": (_u64, [_vp, ctypes.c_int, ctypes.c_int, ctypes.c_int]),
    "hgo_num_moduli_needed_for_bits": (ctypes.c_int, [_vp, _u64]),
    "hgo_ntt_forward": (None, [_vp, _sz, _vp, ctypes.c_int]),
    "hgo_ntt_reverse": (None, [_vp, _sz, _vp, ctypes.c_int]),
    "hgo_bit_reverse_permute": (None, [_vp, _sz]),
    "hgo_ntt_length": (_sz, [_sz, _sz]),
    "hgo_mpz_mul_ntt": (ctypes.c_int, [_vp, _sz, _vp, _sz, _vp, _sz]),
    "hgo_mpz_square": (ctypes.c_int, [_vp, _sz, _vp, _sz]),
    "hgo_mul_schoolboy": (ctypes.c_int, [_vp, _sz, _vp, _sz, _vp, _sz]),
    "hgo_mul_by_digit": (ctypes.c_int, [_vp, _sz, _u64, _vp, _sz]),
    "hgo_mpz_mul": (ctypes.c_int, [_vp, _sz, ctypes.c_int, _vp, _sz, ctypes.c_int, ctypes.c_int, _sz, _vp, _sz,
                                   ctypes.POINTER(_sz), ctypes.POINTER(ctypes.c_int)]),
    "hgo_set_threads": (None, [ctypes.c_int]),
    "hgo_get_threads": (ctypes.c_int, []),
}


def build() -> str:
    """Compile the oracle with its Makefile (plain C, seconds)."""
    subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB_PATH


def lib() -> ctypes.CDLL:
    global _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < os.path.getmtime(
                    os.path.join(HERE, "hg_oracle.c")):
                build()
            L = ctypes.CDLL(LIB_PATH)
            for name, (res, args) in SIGNATURES.items():
                f = getattr(L, name)
                f.restype = res
                f.argtypes = args
            _lib = L
        return _lib


def _p(a: np.ndarray):
    return a.ctypes.data_as(ctypes.c_void_p)


def _arr(x) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(x, dtype=np.uint64))


def scheme():
    return lib().hgo_default_scheme()


def moduli() -> list[int]:
    buf = np.zeros(8, dtype=np.uint64)
    n = lib().hgo_default_moduli(_p(buf), 8)
    return [int(v) for v in buf[:n]]


def ntt_forward(a, mod_num: int) -> np.ndarray:
    a = _arr(a).copy()
    lib().hgo_ntt_forward(_p(a), len(a), scheme(), mod_num)
    return a


def ntt_reverse(a, mod_num: int) -> np.ndarray:
    a = _arr(a).copy()
    lib().hgo_ntt_reverse(_p(a), len(a), scheme(), mod_num)
    return a


def bit_reverse_permute(a) -> np.ndarray:
    a = _arr(a).copy()
    lib().hgo_bit_reverse_permute(_p(a), len(a))
    return a


def _trim(a: np.ndarray) -> int:
    nz = np.flatnonzero(a)
    return int(nz[-1]) + 1 if nz.size else 0


def mpz_mul_ntt(x, y) -> np.ndarray:
    """Storage (transform length) returned by mpz-*/ntt."""
    x, y = _arr(x), _arr(y)
    n = lib().hgo_ntt_length(_trim(x), _trim(y))
    out = np.zeros(max(n, 1), dtype=np.uint64)
    rc = lib().hgo_mpz_mul_ntt(_p(x), len(x), _p(y), len(y), _p(out), len(out))
    if rc:
        raise RuntimeError(f"oracle mpz-*/ntt failed: {rc}")
    return out


def mpz_square(x) -> np.ndarray:
    x = _arr(x)
    n = lib().hgo_ntt_length(_trim(x), _trim(x))
    out = np.zeros(max(n, 1), dtype=np.uint64)
    rc = lib().hgo_mpz_square(_p(x), len(x), _p(out), len(out))
    if rc:
        raise RuntimeError(f"oracle mpz-square failed: {rc}")
    return out


def mul_schoolboy(x, y) -> np.ndarray:
    x, y = _arr(x), _arr(y)
    out = np.zeros(1 + len(x) + len(y), dtype=np.uint64)
    rc = lib().hgo_mul_schoolboy(_p(x), len(x), _p(y), len(y), _p(out), len(out))
    if rc:
        raise RuntimeError(f"oracle schoolboy failed: {rc}")
    return out


def mul_by_digit(x, d: int) -> np.ndarray:
    x = _arr(x)
    out = np.zeros(len(x) + 2, dtype=np.uint64)
    rc = lib().hgo_mul_by_digit(_p(x), len(x), d, _p(out), len(out))
    if rc:
        raise RuntimeError(f"oracle by-digit failed: {rc}")
    return out


def mpz_mul(x, sx: int, y, sy: int, same_object: bool = False, threshold: int = 100):
    """mpz-* dispatch; returns (trimmed magnitude, sign)."""
    x, y = _arr(x), _arr(y)
    out = np.zeros(len(x) + len(y) + 2 + hg_len(len(x), len(y)), dtype=np.uint64)
    nres = _sz(0)
    sres = ctypes.c_int(0)
    rc = lib().hgo_mpz_mul(_p(x), len(x), sx, _p(y), len(y), sy, int(same_object), threshold, _p(out), len(out),
                           ctypes.byref(nres), ctypes.byref(sres))
    if rc:
        raise RuntimeError(f"oracle mpz-* failed: {rc}")
    return out[: nres.value].copy(), sres.value


def hg_len(nx: int, ny: int) -> int:
    return int(lib().hgo_ntt_length(nx, ny))


def set_threads(n: int) -> None:
    lib().hgo_set_threads(n)
