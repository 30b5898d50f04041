"""ctypes binding of libhg_gb300.so (the C ABI in include/hypergeometrica_gb300.h).

The library is the only compute path: if it is missing or fails to load,
every call raises HGError.  There is no CPU fallback.
"""

from __future__ import annotations

import ctypes
import os
import re
import threading

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
LIB_PATH = os.path.join(HERE, "libhg_gb300.so")
# HG_CHECKED=1 in the environment loads the checked build instead (range,
# bounds and product checks in every kernel; see hg_build_checked).
CHECKED_LIB_PATH = os.path.join(HERE, "libhg_gb300_checked.so")
HEADER = os.path.join(ROOT, "include", "hypergeometrica_gb300.h")

HG_OK = 0
HG_ERR_ARG = -1
HG_ERR_MODULI = -2
HG_ERR_OOM = -3
HG_ERR_CUDA = -4
HG_ERR_INCONSISTENT = -5
HG_ERR_TIMEOUT = -6
HG_ERR_NOT_INIT = -7

ERROR_NAMES = {
    HG_ERR_ARG: "HG_ERR_ARG",
    HG_ERR_MODULI: "HG_ERR_MODULI",
    HG_ERR_OOM: "HG_ERR_OOM",
    HG_ERR_CUDA: "HG_ERR_CUDA",
    HG_ERR_INCONSISTENT: "HG_ERR_INCONSISTENT",
    HG_ERR_TIMEOUT: "HG_ERR_TIMEOUT",
    HG_ERR_NOT_INIT: "HG_ERR_NOT_INIT",
}


class HGError(RuntimeError):
    """A failed library call (the reference signals a CL error instead)."""

    def __init__(self, code: int, message: str):
        super().__init__(f"{ERROR_NAMES.get(code, code)}: {message}")
        self.code = code


_u64p = ctypes.POINTER(ctypes.c_uint64)
_sz = ctypes.c_size_t
_vp = ctypes.c_void_p


class HgHostProduct(ctypes.Structure):
    """hg_host_product: one product of hg_mul_host_pipeline (host pointers; y NULL squares x)."""

    _fields_ = [("x", _vp), ("nx", _sz), ("y", _vp), ("ny", _sz), ("out", _vp), ("nout", _sz)]


class HgProduct(ctypes.Structure):
    """hg_product: one product of a batch (device pointers; y NULL squares x)."""

    _fields_ = [("x", _vp), ("nx", _sz), ("y", _vp), ("ny", _sz), ("out", _vp), ("nout", _sz)]


HG_BATCH_AUTOTUNE = 1
HG_BATCH_PER_PASS = 2
HG_BATCH_PERSISTENT = 4


class HgPoly(ctypes.Structure):
    """hg_poly: an integer polynomial with an optional value at 0."""

    _fields_ = [("coef", ctypes.c_int64 * 8), ("degree", ctypes.c_int32), ("has_zero_value", ctypes.c_int32),
                ("zero_value", ctypes.c_int64)]


class HgSvcStats(ctypes.Structure):
    """hg_svc_report: counters and submit-to-completion latency of a service."""

    _fields_ = [("submitted", ctypes.c_uint64), ("completed", ctypes.c_uint64), ("failed", ctypes.c_uint64),
                ("batches", ctypes.c_uint64), ("pending", ctypes.c_uint64), ("in_flight", ctypes.c_uint64),
                ("peak_batch_products", ctypes.c_uint64), ("peak_batch_workspace_bytes", ctypes.c_uint64),
                ("slot_workspace_bytes", ctypes.c_uint64), ("latency_samples", ctypes.c_uint64),
                ("slots", ctypes.c_int), ("p50_us", ctypes.c_double), ("p99_us", ctypes.c_double),
                ("mean_us", ctypes.c_double), ("max_us", ctypes.c_double), ("products_per_s", ctypes.c_double)]

# name -> (restype, argtypes)
SIGNATURES = {
    "hg_init": (ctypes.c_int, [_u64p, ctypes.c_int, ctypes.c_int]),
    "hg_init_scheme": (ctypes.c_int, [_u64p, ctypes.c_int, _u64p, ctypes.c_int, ctypes.c_int]),
    "hg_shutdown": (ctypes.c_int, []),
    "hg_last_error": (ctypes.c_int, [ctypes.c_char_p, _sz]),
    "hg_build_checked": (ctypes.c_int, []),
    "hg_scheme_moduli": (ctypes.c_int, [_u64p, ctypes.c_int]),
    "hg_ntt_length": (_sz, [_sz, _sz]),
    "hg_chunk_plan": (ctypes.c_int, [_sz, _sz, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(_sz), ctypes.POINTER(_sz)]),
    "hg_set_chunking": (ctypes.c_int, [ctypes.c_int]),
    "hg_mul": (ctypes.c_int, [_vp, _sz, _vp, _sz, _vp, _sz]),
    "hg_sqr": (ctypes.c_int, [_vp, _sz, _vp, _sz]),
    "hg_mul_host_pipeline": (ctypes.c_int, [ctypes.POINTER(HgHostProduct), _sz]),
    "hg_mul_schoolboy": (ctypes.c_int, [_vp, _sz, _vp, _sz, _vp, _sz]),
    "hg_mul_digit": (ctypes.c_int, [_vp, _sz, ctypes.c_uint64, _vp, _sz]),
    "hg_mpz_mul": (ctypes.c_int, [_vp, _sz, ctypes.c_int, _vp, _sz, ctypes.c_int, ctypes.c_int, _sz, _vp, _sz,
                                  ctypes.POINTER(_sz), ctypes.POINTER(ctypes.c_int)]),
    "hg_mul_device": (ctypes.c_int, [_vp, _sz, _vp, _sz, _vp, _sz, _vp]),
    "hg_sqr_device": (ctypes.c_int, [_vp, _sz, _vp, _sz, _vp]),
    "hg_mul_schoolboy_device": (ctypes.c_int, [_vp, _sz, _vp, _sz, _vp, _sz, _vp]),
    "hg_mul_device_noalloc": (ctypes.c_int, [_vp, _sz, _vp, _sz, _vp, _sz, _vp]),
    "hg_sync": (ctypes.c_int, [_vp]),
    "hg_batch_create": (ctypes.c_int, [ctypes.POINTER(HgProduct), _sz, ctypes.c_int, ctypes.POINTER(_vp)]),
    "hg_batch_run": (ctypes.c_int, [_vp, _vp]),
    "hg_batch_destroy": (ctypes.c_int, [_vp]),
    "hg_batch_schedule": (ctypes.c_int, [_vp, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(_sz)]),
    "hg_mul_batch_device": (ctypes.c_int, [ctypes.POINTER(HgProduct), _sz, _vp]),
    "hg_add_batch_device": (ctypes.c_int, [_vp, _sz, _vp, _vp]),
    "hg_trim_batch_device": (ctypes.c_int, [_vp, _sz, _vp, _vp]),
    "hg_mul_small_batch_device": (ctypes.c_int, [_vp, _sz, _vp]),
    "hg_series_leaves_device": (ctypes.c_int, [_vp, ctypes.c_uint64, ctypes.c_uint64, _vp, _vp, _vp]),
    "hg_series_nodes_device": (ctypes.c_int, [_vp, _vp, ctypes.c_uint64, ctypes.c_uint64, _vp, _vp, _vp, _vp]),
    "hg_butterfly_peak": (ctypes.c_int, [ctypes.POINTER(ctypes.c_double)]),
    "hg_svc_open": (ctypes.c_int, [_sz, ctypes.c_int, _sz, ctypes.POINTER(_vp)]),
    "hg_svc_submit": (ctypes.c_int, [_vp, ctypes.POINTER(HgProduct), _sz, ctypes.POINTER(ctypes.c_uint64)]),
    "hg_svc_status": (ctypes.c_int, [_vp, ctypes.c_uint64]),
    "hg_svc_wait": (ctypes.c_int, [_vp, ctypes.c_uint64, ctypes.c_double]),
    "hg_svc_wait_all": (ctypes.c_int, [_vp, ctypes.c_double]),
    "hg_svc_stats": (ctypes.c_int, [_vp, ctypes.POINTER(HgSvcStats), ctypes.c_int]),
    "hg_svc_close": (ctypes.c_int, [_vp]),
    "hg_ntt_forward_device": (ctypes.c_int, [_vp, _sz, ctypes.c_int, _vp]),
    "hg_ntt_reverse_device": (ctypes.c_int, [_vp, _sz, ctypes.c_int, _vp]),
    "hg_profile_enable": (ctypes.c_int, [ctypes.c_int]),
    "hg_profile_read": (ctypes.c_int, [_u64p, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double),
                                       ctypes.c_int]),
}

def chunk_plan(nx: int, ny: int):
    """(log2 transform length, chunk limbs, chunks) of an nx x ny product run
    in chunks, or None when it runs as one transform."""
    L = ctypes.c_int()
    c = _sz()
    k = _sz()
    if not load().hg_chunk_plan(nx, ny, ctypes.byref(L), ctypes.byref(c), ctypes.byref(k)):
        return None
    return L.value, c.value, k.value


def set_chunking(on: bool) -> bool:
    """Allow (True) or forbid unbalanced products in chunks; returns the
    previous setting."""
    return bool(load().hg_set_chunking(1 if on else 0))


KERNEL_CLASSES = ["ntt_forward", "ntt_inverse", "middle", "carry", "small", "other", "batch"]


def profile_enable(on: bool) -> None:
    check(load().hg_profile_enable(1 if on else 0))


def profile_read() -> dict:
    """Per kernel class: launches, device ms (while recording) and algorithmic
    bytes since the last read."""
    n = len(KERNEL_CLASSES)
    la = (ctypes.c_uint64 * n)()
    ms = (ctypes.c_double * n)()
    by = (ctypes.c_double * n)()
    check(load().hg_profile_read(la, ms, by, n))
    return {k: {"launches": int(la[i]), "ms": float(ms[i]), "bytes": float(by[i])}
            for i, k in enumerate(KERNEL_CLASSES)}

_lock = threading.Lock()
_lib = None


def header_symbols(path: str = HEADER) -> list[str]:
    """Function names declared in the public header."""
    text = open(path).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    text = re.sub(r"//[^\n]*", "", text)
    return re.findall(r"\b(hg_[a-z0-9_]+)\s*\(", text)


def load() -> ctypes.CDLL:
    """Load the library (once).  Raises HGError when it is not built."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = CHECKED_LIB_PATH if os.environ.get("HG_CHECKED") == "1" else LIB_PATH
        if not os.path.exists(path):
            raise HGError(HG_ERR_NOT_INIT, f"{path} is not built; run `python -m hypergeometrica_gb300.build`"
                          + (" --checked" if path == CHECKED_LIB_PATH else ""))
        lib = ctypes.CDLL(path)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
        return lib


def last_error() -> str:
    buf = ctypes.create_string_buffer(512)
    load().hg_last_error(buf, len(buf))
    return buf.value.decode(errors="replace")


def check(rc: int) -> None:
    if rc != HG_OK:
        raise HGError(rc, last_error())
