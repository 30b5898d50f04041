"""Generate tests/golden/mpd_pi.json: the oracle's untruncated mpd-pi
(src/pi.lisp:53-74, restated in oracle/mpd_oracle.py) at precisions where the
mantissa grows to hundreds of millions of bits.

The reference never truncates, so its MPD-PI mantissa at b bits is far
longer than b: 11.9 million bits at b = 10^4, 142 million at 3 * 10^4.  The
oracle multiplies with Python integers (Karatsuba), which takes minutes at
those sizes; here mpd_mul's mantissa product runs through GMP's mpz_mul
instead (loaded with ctypes; prototypes hand-declared from the public GMP
manual).  Both are exact products, so the MPD is the same; the script checks
that at 10^4 bits against the unpatched oracle.

Each fixture records the exponent, the mantissa's sign and length in 64-bit
limbs, its lowest and highest limbs, and the SHA-256 of its little-endian
limbs.  Usage (in a checkout with the reference-free oracle; needs libgmp):

    python tests/golden/make_mpd_pi_golden.py [bits ...]
"""

from __future__ import annotations

import ctypes
import ctypes.util
import hashlib
import json
import os
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import mpd_oracle as M  # noqa: E402

DEFAULT_BITS = (10000, 30000, 1 << 15, 1 << 16)
OUT = os.path.join(HERE, "mpd_pi.json")


class _MPZ(ctypes.Structure):
    _fields_ = [("alloc", ctypes.c_int), ("size", ctypes.c_int), ("d", ctypes.c_void_p)]


def _gmp():
    name = ctypes.util.find_library("gmp")
    if not name:
        raise SystemExit("libgmp not found")
    g = ctypes.CDLL(name)
    P = ctypes.POINTER(_MPZ)
    for f in ("__gmpz_init", "__gmpz_clear"):
        getattr(g, f).argtypes = [P]
    g.__gmpz_import.argtypes = [P, ctypes.c_size_t, ctypes.c_int, ctypes.c_size_t, ctypes.c_int, ctypes.c_size_t,
                                ctypes.c_void_p]
    g.__gmpz_export.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_size_t), ctypes.c_int, ctypes.c_size_t,
                                ctypes.c_int, ctypes.c_size_t, P]
    g.__gmpz_export.restype = ctypes.c_void_p
    g.__gmpz_mul.argtypes = [P, P, P]
    return g


_G = None


def gmp_mul(a: int, b: int) -> int:
    """a * b through GMP for large operands (exact), Python otherwise."""
    if a.bit_length() < (1 << 16) or b.bit_length() < (1 << 16):
        return a * b
    global _G
    if _G is None:
        _G = _gmp()
    neg = (a < 0) != (b < 0)
    a, b = abs(a), abs(b)

    def load(v):
        z = _MPZ()
        _G.__gmpz_init(ctypes.byref(z))
        buf = v.to_bytes((v.bit_length() + 7) // 8, "little")
        _G.__gmpz_import(ctypes.byref(z), len(buf), -1, 1, 0, 0, buf)
        return z

    za, zb, zr = load(a), load(b), _MPZ()
    _G.__gmpz_init(ctypes.byref(zr))
    _G.__gmpz_mul(ctypes.byref(zr), ctypes.byref(za), ctypes.byref(zb))
    n = (a.bit_length() + b.bit_length() + 7) // 8
    out = ctypes.create_string_buffer(n + 8)
    cnt = ctypes.c_size_t(0)
    _G.__gmpz_export(out, ctypes.byref(cnt), -1, 1, 0, 0, ctypes.byref(zr))
    for z in (za, zb, zr):
        _G.__gmpz_clear(ctypes.byref(z))
    r = int.from_bytes(out.raw[: cnt.value], "little")
    return -r if neg else r


def fixture(x: M.MPD, bits: int, seconds: float) -> dict:
    m = abs(x.m)
    limbs = (m.bit_length() + 63) // 64
    raw = m.to_bytes(8 * limbs, "little")
    return {
        "bits": bits, "exponent": x.e, "sign": (x.m > 0) - (x.m < 0), "limbs": limbs,
        "low_limb": hex(int.from_bytes(raw[:8], "little")),
        "high_limb": hex(int.from_bytes(raw[-8:], "little")),
        "sha256": hashlib.sha256(raw).hexdigest(),
        "oracle_seconds": round(seconds, 1),
    }


def main(argv: list[str]) -> None:
    bits_list = [int(a) for a in argv] or list(DEFAULT_BITS)
    plain = M.mpd_pi(10000)  # the unpatched oracle
    M.mpd_mul = lambda a, b: M.MPD(gmp_mul(a.m, b.m), a.e + b.e)  # mpd_mul (mpd.lisp:83-88), exact
    check = M.mpd_pi(10000)
    assert (check.m, check.e) == (plain.m, plain.e), "GMP-backed oracle disagrees at 10^4 bits"
    out = []
    for bits in bits_list:
        t = time.time()
        x = M.mpd_pi(bits)
        f = fixture(x, bits, time.time() - t)
        print(json.dumps(f), flush=True)
        out.append(f)
    with open(OUT, "w") as fh:
        json.dump({"generator": "tests/golden/make_mpd_pi_golden.py", "fixtures": out}, fh, indent=1)
        fh.write("\n")


if __name__ == "__main__":
    main(sys.argv[1:])
