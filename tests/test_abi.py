"""The C-ABI library builds, loads and exports every symbol the public header
declares (CPU only: no compute calls)."""

import ctypes
import glob
import os

import pytest

from conftest import ROOT


@pytest.fixture(scope="module")
def lib():
    from hypergeometrica_gb300 import build as B

    B.build()
    from hypergeometrica_gb300 import _lib

    return _lib.load()


def test_every_declared_symbol_is_exported(lib):
    from hypergeometrica_gb300 import _lib

    declared = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        declared.update(_lib.header_symbols(h))
    assert declared, "no declarations found"
    for name in sorted(declared):
        assert hasattr(lib, name), f"{name} declared but not exported"
    # The ctypes signatures cover the header exactly.
    assert declared == set(_lib.SIGNATURES)


def test_host_only_queries(lib):
    assert lib.hg_ntt_length(3, 5) == 8
    assert lib.hg_ntt_length(4096, 4096) == 8192
    assert lib.hg_ntt_length(4097, 4096) == 16384
    buf = (ctypes.c_uint64 * 4)()
    assert lib.hg_scheme_moduli(buf, 4) == 3
    assert list(buf)[:3] == [0x6280000000000001, 0x5700000000000001, 0x4180000000000001]


def test_chunk_plan_invariants(lib):
    """The unbalanced-product planner: chunks of C limbs (a multiple of 8)
    against the short operand fit a 2^L-point cyclic product without wrap,
    at most two chunk products meet at any position, the chunks cover the
    long operand exactly, and balanced products are not chunked."""
    from hypergeometrica_gb300 import _lib

    assert _lib.chunk_plan(1 << 24, 1 << 24) is None
    assert _lib.chunk_plan(100000, 31000) is None
    assert _lib.chunk_plan(0, 5) is None
    seen = set()
    for nl, ns in [(1 << 24, 1 << 16), (1 << 25, 1 << 20), (1 << 20, 1 << 6), (65536, 64), (3000, 7),
                   (1 << 18, 5), (200003, 1000), ((1 << 20) + 12345, 3001), (1 << 26, 2), (10 ** 6, 77777)]:
        for a, b in ((nl, ns), (ns, nl)):
            plan = _lib.chunk_plan(a, b)
            assert plan is not None, (a, b)
            L, c, k = plan
            T = 1 << L
            assert c % 8 == 0 and 2 * c >= T and c + ns <= T, plan
            assert (k - 1) * c < nl <= k * c and k >= 2, plan
            assert L < (nl + ns - 1).bit_length(), plan
            seen.add(L)
    assert any(L <= 12 for L in seen) and any(L > 12 for L in seen)
    # With chunking off every product runs as one transform.
    assert _lib.set_chunking(False) is True
    try:
        assert _lib.chunk_plan(1 << 24, 1 << 16) is None
    finally:
        assert _lib.set_chunking(True) is False
    assert _lib.chunk_plan(1 << 24, 1 << 16) is not None


def test_no_cpu_fallback_without_gpu(lib):
    """Without a GPU the product entry points fail loudly."""
    try:
        import torch

        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    import numpy as np

    import hypergeometrica_gb300 as H

    x = H.MPZ.from_int(3**500)
    with pytest.raises(H.HGError):
        H.mpz_mul_ntt(x, x)
    a = np.ones(4, dtype=np.uint64)
    out = np.zeros(8, dtype=np.uint64)
    assert lib.hg_mul(a.ctypes.data, 4, a.ctypes.data, 4, out.ctypes.data, 8) != 0
