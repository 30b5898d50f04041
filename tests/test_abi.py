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
    assert lib.hg_build_checked() == 0  # the regular build; HG_CHECKED=1 selects the checked one
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
    with pytest.raises(H.HGError):
        H.mul_host_pipeline([(a, a, out), (a, None, out.copy())])


def _scheme_roots(oracle, maxlg):
    """w_{2^q} for every modulus, q = 0 .. maxlg, from the oracle's restated
    make-modular-scheme (the Lisp table's [q][i][0][0])."""
    s = oracle.scheme()
    L = oracle.lib()
    return [[int(L.hgo_scheme_root(s, q, i, 0, 0)) for q in range(maxlg + 1)] for i in range(3)]


def _init_scheme(lib, moduli, roots, maxlg):
    from hypergeometrica_gb300 import _lib

    m = (ctypes.c_uint64 * 3)(*moduli)
    flat = [w for row in roots for w in row]
    r = (ctypes.c_uint64 * len(flat))(*flat)
    rc = lib.hg_init_scheme(m, 3, r, maxlg, -1)
    return rc, _lib.last_error()


def test_init_checks_scheme_roots(lib, oracle):
    """hg_init_scheme accepts the reference's own roots table and rejects a
    perturbed one, or one past the scheme's 2^55 limit, with HG_ERR_NOT_INIT
    before touching the device (src/moduli.lisp:302-353)."""
    from hypergeometrica_gb300 import _lib

    moduli = oracle.moduli()
    good = _scheme_roots(oracle, 55)
    rc, _ = _init_scheme(lib, moduli, good, 55)
    assert rc in (_lib.HG_OK, _lib.HG_ERR_CUDA)  # HG_ERR_CUDA: no GPU in this process
    rc, _ = _init_scheme(lib, moduli, [row[:31] for row in good], 30)
    assert rc in (_lib.HG_OK, _lib.HG_ERR_CUDA)
    for i, q in ((0, 30), (1, 7), (2, 55), (0, 1)):
        bad = [row[:] for row in good]
        bad[i][q] = (bad[i][q] * 3) % moduli[i]
        rc, msg = _init_scheme(lib, moduli, bad, 55)
        assert rc == _lib.HG_ERR_NOT_INIT and f"2^{q}-th root" in msg, (i, q, msg)
    # roots of another generator: w_{2^q} = 5^((m - 1) / 2^q) is not the scheme's for modulus 0
    other = [row[:] for row in good]
    other[0] = [pow(5, (moduli[0] - 1) >> q, moduli[0]) for q in range(56)]
    rc, _ = _init_scheme(lib, moduli, other, 55)
    assert rc == _lib.HG_ERR_NOT_INIT
    rc, msg = _init_scheme(lib, moduli, [row + [1] for row in good], 56)
    assert rc == _lib.HG_ERR_NOT_INIT and "2^55" in msg
