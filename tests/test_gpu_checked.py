"""The checked build (libhg_gb300_checked.so, -DHG_CHECKED=1) on the GPU.

It does what the reference does with :hypergeometrica-safe and -paranoid
(src/config.lisp:31-37): every residue a pass reads or writes is checked
against its range, every residue index against its array, and every modular
product against an exact reduction of the 128-bit product.  The parity
checks below run under it at small sizes and must stay bit-exact with the
oracle and fault-free; a forward spectrum whose input holds a value >= p
(ntt-forward asserts its inputs are below m,
src/number-theoretic-transform.lisp:63-64) must be reported as
HG_ERR_INCONSISTENT by the next hg_sync.  The checked library is loaded in a
child process (HG_CHECKED=1), since a process loads one build.
"""

import os
import subprocess
import sys

import pytest

from conftest import ROOT

pytestmark = pytest.mark.gpu

SCRIPT = r"""
import os
import sys
root = os.environ["HG_TEST_ROOT"]
sys.path[:0] = [root, os.path.join(root, "oracle")]
import numpy as np
import torch

import hypergeometrica_gb300 as H
import oracle as O
from hypergeometrica_gb300 import _lib
from hypergeometrica_gb300 import device as D
from hypergeometrica_gb300 import workloads as W

assert _lib.load().hg_build_checked() == 1, "the regular build was loaded"
assert _lib.load()._name.endswith("libhg_gb300_checked.so")
H.init(0)
# single pass (2^3, 2^7), strided + contiguous (2^13, 2^14), chunked (20000 x 300), squares
for nx, ny in [(3, 5), (100, 28), (3000, 2500), (9000, 7000), (20000, 300)]:
    for dist in ("uniform", "ones"):
        x, y = W.limbs(nx, nx, dist), W.limbs(ny + 7, ny, dist)
        got = H.mpz_mul_ntt(H.MPZ(1, x), H.MPZ(1, y)).storage
        assert np.array_equal(got, O.mpz_mul_ntt(x, y)), (nx, ny, dist)
        got = H.mpz_square(H.MPZ(1, x)).storage
        assert np.array_equal(got, O.mpz_square(x)), (nx, dist)
# spectra, and a batch (the persistent launch and the per-pass schedule)
for lg in (5, 13, 16):
    v = W.splitmix64(lg, 1 << lg) % np.uint64(O.moduli()[1])
    t = torch.from_numpy(v.view(np.int64)).cuda()
    D.ntt_forward(t, 1)
    D.sync()
    assert np.array_equal(t.cpu().numpy().view(np.uint64), O.ntt_forward(v, 1)), lg
    D.ntt_reverse(t, 1)
    D.sync()
    assert np.array_equal(t.cpu().numpy().view(np.uint64), v), lg
items, want = [], []
for k in range(40):
    nx, ny = 50 + 97 * k, 30 + 211 * k
    x, y = W.limbs(500 + k, nx), W.limbs(600 + k, ny)
    out = torch.full((nx + ny,), -1, dtype=torch.int64, device="cuda")
    items.append((torch.from_numpy(x.view(np.int64)).cuda(), torch.from_numpy(y.view(np.int64)).cuda(), out))
    want.append(O.mpz_mul_ntt(x, y)[: nx + ny])
for sched in ("persistent", "per_pass"):
    b = D.Batch(items, autotune=False, schedule=sched)
    b.run()
    D.sync()
    for k, it in enumerate(items):
        assert np.array_equal(it[2].cpu().numpy().view(np.uint64), want[k]), (sched, k)
    b.close()
# a forward spectrum input >= p is reported, and the library keeps working
m = O.moduli()[0]
v = W.splitmix64(5, 1 << 13) % np.uint64(m)
v[17] = np.uint64(m + 3)
t = torch.from_numpy(v.view(np.int64)).cuda()
D.ntt_forward(t, 0)
try:
    D.sync()
    raise SystemExit("an input >= p went unreported")
except _lib.HGError as e:
    assert e.code == _lib.HG_ERR_INCONSISTENT and "range" in str(e), e
D.sync()  # the report cleared the fault words
x = W.limbs(9, 4000)
assert np.array_equal(H.mpz_square(H.MPZ(1, x)).storage, O.mpz_square(x))
print("checked build ok")
"""


def test_checked_build_parity_and_range_fault(hg):
    from hypergeometrica_gb300 import build as B

    B.build(checked=True)
    env = dict(os.environ, HG_CHECKED="1", HG_TEST_ROOT=ROOT)
    r = subprocess.run([sys.executable, "-c", SCRIPT], env=env,
                       capture_output=True, text=True, timeout=900)
    assert r.returncode == 0 and "checked build ok" in r.stdout, r.stdout[-3000:] + r.stderr[-3000:]
