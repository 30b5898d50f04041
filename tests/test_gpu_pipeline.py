"""hg_mul_host_pipeline on the GPU: many host-memory products in one call,
one product's download overlapping the next one's upload and transforms in a
second set of device buffers.  Every result must equal hg_mul's (hg_sqr's for
a square) limb for limb, tails zeroed, whether the buffers are pinned or
pageable, for every size class (one contiguous pass, strided passes,
unbalanced products in chunks, an empty operand) and with output buffers
reused two products apart."""

import numpy as np
import pytest

from hypergeometrica_gb300 import workloads as W

pytestmark = pytest.mark.gpu

SPECS = [(3, 5), (2000, 2048), (300000, 200001), (None, 70000), (1 << 20, 1 << 12), (0, 9), (5000, None),
         (1 << 19, 1 << 19), (777, 1)]


def _ref(hg, x, y, nout):
    out = np.zeros(nout, dtype=np.uint64)
    if y is None:
        got = hg.mpz_square(hg.MPZ(1, x)).storage
    else:
        got = hg.mpz_mul_ntt(hg.MPZ(1, x), hg.MPZ(1, y)).storage if len(x) and len(y) else np.zeros(0, np.uint64)
    n = min(len(got), nout)
    out[:n] = got[:n]
    assert not got[n:].any()
    return out


@pytest.mark.parametrize("pinned", [True, False])
def test_pipeline_matches_single_products(hg, pinned):
    import torch

    items, want = [], []
    for k, (nx, ny) in enumerate(SPECS):
        if nx is None:  # square of a long operand
            nx, ny, sq = ny, None, True
        x = W.limbs(40 + k, nx) if nx else np.zeros(0, dtype=np.uint64)
        y = None if ny is None else W.limbs(80 + k, ny)
        nout = (2 * nx if y is None else nx + ny) + (k % 3) * 5
        want.append(_ref(hg, x, y, nout))
        if pinned:
            tx = torch.from_numpy(x.view(np.int64)).pin_memory() if nx else torch.zeros(1, dtype=torch.int64).pin_memory()
            ty = None if y is None else torch.from_numpy(y.view(np.int64)).pin_memory()
            to = torch.full((nout,), -1, dtype=torch.int64).pin_memory()
            items.append((tx if nx else None, ty, to, nx))
        else:
            items.append((x, y, np.full(nout, 0xFFFFFFFFFFFFFFFF, dtype=np.uint64), nx))
    pl = []
    for x, y, out, nx in items:
        pl.append((x if nx else (np.zeros(0, dtype=np.uint64)), y, out))
    for _ in range(2):  # a second call reuses both lanes' buffers
        for _, _, out in pl:
            (out.fill_(-1) if hasattr(out, "fill_") else out.fill(0xFFFFFFFFFFFFFFFF))
        hg.mul_host_pipeline(pl)
        for k, (_, _, out) in enumerate(pl):
            got = out.numpy().view(np.uint64) if hasattr(out, "numpy") else out
            assert np.array_equal(got, want[k]), (k, SPECS[k])


def test_pipeline_shared_outputs_two_apart(hg):
    """Six products into two pinned output buffers, alternating: each buffer
    is written in list order, so it ends holding the last product it got."""
    import torch

    n = 1 << 18
    xs = [W.limbs(700 + k, n) for k in range(6)]
    ys = [W.limbs(800 + k, n) for k in range(6)]
    outs = [torch.zeros(2 * n, dtype=torch.int64).pin_memory() for _ in range(2)]
    hg.mul_host_pipeline([(torch.from_numpy(xs[k].view(np.int64)).pin_memory(),
                           torch.from_numpy(ys[k].view(np.int64)).pin_memory(), outs[k % 2]) for k in range(6)])
    for b, k in ((0, 4), (1, 5)):
        assert np.array_equal(outs[b].numpy().view(np.uint64), _ref(hg, xs[k], ys[k], 2 * n)), k
