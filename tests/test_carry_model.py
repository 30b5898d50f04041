"""The two-launch carry of hg_crt.cu, modelled on the CPU with small tiles.

The reconstruction leaves, at every position i, a coefficient V_i of three
64-bit words; the product is sum_i V_i 2^(64 i).  The kernels fold each
position's words into a low word A_i and a one-bit carry, scan every tile
with carry-in 0 (publishing the tile's generate/propagate pair), then a
second launch composes each tile's carry-in from the pairs below it and, where
it is 1, zeroes the tile's leading limbs equal to 2^64 - 1 and adds 1 to the
next.  This model follows those steps with 8-position tiles and checks the
limbs against Python's exact integer sum, on random coefficients and on the
patterns that make long propagate runs (all-ones products, sums whose carry
crosses many tiles).  The CUDA kernels themselves are checked on the GPU
(test_gpu_parity, test_gpu_batch, test_gpu_series).
"""

import random

MASK = (1 << 64) - 1
TILE = 8


def _exact(v):
    total = sum((w0 | (w1 << 64) | (w2 << 128)) << (64 * i) for i, (w0, w1, w2) in enumerate(v))
    return [(total >> (64 * i)) & MASK for i in range(len(v))], total >> (64 * len(v))


def _two_launch(v):
    n = len(v)
    # A_i = low word of v0_i + v1_(i-1) + v2_(i-2) + (its high part from i - 1)
    al, g, p = [], [], []
    whp = 0
    for i in range(n):
        w = v[i][0] + (v[i - 1][1] if i >= 1 else 0) + (v[i - 2][2] if i >= 2 else 0)
        wl, wh = w & MASK, w >> 64
        a = wl + whp
        al.append(a & MASK)
        g.append(a >> 64)
        p.append(1 if (a & MASK) == MASK and not (a >> 64) else 0)
        whp = wh
    spill = whp  # the high part of W_(n-1): lands at position n, as do v1_(n-1) and v2_(n-2)
    # launch 1: each tile with carry-in 0, aggregate (g, p)
    out, agg = [], []
    for t0 in range(0, n, TILE):
        c, tg, tp = 0, 0, 1
        for i in range(t0, min(t0 + TILE, n)):
            out.append((al[i] + c) & MASK)
            c = g[i] | (p[i] & c)
            tg, tp = g[i] | (p[i] & tg), p[i] & tp
        agg.append((tg, tp))
    # launch 2: carry-in of each tile from the aggregates below it, then the ripple
    top = 0
    for t in range(len(agg)):
        cin = 0
        for j in range(t - 1, -1, -1):  # nearest predecessor that does not propagate decides
            gj, pj = agg[j]
            if not pj:
                cin = gj
                break
        if t == len(agg) - 1:
            top = agg[t][0] | (agg[t][1] & cin)
        if cin:
            for i in range(t * TILE, min(t * TILE + TILE, n)):
                if out[i] == MASK:
                    out[i] = 0
                    continue
                out[i] += 1
                break
    return out, top, spill


def _check(v):
    got, top, spill = _two_launch(v)
    want, over = _exact(v)
    assert got == want
    # what lies above the n limbs: the scan's carry out of the top, the high
    # part of the top position's sum, and the words that start past the top
    n = len(v)
    above = top + spill + v[-1][1] + (v[-2][2] if n >= 2 else 0) + (v[-1][2] << 64)
    assert over == above


def _coeffs_of_product(x, y):
    """The exact convolution coefficients of two limb lists as 3-word values."""
    n = len(x) + len(y)
    c = [0] * n
    for i, a in enumerate(x):
        for j, b in enumerate(y):
            c[i + j] += a * b
    return [(z & MASK, (z >> 64) & MASK, z >> 128) for z in c]


def test_random_coefficients():
    rnd = random.Random(5)
    for n in (1, 2, 7, 8, 9, 31, 64, 100):
        for _ in range(20):
            _check([(rnd.getrandbits(64), rnd.getrandbits(64), rnd.getrandbits(58)) for _ in range(n)])


def test_all_ones_products():
    for nx, ny in ((1, 1), (5, 3), (8, 8), (17, 16), (40, 25), (64, 64)):
        _check(_coeffs_of_product([MASK] * nx, [MASK] * ny))


def test_carries_through_many_tiles():
    # 2^64 - 1 everywhere and a carry generated at position 0: the carry runs
    # through every tile, each of which propagates (p = 1).
    for n in (9, 40, 129):
        _check([(MASK, 0, 0)] * n)
        _check([(MASK, 1, 0)] + [(MASK, 0, 0)] * (n - 1))
        _check([(MASK, 0, 0)] * (n - 3) + [(2, 0, 0)] + [(0, 0, 0)] * 2)


def test_sparse_and_edge_values():
    rnd = random.Random(9)
    for n in (16, 33, 80):
        v = []
        for _ in range(n):
            r = rnd.random()
            if r < 0.3:
                v.append((MASK, MASK, 0))
            elif r < 0.6:
                v.append((MASK, 0, 0))
            elif r < 0.8:
                v.append((0, 0, 0))
            else:
                v.append((rnd.getrandbits(64), rnd.getrandbits(64), rnd.getrandbits(8)))
        _check(v)
