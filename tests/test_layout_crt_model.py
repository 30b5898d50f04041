"""Arithmetic the kernels rely on, modelled on the CPU.

* The prescaled reconstruction (hg_carry.cuh, CrtProducerT<_, true>): when a
  product's last inverse pass has folded N^-1 2^64 into its table, the
  residues are the coefficient c mod p_j, left in [0, 2p_j).  Garner then
  takes y0 = r0 folded, t1 = (r1 folded - y0 folded mod p1 + p1) p0^-1 mod p1,
  and t2 = (r2 - y0 folded mod p2 + p2) (p0 p1)^-1 - t1 p0 (p0 p1)^-1 mod p2.
  The model runs those steps with the same 64-bit operations (fold by the
  sign of x - p, Shoup products with their companions) and checks
  y0 + p0 t1 + p0 p1 t2 = c exactly, with the bounds the host checks before
  it prescales (p0 < 2 p1, p0 < 2 p2, 3 p2 < 2^64).
* The scale factors: N^-1 2^64 mod p_j in Montgomery form, so that a
  Montgomery product with a table entry w 2^64 yields the entry of w N^-1 2^64.
* The layouts of hg_internal.h: tw_pos (twiddle tables of the contiguous
  pass) is additive over disjoint bits and sends 8 lanes at a power-of-two
  stride of up to 2^8 entries to 8 different 16-byte bank quads; data_swz
  (contiguous-pass shared memory) sends the 16 lanes of a half-warp to 16
  different 8-byte bank pairs for the lane patterns of every round.

The CUDA code itself is checked on the GPU (test_gpu_parity,
test_gpu_configs_exact, test_gpu_chunked, test_gpu_batch).
"""

import random

MASK = (1 << 64) - 1
CS = (197, 174, 131)  # default-moduli, src/moduli.lisp:257-264
PS = tuple(c * (1 << 55) + 1 for c in CS)


def fold_p(x, p):
    """x - p when x >= p, for x < 2p: the sign of x - p decides (p < 2^63)."""
    assert 0 <= x < 2 * p
    d = (x - p) & MASK
    return x if d >> 63 else d


def shoup(a, w, p):
    """Shoup product a w mod p for any 64-bit a: q from the companion, one fold."""
    wq = (w << 64) // p
    q = (a * wq) >> 64
    r = (a * w - q * p) & MASK
    assert r < 2 * p
    return fold_p(r, p)


def sub_mod(a, b, p):
    return (a - b) % p


def garner_prescaled(r0, r1, r2):
    p0, p1, p2 = PS
    inv01 = pow(p0, -1, p1)
    inv012 = pow(p0 * p1 % p2, -1, p2)
    k2c = p0 % p2 * inv012 % p2
    y0 = fold_p(r0, p0)
    z1 = fold_p(r1, p1) - fold_p(y0, p1) + p1
    assert 0 < z1 < 2 * p1
    t1 = shoup(z1, inv01, p1)
    z2 = r2 - fold_p(y0, p2) + p2
    assert 0 < z2 < 3 * p2 <= MASK
    t2 = sub_mod(shoup(z2, inv012, p2), shoup(t1, k2c, p2), p2)
    return y0 + p0 * t1 + p0 * p1 * t2


def test_prescale_bounds_hold_for_the_scheme():
    p0, p1, p2 = PS
    assert p0 < 2 * p1 and p0 < 2 * p2 and 3 * p2 < (1 << 64)


def test_prescaled_garner_reconstructs_every_coefficient():
    rng = random.Random(7)
    M = PS[0] * PS[1] * PS[2]
    cases = [0, 1, M - 1, M // 2, (1 << 153) - 1, PS[0] - 1, PS[0], PS[0] * PS[1]]
    cases += [rng.randrange(M) for _ in range(20000)]
    for c in cases:
        # residues as the inverse pass leaves them: anywhere in [0, 2p)
        r = [c % p + (p if rng.random() < 0.5 and c % p < p else 0) for p in PS]
        assert garner_prescaled(*r) == c, c


def test_scale_factors_turn_the_table_into_the_coefficient():
    rng = random.Random(11)
    for L in (13, 19, 25, 27):
        N = 1 << L
        for p in PS:
            R = (1 << 64) % p
            s = pow(N, -1, p) * R % p  # N^-1 2^64, the factor the unscaled reconstruction applies
            S = s * R % p  # its Montgomery form, as prescale_factors builds it
            w = rng.randrange(1, p)
            wt = w * R % p  # a table entry: w in Montgomery form
            mont = wt * S * pow(R, -1, p) % p  # mont_mul(wt, S)
            assert mont == w * s % p * R % p  # the entry of w * s, Montgomery form
            # a residue r of N c 2^-64 times the scaled twiddle gives c
            c = rng.randrange(p)
            r = N * c * pow(R, -1, p) % p
            assert r * s % p == c


def tw_pos(e):
    return e + (e >> 3) + (e >> 6) + (e >> 9)


def data_swz(x):
    return x ^ ((x >> 4) & 15)


def test_tw_pos_is_additive_over_disjoint_bits():
    rng = random.Random(3)
    for _ in range(20000):
        e = rng.randrange(1 << 11)
        mask = rng.randrange(1 << 11)
        a, b = e & mask, e & ~mask
        assert tw_pos(a | b) == tw_pos(a) + tw_pos(b)


def test_tw_pos_spreads_strided_lanes_over_bank_quads():
    # 8 lanes of a 16-byte access read entries j 2^k (j < 8) plus a common part
    for k in range(0, 9):
        for base in range(0, 1 << 11, 97):
            if base & (7 << k):
                continue
            quads = {tw_pos(base | (j << k)) % 8 for j in range(8) if (base | (j << k)) < (1 << 11)}
            n = sum(1 for j in range(8) if (base | (j << k)) < (1 << 11))
            assert len(quads) == n, (k, base)


def test_data_swz_spreads_half_warps_over_bank_pairs():
    # lane bits of a half-warp in the contiguous pass's rounds (16 registers
    # per thread): position bits {4..7} (register block at 0) or {0..3}
    for lane_bits in ((4, 5, 6, 7), (0, 1, 2, 3)):
        for rest in range(0, 1 << 12, 113):
            base = rest
            for b in lane_bits:
                base &= ~(1 << b)
            pairs = {data_swz(base | sum(((j >> i) & 1) << b for i, b in enumerate(lane_bits))) % 16 for j in range(16)}
            assert len(pairs) == 16, (lane_bits, rest)


def test_data_swz_is_linear():
    rng = random.Random(5)
    for _ in range(10000):
        a, b = rng.randrange(1 << 12), rng.randrange(1 << 12)
        assert data_swz(a ^ b) == data_swz(a) ^ data_swz(b)
