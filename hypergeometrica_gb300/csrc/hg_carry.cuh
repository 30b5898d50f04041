// hg_carry.cuh -- reconstruction and carry bodies shared by the per-launch
// carry kernels (hg_crt.cu) and the persistent batch kernel (hg_persist.cu).
//
// The reference rebuilds each convolution coefficient as a bignum
// sum_j f_j r_j mod M and adds it at limb i with a recursive carry ripple
// (src/ntt-multiply.lisp:10-51, 242-253).  CrtProducer gives each
// coefficient by Garner's mixed radix; carry_body writes one tile of limbs
// with carry-in 0 and publishes the tile's (generate, propagate) aggregate;
// fix_body, run after every tile of the product has published, composes a
// tile's carry-in from the aggregates below it and applies it.
#pragma once

#include "hg_internal.h"

namespace hg {
namespace carry {

constexpr int kCarryPer = 8;  // positions per thread

template <int TILE>
__device__ __forceinline__ uint64_t carry_tiles_dev(uint64_t n) { return (n + TILE - 1) / TILE; }

struct V3 {
  uint64_t w0, w1, w2;
};

__device__ __forceinline__ void add128_to(V3 &acc, uint64_t lo, uint64_t hi) {
  const uint64_t s0 = acc.w0 + lo;
  const uint64_t c0 = s0 < lo;
  const uint64_t t1 = acc.w1 + hi;
  const uint64_t c1 = t1 < hi;
  const uint64_t s1 = t1 + c0;
  const uint64_t c2 = s1 < c0;
  acc.w0 = s0;
  acc.w1 = s1;
  acc.w2 += c1 + c2;
}

// COHERENT: the residues were written earlier in the same launch (the
// persistent batch kernel), so they are read through L2 (ld.global.cg)
// rather than the read-only data path, which is coherent only for data no
// CTA of the launch writes.  PRESCALED: the residues are the coefficients
// mod p_j (CrtConst::prescaled).
template <bool COHERENT = false, bool PRESCALED = false>
struct CrtProducerT {
  const uint64_t *res;  // [3][N] natural-order residues from the unscaled inverse
  uint64_t n;           // N
  CrtConst k;

  __device__ __forceinline__ static ulonglong2 load2(const ulonglong2 *p) {
    if constexpr (COHERENT)
      return __ldcg(p);
    else
      return __ldg(p);
  }

  // Coefficient i of the product whose residues start `off` words past res.
  __device__ __forceinline__ V3 at(uint64_t off, uint64_t i) const {
    const uint64_t *r = res + off;
    return garner(r[i], r[n + i], r[2 * n + i]);
  }

  // Eight consecutive positions from i0 (a multiple of 8): 16-byte loads.
  __device__ __forceinline__ void eight(uint64_t off, uint64_t i0, uint64_t nproc, V3 (&v)[8]) const {
    if (i0 + 8 <= nproc) {
      uint64_t r[3][8];
#pragma unroll
      for (int j = 0; j < 3; ++j) {
        const ulonglong2 *src = reinterpret_cast<const ulonglong2 *>(res + off + j * n + i0);
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          const ulonglong2 w = load2(src + q);
          r[j][2 * q] = w.x;
          r[j][2 * q + 1] = w.y;
        }
      }
#pragma unroll
      for (int k8 = 0; k8 < 8; ++k8) v[k8] = garner(r[0][k8], r[1][k8], r[2][k8]);
    } else {
#pragma unroll
      for (int k8 = 0; k8 < 8; ++k8) v[k8] = (i0 + k8 < nproc) ? at(off, i0 + k8) : V3{0, 0, 0};
    }
  }

  __host__ __device__ __forceinline__ bool drop_top() const { return false; }

  // Residues lie in [0, 2p) (the inverse leaves them there).  Unscaled,
  // every one enters through a Shoup product that also applies N^-1 2^64.
  // Prescaled (the residues are the coefficient mod p_j), Garner's steps
  // need three Shoup products instead of six: y0 = c mod p0 is r0 folded,
  // t1 = (c - y0) / p0 mod p1 takes (r1 - y0) reduced to (0, 2 p1), and
  // t2 takes r2 - y0 + p2 in (0, 3 p2) as it is.  The host prescales only
  // where p0 < 2 p1, p0 < 2 p2 and 3 p2 < 2^64 (the reference's moduli).
  __device__ __forceinline__ V3 garner(uint64_t r0, uint64_t r1, uint64_t r2) const {
    const uint64_t p0 = k.pc[0].p, p1 = k.pc[1].p, p2 = k.pc[2].p;
    const uint32_t c0 = k.pc[0].c, c1 = k.pc[1].c, c2 = k.pc[2].c;
    check_below(r0, 2 * p0);  // inverse residues live in [0, 2p)
    check_below(r1, 2 * p1);
    check_below(r2, 2 * p2);
    uint64_t y0, t1, t2;
    if constexpr (PRESCALED) {
      y0 = fold_p(r0, p0);
      t1 = shoup_mul(fold_p(r1, p1) - fold_p(y0, p1) + p1, k.k1b.x, k.k1b.y, p1, c1);
      t2 = sub_mod_borrow(shoup_mul(r2 - fold_p(y0, p2) + p2, k.k2b.x, k.k2b.y, p2, c2),
                          shoup_mul(t1, k.k2c.x, k.k2c.y, p2, c2), p2);
    } else {
      y0 = shoup_mul(r0, k.k0.x, k.k0.y, p0, c0);
      t1 = sub_mod_borrow(shoup_mul(r1, k.k1a.x, k.k1a.y, p1, c1), shoup_mul(y0, k.k1b.x, k.k1b.y, p1, c1), p1);
      t2 = sub_mod_borrow(shoup_mul(r2, k.k2a.x, k.k2a.y, p2, c2), shoup_mul(y0, k.k2b.x, k.k2b.y, p2, c2), p2);
      t2 = sub_mod_borrow(t2, shoup_mul(t1, k.k2c.x, k.k2c.y, p2, c2), p2);
    }
    // V = y0 + p0 t1 + (p0 p1) t2 < p0 p1 p2 < 2^188
    V3 v{y0, 0, 0};
    add128_to(v, p0 * t1, __umul64hi(p0, t1));
    const uint64_t a0 = k.p01_lo * t2, a1 = __umul64hi(k.p01_lo, t2);
    const uint64_t b0 = k.p01_hi * t2, b1 = __umul64hi(k.p01_hi, t2);
    // (p0p1) t2 = a0 + (a1 + b0) 2^64 + b1 2^128
    const uint64_t m1 = a1 + b0;
    const uint64_t mc = m1 < a1;
    add128_to(v, a0, m1);
    v.w2 += b1 + mc;
    return v;
  }
};

using CrtProducer = CrtProducerT<false>;

// A tile's published aggregate: the launch's epoch in the high word, then
// p, g and the state bit 1 ("published").
__device__ __forceinline__ unsigned long long flag_word(uint32_t epoch, uint32_t g, uint32_t p) {
  return (static_cast<unsigned long long>(epoch) << 32) | (p << 3) | (g << 2) | 1u;
}

// One tile of NT * 8 output limbs per CTA (tile gt).  Batch (batch !=
// nullptr): tiles run product-major, tpp tiles per product; product k's
// residues are rebased by k * ws_stride and its output is
// batch[k].out[0, min(nout, n)).  The per-launch carry runs 256-thread
// CTAs (2048-limb tiles), four per SM at 64 registers, as does the
// persistent batch kernel.
//
// Each tile is written as if its carry-in were 0 and publishes its
// aggregate (g, p) once; carry_fix_kernel, launched next on the same
// stream, then adds the true carry-in.  No CTA waits on another, so the
// tiles stream at the memory and integer-pipe rate.
//
// carry_body is one CTA of NT threads on tile gt (NT * 8 positions);
// s_prev holds NT * 9 words and s_warp NT / 32 pairs of shared memory.
template <class Producer, int NT>
__device__ __forceinline__ void carry_body(const Producer &prod, uint64_t *__restrict__ out, uint64_t nproc,
                                           const ScanState &ss, const ProductDesc *batch, uint64_t tpp,
                                           uint64_t ws_stride, uint64_t n, uint64_t gt, uint64_t (*s_prev)[9],
                                           GP *s_warp) {
  constexpr int kCarryTile = NT * kCarryPer;
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  // Product k's residues are addressed through an explicit word offset.
  uint64_t tile = gt, off = 0;
  if (batch) {
    const uint64_t k = gt / tpp;
    tile = gt - k * tpp;
    off = k * ws_stride;
    out = batch[k].out;
    nproc = batch[k].nout < n ? batch[k].nout : n;
  }
  const uint64_t i0 = tile * kCarryTile + static_cast<uint64_t>(tid) * kCarryPer;

  V3 v[kCarryPer];
  prod.eight(off, i0, nproc, v);
  s_prev[tid][0] = v[5].w0; s_prev[tid][1] = v[5].w1; s_prev[tid][2] = v[5].w2;
  s_prev[tid][3] = v[6].w0; s_prev[tid][4] = v[6].w1; s_prev[tid][5] = v[6].w2;
  s_prev[tid][6] = v[7].w0; s_prev[tid][7] = v[7].w1; s_prev[tid][8] = v[7].w2;
  V3 pm3{0, 0, 0}, pm2{0, 0, 0}, pm1{0, 0, 0};
  if (tid == 0 && i0 >= 3) {
    pm3 = prod.at(off, i0 - 3);
    pm2 = prod.at(off, i0 - 2);
    pm1 = prod.at(off, i0 - 1);
  }
  __syncthreads();
  if (tid > 0) {
    pm3 = V3{s_prev[tid - 1][0], s_prev[tid - 1][1], s_prev[tid - 1][2]};
    pm2 = V3{s_prev[tid - 1][3], s_prev[tid - 1][4], s_prev[tid - 1][5]};
    pm1 = V3{s_prev[tid - 1][6], s_prev[tid - 1][7], s_prev[tid - 1][8]};
  }

  // W_i = v0_i + v1_(i-1) + v2_(i-2) = wl + wh 2^64 (wh <= 2); then
  // A_i = wl_i + wh_(i-1) = al + ah 2^64 (ah <= 1).
  auto wsum = [](uint64_t a, uint64_t b, uint64_t c, uint64_t &hi) {
    const uint64_t s = a + b;
    uint64_t h = s < a;
    const uint64_t t = s + c;
    h += t < s;
    hi = h;
    return t;
  };
  uint64_t whp;
  (void)wsum(pm1.w0, pm2.w1, pm3.w2, whp);  // W_(i0-1)
  uint64_t al[kCarryPer];
  uint32_t gbits = 0, pbits = 0;
#pragma unroll
  for (int k = 0; k < kCarryPer; ++k) {
    const V3 &c1 = (k >= 1) ? v[k - 1] : pm1;
    const V3 &c2 = (k >= 2) ? v[k - 2] : (k == 1 ? pm1 : pm2);
    uint64_t wh;
    const uint64_t wl = wsum(v[k].w0, c1.w1, c2.w2, wh);
    const uint64_t a = wl + whp;
    const uint32_t ah = a < wl;
    al[k] = a;
    gbits |= ah << k;
    pbits |= ((a == ~0ull) && !ah ? 1u : 0u) << k;
    whp = wh;
  }
  // Thread aggregate over its 8 positions (position 0 least significant).
  GP t{0, 1};
#pragma unroll
  for (int k = 0; k < kCarryPer; ++k) t = gp_compose(t, GP{(gbits >> k) & 1u, (pbits >> k) & 1u});

  // Inclusive warp scan, then across warps.
  GP inc = t;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const uint32_t og = __shfl_up_sync(0xffffffffu, inc.g, d);
    const uint32_t op = __shfl_up_sync(0xffffffffu, inc.p, d);
    if (lane >= d) inc = gp_compose(GP{og, op}, inc);
  }
  if (lane == 31) s_warp[wid] = inc;
  __syncthreads();
  GP wpre{0, 1};
  for (int w = 0; w < wid; ++w) wpre = gp_compose(wpre, s_warp[w]);
  GP excl;
  {
    const uint32_t og = __shfl_up_sync(0xffffffffu, inc.g, 1);
    const uint32_t op = __shfl_up_sync(0xffffffffu, inc.p, 1);
    excl = lane == 0 ? GP{0, 1} : GP{og, op};
  }
  excl = gp_compose(wpre, excl);  // runs over positions before this thread, within the tile
  if (tid == 0) {
    GP agg{0, 1};
    for (int w = 0; w < NT / 32; ++w) agg = gp_compose(agg, s_warp[w]);
    ss.flags[gt] = flag_word(ss.epoch, agg.g, agg.p);
  }
  uint32_t cin = excl.g;  // carry-in 0 at the tile's first position
  // Stage the tile's limbs in shared memory (reusing s_prev) and store them
  // with consecutive lanes on consecutive limbs: full 256-byte segments,
  // which also suits an output that lives in host memory.
  uint64_t *s_out = &s_prev[0][0];
  auto oswz = [](uint32_t w) { return w ^ ((w >> 3) & 7u); };
#pragma unroll
  for (int k = 0; k < kCarryPer; ++k) {
    const uint64_t z = al[k] + cin;
    cin = ((gbits >> k) & 1u) | (((pbits >> k) & 1u) & cin);
    s_out[oswz(static_cast<uint32_t>(tid * kCarryPer + k))] = z;
  }
  __syncthreads();
  const uint64_t tbase = tile * kCarryTile;
#pragma unroll
  for (int k = 0; k < kCarryPer; ++k) {
    const uint32_t w = static_cast<uint32_t>(tid + k * NT);
    if (tbase + w < nproc) out[tbase + w] = s_out[oswz(w)];
  }
}

// The second launch of a carry, one warp per tile.  Tile t's carry-in is
// the composition of the aggregates of tiles t - 1, t - 2, ... up to the
// nearest one that does not propagate (p = 0), or 0 before the product's
// first tile.  Every flag is final here (the tile launch ran to completion
// earlier on the stream), so nothing waits; a flag of another launch is an
// error.  A warp reads 128 predecessors per round, four per lane.  Batches
// (batch != nullptr) index tiles as the tile launch does.
//
// A carry-in of 1 changes only the tile's leading run of positions that
// propagate.  A position propagates exactly when its low word before
// carries, A, is 2^64 - 1: a position that generates a carry wraps to a low
// word of at most 1.  The tile launch wrote exactly A at every position of
// that run, so the run is the tile's leading limbs equal to 2^64 - 1.  They
// become 0 and the first limb after them gains 1; a tile that is one run
// becomes 0 and passes the carry on, as its p = 1 aggregate already says.
//
// fix_body is one warp on tile gt of TILE positions.
constexpr int kFixWarps = 8;

template <int TILE>
__device__ __forceinline__ void fix_body(uint64_t *out, uint64_t nproc, uint64_t tiles, const ScanState &ss,
                                         bool drop_top, const ProductDesc *batch, uint64_t tpp, uint64_t n,
                                         uint64_t gt) {
  constexpr int kCarryTile = TILE;
  const int lane = threadIdx.x & 31;
  if (gt >= tiles) return;
  uint64_t t = gt, first = 0;
  if (batch) {
    const uint64_t k = gt / tpp;
    t = gt - k * tpp;
    first = k * tpp;
    out = batch[k].out;
    nproc = batch[k].nout < n ? batch[k].nout : n;
  }
  const uint64_t ntiles = carry_tiles_dev<TILE>(nproc);  // tiles that hold positions
  if (t >= ntiles) return;
  const unsigned long long *flags = ss.flags;
  auto gp_of = [&](unsigned long long w, bool &bad) {
    if ((w >> 32) != ss.epoch || (w & 3u) != 1u) bad = true;
    return GP{static_cast<uint32_t>((w >> 2) & 1u), static_cast<uint32_t>((w >> 3) & 1u)};
  };
  GP acc{0, 1};
  bool bad = false;
  for (int64_t hi = static_cast<int64_t>(gt) - 1;; hi -= 128) {
    // Lane l composes tiles hi - 4l (most significant) down to hi - 4l - 3;
    // positions before the product's first tile emit carry 0.
    GP mine{0, 1};
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int64_t j = hi - 4 * lane - q;
      const GP f = j >= static_cast<int64_t>(first) ? gp_of(flags[j], bad) : GP{0, 0};
      mine = gp_compose(f, mine);
    }
    if (__any_sync(0xffffffffu, bad)) {
      if (lane == 0) atomicCAS(ss.err, kDevOk, kDevTicket);
      return;
    }
    // Lane 0 most significant, lane 31 least.
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const uint32_t og = __shfl_down_sync(0xffffffffu, mine.g, d);
      const uint32_t op = __shfl_down_sync(0xffffffffu, mine.p, d);
      if (lane + d < 32) mine = gp_compose(GP{og, op}, mine);
    }
    const GP win{__shfl_sync(0xffffffffu, mine.g, 0), __shfl_sync(0xffffffffu, mine.p, 0)};
    acc = gp_compose(win, acc);
    if (!acc.p) break;  // decided: a window that reaches past the first tile always ends here
  }
  const uint32_t cin = acc.g;
  const uint64_t base = t * kCarryTile;
  const uint64_t end = base + kCarryTile < nproc ? base + kCarryTile : nproc;
  if (t == ntiles - 1 && lane == 0 && !drop_top) {
    bool b2 = false;
    const GP own = gp_of(flags[gt], b2);
    if (own.g | (own.p & cin)) atomicCAS(ss.err, kDevOk, kDevCarryOverflow);
  }
  if (!cin) return;
  for (uint64_t i = base; i < end; i += 32) {
    const uint64_t k = i + lane;
    const bool valid = k < end;
    const uint64_t w = valid ? out[k] : 0;
    const unsigned stop = __ballot_sync(0xffffffffu, valid && w != ~0ull);
    if (!stop) {
      if (valid) out[k] = 0;
      continue;
    }
    const int f = __ffs(stop) - 1;
    if (lane < f) out[k] = 0;
    if (lane == f) out[k] = w + 1;
    break;
  }
}

}  // namespace carry
}  // namespace hg
