// hg_crt.cu -- coefficient reconstruction and carry propagation.
//
// The reference rebuilds each convolution coefficient as a bignum
// sum_j f_j r_j mod M (f_j = (M/m_j) * ((M/m_j)^-1 mod m_j)) and adds it at
// limb i with a recursive carry ripple (src/ntt-multiply.lisp:10-51,
// 242-253).  The value is the unique residue mod M = m0 m1 m2, so any exact
// reconstruction gives the same limbs.  Here Garner's mixed radix
// (src/modular-arithmetic.lisp:235-267) produces each coefficient as three
// limbs V_i = y0 + p0 t1 + p0 p1 t2, the overlap-add sum_i V_i 2^(64 i) is
// formed per position, and carries are resolved by a carry-lookahead scan
// within a CTA by warp shuffles.  Across CTAs each tile is written with
// carry-in 0 and publishes its (generate, propagate) aggregate; a second
// launch composes every tile's carry-in from the aggregates below it and
// applies it.  No kernel here waits on another CTA.
//
// The same overlap-add + scan finishes the schoolboy and by-digit products
// (src/mpz-ram.lisp:367-431), with V_i = sum_j x_(i-j) y_j.
#include "hg_internal.h"

namespace hg {
namespace {

constexpr int kCarryThreads = 512;
constexpr int kCarryMinBlocks = 2;  // 64 registers
constexpr int kCarryPer = 8;
constexpr int kCarryTile = kCarryThreads * kCarryPer;

__device__ __forceinline__ uint64_t carry_tiles_dev(uint64_t n) { return (n + kCarryTile - 1) / kCarryTile; }

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

struct CrtProducer {
  const uint64_t *res;  // [3][N] natural-order residues from the unscaled inverse
  uint64_t n;           // N
  CrtConst k;

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
          const ulonglong2 w = __ldg(src + q);
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

  // Residues may be any 64-bit values congruent to the coefficient (the
  // inverse leaves [0, 2p)): every one enters through a Shoup product.
  __device__ __forceinline__ V3 garner(uint64_t r0, uint64_t r1, uint64_t r2) const {
    const uint64_t p0 = k.pc[0].p, p1 = k.pc[1].p, p2 = k.pc[2].p;
    const uint32_t c0 = k.pc[0].c, c1 = k.pc[1].c, c2 = k.pc[2].c;
    const uint64_t y0 = shoup_mul(r0, k.k0.x, k.k0.y, p0, c0);
    const uint64_t t1 =
        sub_mod_borrow(shoup_mul(r1, k.k1a.x, k.k1a.y, p1, c1), shoup_mul(y0, k.k1b.x, k.k1b.y, p1, c1), p1);
    uint64_t t2 =
        sub_mod_borrow(shoup_mul(r2, k.k2a.x, k.k2a.y, p2, c2), shoup_mul(y0, k.k2b.x, k.k2b.y, p2, c2), p2);
    t2 = sub_mod_borrow(t2, shoup_mul(t1, k.k2c.x, k.k2c.y, p2, c2), p2);
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

// The product of a long operand cut into chunks of `chunk` limbs with a
// short one: chunk k's cyclic product (2^logN > chunk + short - 1 points, no
// wrap) covers result positions [k chunk, k chunk + 2^logN), and chunk >=
// 2^(logN-1) makes at most two chunks meet at a position.  Their residues
// are added before the reconstruction: the sum of the two coefficients is
// below 2 * short * 2^128, far below p0 p1 p2, so Garner's value of the
// summed residues is the exact sum.  The inverse leaves residues in
// [0, 2p); each is folded to [0, p) before the sum, and Garner's Shoup
// products take the sum in [0, 2p) as it is.
struct ChunkProducer {
  CrtProducer crt;      // res = chunk 0's residues, n = 2^logN
  uint64_t stride;      // words between consecutive chunks' residues
  uint64_t chunk, nchunks;

  __host__ __device__ __forceinline__ bool drop_top() const { return false; }

  __device__ __forceinline__ static uint64_t sum2(uint64_t a, uint64_t b, uint64_t p) {
    return fold_p(a, p) + fold_p(b, p);
  }

  __device__ __forceinline__ uint64_t sum_res(const uint64_t *r0, const uint64_t *r1, int j) const {
    const uint64_t a = r0 ? r0[j * crt.n] : 0, b = r1 ? r1[j * crt.n] : 0;
    return sum2(a, b, crt.k.pc[j].p);
  }

  // Residue pointers of position i: the chunk that starts at or below i, and
  // the one before it when position i is inside its product.
  __device__ __forceinline__ void sources(uint64_t i, const uint64_t *&r0, const uint64_t *&r1) const {
    const uint64_t k = i / chunk, o = i - k * chunk;
    r0 = k < nchunks ? crt.res + k * stride + o : nullptr;
    r1 = (k >= 1 && k - 1 < nchunks && o + chunk < crt.n) ? crt.res + (k - 1) * stride + o + chunk : nullptr;
  }

  __device__ __forceinline__ V3 at(uint64_t, uint64_t i) const {
    const uint64_t *r0, *r1;
    sources(i, r0, r1);
    return crt.garner(sum_res(r0, r1, 0), sum_res(r0, r1, 1), sum_res(r0, r1, 2));
  }

  // Eight positions from i0 (a multiple of 8, as is chunk): one chunk pair.
  __device__ __forceinline__ void eight(uint64_t, uint64_t i0, uint64_t nproc, V3 (&v)[8]) const {
    if (i0 + 8 > nproc) {
#pragma unroll
      for (int k8 = 0; k8 < 8; ++k8) v[k8] = (i0 + k8 < nproc) ? at(0, i0 + k8) : V3{0, 0, 0};
      return;
    }
    const uint64_t *r0, *r1;
    sources(i0, r0, r1);
    uint64_t r[3][8];
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      const uint64_t p = crt.k.pc[j].p;
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        ulonglong2 a = make_ulonglong2(0, 0), b = make_ulonglong2(0, 0);
        if (r0) a = __ldg(reinterpret_cast<const ulonglong2 *>(r0 + j * crt.n) + q);
        if (r1) b = __ldg(reinterpret_cast<const ulonglong2 *>(r1 + j * crt.n) + q);
        r[j][2 * q] = sum2(a.x, b.x, p);
        r[j][2 * q + 1] = sum2(a.y, b.y, p);
      }
    }
#pragma unroll
    for (int k8 = 0; k8 < 8; ++k8) v[k8] = crt.garner(r[0][k8], r[1][k8], r[2][k8]);
  }
};

struct ConvProducer {
  const uint64_t *x;
  uint64_t nx;
  const uint64_t *y;  // null: multiply by dval
  uint64_t ny;
  uint64_t dval;

  __host__ __device__ __forceinline__ bool drop_top() const { return false; }

  __device__ __forceinline__ void eight(uint64_t, uint64_t i0, uint64_t nproc, V3 (&v)[8]) const {
#pragma unroll
    for (int k8 = 0; k8 < 8; ++k8) v[k8] = (i0 + k8 < nproc) ? at(0, i0 + k8) : V3{0, 0, 0};
  }

  __device__ __forceinline__ V3 at(uint64_t, uint64_t i) const {
    V3 v{0, 0, 0};
    if (!y) {
      if (i < nx) {
        const uint64_t a = x[i];
        v.w0 = a * dval;
        v.w1 = __umul64hi(a, dval);
      }
      return v;
    }
    const uint64_t jlo = i >= nx ? i - nx + 1 : 0;
    const uint64_t jhi = i < ny - 1 ? i : ny - 1;
    for (uint64_t j = jlo; j <= jhi; ++j) {
      const uint64_t a = x[i - j], b = y[j];
      add128_to(v, a * b, __umul64hi(a, b));
    }
    return v;
  }
};

// mpz-+ of two long magnitudes over the whole GPU (%add-storages/unsafe and
// %subtract-storages/unsafe, src/mpz-ram.lisp:184-274): position i holds
// x_i + y_i as (low, carry).  With opposite signs y is the smaller
// magnitude's complement over n = max(na, nb) limbs plus 1 at position 0,
// and the carry out of the top is dropped.  `top` is then the highest index
// where a and b differ (or -1), found before the scan; it picks the larger.
struct SumProducer {
  const uint64_t *a, *b;
  uint64_t na, nb, n;
  const long long *top;  // subtraction only

  __host__ __device__ __forceinline__ bool drop_top() const { return top != nullptr; }

  __device__ __forceinline__ bool a_larger() const {
    if (!top) return true;
    const long long t = *top;
    if (t < 0) return true;
    const uint64_t u = static_cast<uint64_t>(t);
    return (u < na ? a[u] : 0) >= (u < nb ? b[u] : 0);
  }

  __device__ __forceinline__ V3 value(uint64_t i, bool ax) const {
    if (i >= n) return V3{0, 0, 0};
    const uint64_t *X = ax ? a : b, *Y = ax ? b : a;
    const uint64_t nX = ax ? na : nb, nY = ax ? nb : na;
    const uint64_t x = i < nX ? X[i] : 0;
    uint64_t y = i < nY ? Y[i] : 0;
    if (top) y = ~y;
    uint64_t lo = x + y;
    uint64_t c = lo < x ? 1 : 0;
    if (top && i == 0) {
      lo += 1;
      c += lo == 0 ? 1 : 0;
    }
    return V3{lo, c, 0};
  }

  __device__ __forceinline__ void prefetch(uint64_t, uint64_t, uint64_t) const {}

  __device__ __forceinline__ V3 at(uint64_t, uint64_t i) const { return value(i, a_larger()); }

  __device__ __forceinline__ void eight(uint64_t, uint64_t i0, uint64_t nproc, V3 (&v)[8]) const {
    const bool ax = a_larger();
#pragma unroll
    for (int k8 = 0; k8 < 8; ++k8) v[k8] = (i0 + k8 < nproc) ? value(i0 + k8, ax) : V3{0, 0, 0};
  }
};

// *top = max index i < n with a_i != b_i (the caller set it to -1).
__global__ void top_diff_kernel(const uint64_t *a, uint64_t na, const uint64_t *b, uint64_t nb, uint64_t n,
                                long long *top) {
  long long best = -1;
  const uint64_t stride = static_cast<uint64_t>(gridDim.x) * blockDim.x;
  for (uint64_t i = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; i < n; i += stride)
    if ((i < na ? a[i] : 0) != (i < nb ? b[i] : 0)) best = static_cast<long long>(i);
#pragma unroll
  for (int d = 16; d > 0; d >>= 1) {
    const long long o = __shfl_down_sync(0xffffffffu, best, d);
    best = o > best ? o : best;
  }
  if ((threadIdx.x & 31) == 0 && best >= 0) atomicMax(top, best);
}

// result = (sign, size) of out[0, nproc): the highest nonzero limb, scanned
// from the top 2048 limbs at a time by one CTA.
__global__ void sum_finish_kernel(const uint64_t *out, uint64_t nproc, SumProducer prod, int64_t sa, int64_t sb,
                                  int64_t *result) {
  __shared__ long long s_top;
  if (threadIdx.x == 0) s_top = -1;
  __syncthreads();
  for (uint64_t hi = nproc; hi > 0;) {
    const uint64_t lo = hi > 2048 ? hi - 2048 : 0;
    for (uint64_t i = lo + threadIdx.x; i < hi; i += blockDim.x)
      if (out[i]) atomicMax(&s_top, static_cast<long long>(i));
    __syncthreads();
    const bool found = s_top >= 0;  // read by all before any update for the next chunk
    __syncthreads();
    if (found) break;
    hi = lo;
  }
  if (threadIdx.x == 0) {
    const int64_t size = s_top + 1;
    const int64_t sign = prod.a_larger() ? sa : sb;
    result[0] = size ? sign : 1;
    result[1] = size;
  }
}

// A tile's published aggregate: the launch's epoch in the high word, then
// p, g and the state bit 1 ("published").
__device__ __forceinline__ unsigned long long flag_word(uint32_t epoch, uint32_t g, uint32_t p) {
  return (static_cast<unsigned long long>(epoch) << 32) | (p << 3) | (g << 2) | 1u;
}

// One tile of 4096 output limbs per CTA, in ticket order.  Batch (batch !=
// nullptr): tickets run product-major, tpp tiles per product; product k's
// residues are rebased by k * ws_stride and its output is
// batch[k].out[0, min(nout, n)).  Tiles of 4096 limbs, two 512-thread CTAs
// per SM (64 registers).
//
// Each tile is written as if its carry-in were 0 and publishes its
// aggregate (g, p) once; carry_fix_kernel, launched next on the same
// stream, then adds the true carry-in.  No CTA waits on another, so the
// tiles stream at the memory and integer-pipe rate.
template <class Producer>
__global__ void __launch_bounds__(kCarryThreads, kCarryMinBlocks) carry_kernel(const Producer prod0, uint64_t *__restrict__ out,
                                                              uint64_t nproc, ScanState ss, const ProductDesc *batch,
                                                              uint64_t tpp, uint64_t ws_stride, uint64_t n) {
  __shared__ uint64_t s_prev[kCarryThreads][9];
  __shared__ GP s_warp[kCarryThreads / 32];
  __shared__ unsigned long long s_tile;
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;

  if (tid == 0) s_tile = atomicAdd(ss.ticket, 1ull) - ss.ticket_base;
  __syncthreads();
  const uint64_t gt = s_tile;
  if (gt >= gridDim.x) {  // ticket out of step with this launch: touch nothing
    if (tid == 0) atomicCAS(ss.err, kDevOk, kDevTicket);
    return;
  }
  // The producer stays an unmodified kernel parameter; product k's residues
  // are addressed through an explicit word offset.
  const Producer &prod = prod0;
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
    for (int w = 0; w < kCarryThreads / 32; ++w) agg = gp_compose(agg, s_warp[w]);
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
    const uint32_t w = static_cast<uint32_t>(tid + k * kCarryThreads);
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
constexpr int kFixWarps = 8;

__global__ void __launch_bounds__(kFixWarps * 32)
    carry_fix_kernel(uint64_t *out, uint64_t nproc, uint64_t tiles, ScanState ss, bool drop_top,
                     const ProductDesc *batch, uint64_t tpp, uint64_t n) {
  const int lane = threadIdx.x & 31;
  const uint64_t gt = static_cast<uint64_t>(blockIdx.x) * kFixWarps + (threadIdx.x >> 5);
  if (gt >= tiles) return;
  uint64_t t = gt, first = 0;
  if (batch) {
    const uint64_t k = gt / tpp;
    t = gt - k * tpp;
    first = k * tpp;
    out = batch[k].out;
    nproc = batch[k].nout < n ? batch[k].nout : n;
  }
  const uint64_t ntiles = carry_tiles_dev(nproc);  // tiles that hold positions
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

// The two launches of a carry over `tiles` tiles (a batch: tpp per product).
template <class Producer>
cudaError_t launch_carry(const Producer &prod, uint64_t *out, uint64_t nproc, uint64_t tiles, const ScanState &ss,
                         cudaStream_t st, const ProductDesc *batch = nullptr, uint64_t tpp = 0,
                         uint64_t ws_stride = 0, uint64_t n = 0) {
  if (tiles == 0) return cudaSuccess;
  if (tiles > 0x7fffffffull) return cudaErrorInvalidValue;
  carry_kernel<Producer><<<static_cast<unsigned>(tiles), kCarryThreads, 0, st>>>(prod, out, nproc, ss, batch, tpp,
                                                                                ws_stride, n);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  const uint64_t blocks = (tiles + kFixWarps - 1) / kFixWarps;
  carry_fix_kernel<<<static_cast<unsigned>(blocks), kFixWarps * 32, 0, st>>>(out, nproc, tiles, ss, prod.drop_top(),
                                                                             batch, tpp, n);
  return cudaGetLastError();
}

// out[N, nout) = 0 for product blockIdx.x.
__global__ void zero_tails_kernel(const ProductDesc *batch, uint64_t N) {
  const ProductDesc d = batch[blockIdx.x];
  for (uint64_t i = N + threadIdx.x; i < d.nout; i += blockDim.x) d.out[i] = 0;
}

}  // namespace

uint64_t carry_tiles(uint64_t n) { return (n + kCarryTile - 1) / kCarryTile; }

cudaError_t launch_crt_carry(const uint64_t *res, int logN, const CrtConst &cc, uint64_t *out, uint64_t nout,
                             const ScanState &ss, cudaStream_t st, uint64_t *tiles_used) {
  const uint64_t n = 1ull << logN;
  const uint64_t nproc = nout < n ? nout : n;
  const uint64_t tiles = carry_tiles(nproc);
  *tiles_used = tiles;
  if (tiles == 0) return cudaSuccess;
  return launch_carry(CrtProducer{res, n, cc}, out, nproc, tiles, ss, st);
}

cudaError_t launch_crt_carry_batch(const uint64_t *res, uint64_t ws_stride, int logN, const CrtConst &cc,
                                   const ProductDesc *batch, uint64_t nprod, const ScanState &ss, cudaStream_t st) {
  const uint64_t n = 1ull << logN;
  const uint64_t tpp = carry_tiles(n);
  const uint64_t tiles = tpp * nprod;
  if (tiles == 0) return cudaSuccess;
  if (tiles > 0x7fffffffull) return cudaErrorInvalidValue;
  return launch_carry(CrtProducer{res, n, cc}, nullptr, 0, tiles, ss, st, batch, tpp, ws_stride, n);
}

cudaError_t launch_crt_carry_chunks(const uint64_t *res, uint64_t ws_stride, int logN, uint64_t chunk,
                                    uint64_t nchunks, const CrtConst &cc, uint64_t *out, uint64_t nproc,
                                    const ScanState &ss, cudaStream_t st, uint64_t *tiles_used) {
  const uint64_t n = 1ull << logN;
  if (chunk % 8 || 2 * chunk < n || chunk > n || ws_stride % 2) return cudaErrorInvalidValue;
  const uint64_t tiles = carry_tiles(nproc);
  *tiles_used = tiles;
  if (tiles == 0) return cudaSuccess;
  if (tiles > 0x7fffffffull) return cudaErrorInvalidValue;
  return launch_carry(ChunkProducer{CrtProducer{res, n, cc}, ws_stride, chunk, nchunks}, out, nproc, tiles, ss,
                            st);
}

cudaError_t launch_large_sum(const uint64_t *a, uint64_t na, int64_t sa, const uint64_t *b, uint64_t nb, int64_t sb,
                             uint64_t *out, long long *top, int64_t *result, const ScanState &ss, cudaStream_t st) {
  const uint64_t n = na > nb ? na : nb;
  const bool sub = sa != sb;
  const uint64_t nproc = sub ? n : n + 1;
  const uint64_t tiles = carry_tiles(nproc);
  if (tiles == 0 || tiles > 0x7fffffffull) return cudaErrorInvalidValue;
  SumProducer prod{a, b, na, nb, n, sub ? top : nullptr};
  if (sub) {
    cudaError_t e = cudaMemsetAsync(top, 0xff, sizeof(long long), st);
    if (e != cudaSuccess) return e;
    const uint64_t blocks = (n + 255) / 256 < 152 * 8 ? (n + 255) / 256 : 152 * 8;
    top_diff_kernel<<<static_cast<unsigned>(blocks), 256, 0, st>>>(a, na, b, nb, n, top);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
  }
  cudaError_t e = launch_carry(prod, out, nproc, tiles, ss, st);
  if (e != cudaSuccess) return e;
  sum_finish_kernel<<<1, 256, 0, st>>>(out, nproc, prod, sa, sb, result);
  return cudaGetLastError();
}

cudaError_t launch_zero_tails(const ProductDesc *batch, uint64_t nprod, uint64_t N, cudaStream_t st) {
  if (nprod == 0) return cudaSuccess;
  if (nprod > 0x7fffffffull) return cudaErrorInvalidValue;
  zero_tails_kernel<<<static_cast<unsigned>(nprod), 256, 0, st>>>(batch, N);
  return cudaGetLastError();
}

cudaError_t launch_schoolboy_carry(const uint64_t *x, uint64_t nx, const uint64_t *y, uint64_t ny, uint64_t *out,
                                   uint64_t nout, const ScanState &ss, cudaStream_t st, uint64_t *tiles_used) {
  const uint64_t nproc = nout < nx + ny ? nout : nx + ny;
  const uint64_t tiles = carry_tiles(nproc);
  *tiles_used = tiles;
  if (tiles == 0) return cudaSuccess;
  return launch_carry(ConvProducer{x, nx, y, ny, 0}, out, nproc, tiles, ss, st);
}

cudaError_t launch_digit_carry(const uint64_t *x, uint64_t nx, uint64_t d, uint64_t *out, uint64_t nout,
                               const ScanState &ss, cudaStream_t st, uint64_t *tiles_used) {
  const uint64_t nproc = nout < nx + 1 ? nout : nx + 1;
  const uint64_t tiles = carry_tiles(nproc);
  *tiles_used = tiles;
  if (tiles == 0) return cudaSuccess;
  return launch_carry(ConvProducer{x, nx, nullptr, 1, d}, out, nproc, tiles, ss, st);
}

}  // namespace hg
