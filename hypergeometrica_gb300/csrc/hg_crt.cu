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
#include "hg_carry.cuh"

namespace hg {
namespace {

using namespace carry;

// Tiles of 2048 limbs: four CTAs of 256 threads per SM (64 registers),
// 4.4% faster than two of 512 threads on 4096-limb tiles (fewer threads
// wait at each CTA barrier).
constexpr int kCarryThreads = 256;
constexpr int kCarryMinBlocks = 4;
constexpr int kCarryTile = kCarryThreads * kCarryPer;

// The product of a long operand cut into chunks of `chunk` limbs with a
// short one: chunk k's cyclic product (2^logN > chunk + short - 1 points, no
// wrap) covers result positions [k chunk, k chunk + 2^logN), and chunk >=
// 2^(logN-1) makes at most two chunks meet at a position.  Their residues
// are added before the reconstruction: the sum of the two coefficients is
// below 2 * short * 2^128, far below p0 p1 p2, so Garner's value of the
// summed residues is the exact sum.  The inverse leaves residues in
// [0, 2p); each is folded to [0, p) before the sum, and Garner's Shoup
// products take the sum in [0, 2p) as it is.
template <class Crt>
struct ChunkProducerT {
  Crt crt;              // res = chunk 0's residues, n = 2^logN
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

// One tile per CTA, in ticket order.
template <class Producer>
__global__ void __launch_bounds__(kCarryThreads, kCarryMinBlocks)
    carry_kernel(const Producer prod0, uint64_t *__restrict__ out, uint64_t nproc, ScanState ss,
                 const ProductDesc *batch, uint64_t tpp, uint64_t ws_stride, uint64_t n) {
  __shared__ uint64_t s_prev[kCarryThreads][9];
  __shared__ GP s_warp[kCarryThreads / 32];
  __shared__ unsigned long long s_tile;
  if (threadIdx.x == 0) s_tile = atomicAdd(ss.ticket, 1ull) - ss.ticket_base;
  __syncthreads();
  const uint64_t gt = s_tile;
  if (gt >= gridDim.x) {  // ticket out of step with this launch: touch nothing
    if (threadIdx.x == 0) atomicCAS(ss.err, kDevOk, kDevTicket);
    return;
  }
  carry_body<Producer, kCarryThreads>(prod0, out, nproc, ss, batch, tpp, ws_stride, n, gt, s_prev, s_warp);
}

__global__ void __launch_bounds__(kFixWarps * 32)
    carry_fix_kernel(uint64_t *out, uint64_t nproc, uint64_t tiles, ScanState ss, bool drop_top,
                     const ProductDesc *batch, uint64_t tpp, uint64_t n) {
  fix_body<kCarryTile>(out, nproc, tiles, ss, drop_top, batch, tpp, n,
                       static_cast<uint64_t>(blockIdx.x) * kFixWarps + (threadIdx.x >> 5));
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
  if (cc.prescaled) return launch_carry(carry::CrtProducerT<false, true>{res, n, cc}, out, nproc, tiles, ss, st);
  return launch_carry(CrtProducer{res, n, cc}, out, nproc, tiles, ss, st);
}

cudaError_t launch_crt_carry_batch(const uint64_t *res, uint64_t ws_stride, int logN, const CrtConst &cc,
                                   const ProductDesc *batch, uint64_t nprod, const ScanState &ss, cudaStream_t st) {
  const uint64_t n = 1ull << logN;
  const uint64_t tpp = carry_tiles(n);
  const uint64_t tiles = tpp * nprod;
  if (tiles == 0) return cudaSuccess;
  if (tiles > 0x7fffffffull) return cudaErrorInvalidValue;
  if (cc.prescaled)
    return launch_carry(carry::CrtProducerT<false, true>{res, n, cc}, nullptr, 0, tiles, ss, st, batch, tpp, ws_stride,
                        n);
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
  if (cc.prescaled)
    return launch_carry(ChunkProducerT<carry::CrtProducerT<false, true>>{{res, n, cc}, ws_stride, chunk, nchunks}, out,
                        nproc, tiles, ss, st);
  return launch_carry(ChunkProducerT<CrtProducer>{CrtProducer{res, n, cc}, ws_stride, chunk, nchunks}, out, nproc,
                      tiles, ss, st);
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

#if HG_CHECKED
HG_CHECKED_READER(checked_fault_crt)
#endif

}  // namespace hg
