// hg_ntt.cu -- NTT pass kernels (forward DIF / inverse DIT) and the pointwise
// product.
//
// The reference transforms one prime at a time with radix-2 stages over the
// whole array (ntt-forward / ntt-reverse, src/number-theoretic-transform.lisp:
// 40-143): a j-outer, r-inner loop that strides across the array once per
// stage.  Here a transform of N = 2^L residues runs as a few passes; each
// pass owns a contiguous range of the reference's stages.  Stages
// subn = M .. 2S on blocks of M = R*S residues are equivalent to an R-point
// transform down each of the S columns of a block (bit-reversed output),
// with the row r of column s then multiplied by w_M^(s * bitrev(r)).  A CTA
// loads a 4096-residue tile (R rows x 4096/R columns, or one contiguous
// block of R = 4096), runs the R-point transform in shared memory in rounds
// of up to four radix-2 stages held in registers, applies the twiddle and
// writes back.  All residues stay fully reduced, so every pass writes the
// same values the reference's stages produce: after the forward passes the
// array equals ntt-forward's bit-reversed spectrum.
#include "hg_internal.h"

namespace hg {
namespace {

// Shared-memory word index of tile position x: xor-swizzle the low four
// bits with the next four so that 16 lanes reading 16 positions spaced by a
// power of two hit 16 different 8-byte bank pairs.
__device__ __forceinline__ uint32_t swz(uint32_t x) { return x ^ ((x >> 4) & 15u); }

__device__ __forceinline__ uint32_t bitrev(uint32_t r, int bits) { return __brev(r) >> (32 - bits); }

// Twiddle w_M^E (forward) or w_M^-E (inverse) in Montgomery form, M = 2^logM,
// E < M, from the two-level tables of w_{2^30}.
__device__ __forceinline__ uint64_t pass_twiddle(uint64_t E, int logM, const uint64_t *hi, const uint64_t *lo,
                                                 uint64_t p, uint32_t c) {
  const uint64_t e = E << (kLogNmax - logM);
  const uint64_t th = __ldg(hi + (e >> kTwLevelBits));
  const uint64_t tl = __ldg(lo + (e & ((1u << kTwLevelBits) - 1)));
  return mont_mul(th, tl, p, c);
}

// One round: up to four radix-2 stages on the tile in shared memory.  The
// thread holds 16 residues whose tile positions differ in the four bits
// [a, a+4); the round's NB row bits are register bits [JG, JG+NB).  Tile
// positions at or above 2^T (tiles of fewer than 16 residues) are phantoms.
template <int NB, int JG, bool INV>
__device__ __forceinline__ void tile_round(uint64_t *sm, const uint64_t *tw, int tid, int T, int a, int rowoff,
                                           int logR, int b_lo, uint64_t p, uint32_t c) {
  const uint32_t xt = (static_cast<uint32_t>(tid) & ((1u << a) - 1u)) | ((static_cast<uint32_t>(tid) >> a) << (a + 4));
  const uint32_t xlim = 1u << T;
  uint64_t v[16];
#pragma unroll
  for (int i = 0; i < 16; ++i) {
    const uint32_t x = xt | (static_cast<uint32_t>(i) << a);
    v[i] = (x < xlim) ? sm[swz(x)] : 0;
  }
  if (!INV) {
    // Decimation in frequency: row bits from high to low.
#pragma unroll
    for (int jj = NB - 1; jj >= 0; --jj) {
      const int j = JG + jj;
      const int b = b_lo + jj;
      const uint32_t lowmask = (1u << b) - 1u;
      const int sh = logR - 1 - b;
#pragma unroll
      for (int i = 0; i < 16; ++i) {
        if (i & (1 << j)) continue;
        const uint32_t x = xt | (static_cast<uint32_t>(i) << a);
        const uint32_t rl = (x >> rowoff) & lowmask;
        const uint64_t u = v[i], w = v[i | (1 << j)];
        v[i] = add_mod(u, w, p);
        const uint64_t d = u - w + p;  // in (0, 2p)
        v[i | (1 << j)] = rl ? mont_mul(d, tw[rl << sh], p, c) : (d >= p ? d - p : d);
      }
    }
  } else {
    // Decimation in time: row bits from low to high.
#pragma unroll
    for (int jj = 0; jj < NB; ++jj) {
      const int j = JG + jj;
      const int b = b_lo + jj;
      const uint32_t lowmask = (1u << b) - 1u;
      const int sh = logR - 1 - b;
#pragma unroll
      for (int i = 0; i < 16; ++i) {
        if (i & (1 << j)) continue;
        const uint32_t x = xt | (static_cast<uint32_t>(i) << a);
        const uint32_t rl = (x >> rowoff) & lowmask;
        const uint64_t u = v[i];
        const uint64_t t = rl ? mont_mul(v[i | (1 << j)], tw[rl << sh], p, c) : v[i | (1 << j)];
        v[i] = add_mod(u, t, p);
        v[i | (1 << j)] = sub_mod(u, t, p);
      }
    }
  }
#pragma unroll
  for (int i = 0; i < 16; ++i) {
    const uint32_t x = xt | (static_cast<uint32_t>(i) << a);
    if (x < xlim) sm[swz(x)] = v[i];
  }
}

template <bool INV>
__global__ void __launch_bounds__(kTileThreads) ntt_pass_kernel(const PassArgs A) {
  extern __shared__ uint64_t smem[];
  const int T = A.logT;
  const int nthr = T >= 4 ? (1 << (T - 4)) : 1;
  const int tid = threadIdx.x;

  uint64_t bid = blockIdx.x;
  const int prime = A.prime_lo + static_cast<int>(bid % A.nprimes);
  bid /= A.nprimes;
  const int op = static_cast<int>(bid % A.nops);
  bid /= A.nops;
  const uint64_t tile = bid;

  const uint64_t p = A.pc[prime].p;
  const uint32_t c = A.pc[prime].c;
  const NttTables tb = A.tb[prime];
  uint64_t *data = A.data[op] + static_cast<uint64_t>(prime - A.prime_lo) * A.prime_stride;

  const int logR = A.logR;
  const bool strided = A.logS > 0;
  const int logTC = T - logR;  // columns per tile (strided); 0 for a contiguous pass
  const int rowoff = strided ? logTC : 0;
  const int logM = logR + A.logS;
  uint64_t base, s0 = 0;
  if (strided) {
    const uint64_t ncg = 1ull << (A.logS - logTC);
    const uint64_t blk = tile / ncg, cg = tile % ncg;
    base = (blk << logM) + (cg << logTC);
    s0 = cg << logTC;
  } else {
    base = tile << T;
  }

  uint64_t *sm = smem;
  uint64_t *tw = smem + (1u << T);
  // Sub-transform twiddles w_R^e = w_4096^(e * 4096/R), e < R/2.
  {
    const uint64_t *src = INV ? tb.sub_inv : tb.sub_fwd;
    const int half = 1 << (logR - 1);
    for (int e = tid; e < half; e += nthr) tw[e] = __ldg(src + (static_cast<uint64_t>(e) << (kTileBits - logR)));
  }

  // Load the tile (first forward pass: reduce limbs; inverse: pre-twiddle).
  const uint32_t xlim = 1u << T;
  const uint64_t *limbs = A.limbs[op];
  const uint64_t nl = A.nlimbs[op];
#pragma unroll 4
  for (int k = 0; k < kPerThread; ++k) {
    const uint32_t x = static_cast<uint32_t>(tid + k * nthr);
    if (x >= xlim) break;
    const uint64_t off = strided ? base + ((static_cast<uint64_t>(x >> logTC)) << A.logS) + (x & ((1u << logTC) - 1u))
                                 : base + x;
    uint64_t v;
    if (limbs) {
      v = off < nl ? reduce64(__ldg(limbs + off), p) : 0;
    } else {
      v = data[off];
    }
    if (INV && strided) {
      const uint32_t r = (x >> logTC);
      const uint64_t s = s0 + (x & ((1u << logTC) - 1u));
      const uint64_t E = s * bitrev(r, logR);
      if (E) v = mont_mul(v, pass_twiddle(E, logM, tb.hi_inv, tb.lo_inv, p, c), p, c);
    }
    sm[swz(x)] = v;
  }
  __syncthreads();

  // Rounds of four stages: groups g cover row bits [4g, min(4g+4, logR)).
  const int G = (logR + 3) >> 2;
  for (int step = 0; step < G; ++step) {
    const int g = INV ? step : G - 1 - step;
    const int b_lo = 4 * g;
    const int nb = min(4, logR - b_lo);
    const int gx = rowoff + b_lo;  // tile bit of the group's lowest row bit
    if (nb == 4) {
      tile_round<4, 0, INV>(sm, tw, tid, T, gx, rowoff, logR, b_lo, p, c);
    } else if (T >= 4) {
      // Top group of rows: the register block [T-4, T) ends with it.
      const int a = T - 4;
      if (nb == 3) tile_round<3, 1, INV>(sm, tw, tid, T, a, rowoff, logR, b_lo, p, c);
      else if (nb == 2) tile_round<2, 2, INV>(sm, tw, tid, T, a, rowoff, logR, b_lo, p, c);
      else tile_round<1, 3, INV>(sm, tw, tid, T, a, rowoff, logR, b_lo, p, c);
    } else {
      // Tile of 2..8 residues: one thread, register bits [0, T) real.
      if (nb == 3) tile_round<3, 0, INV>(sm, tw, tid, T, 0, rowoff, logR, b_lo, p, c);
      else if (nb == 2) tile_round<2, 0, INV>(sm, tw, tid, T, 0, rowoff, logR, b_lo, p, c);
      else tile_round<1, 0, INV>(sm, tw, tid, T, 0, rowoff, logR, b_lo, p, c);
    }
    __syncthreads();
  }

  // Store (forward: post-twiddle).
#pragma unroll 4
  for (int k = 0; k < kPerThread; ++k) {
    const uint32_t x = static_cast<uint32_t>(tid + k * nthr);
    if (x >= xlim) break;
    const uint64_t off = strided ? base + ((static_cast<uint64_t>(x >> logTC)) << A.logS) + (x & ((1u << logTC) - 1u))
                                 : base + x;
    uint64_t v = sm[swz(x)];
    if (!INV && strided) {
      const uint32_t r = (x >> logTC);
      const uint64_t s = s0 + (x & ((1u << logTC) - 1u));
      const uint64_t E = s * bitrev(r, logR);
      if (E) v = mont_mul(v, pass_twiddle(E, logM, tb.hi_fwd, tb.lo_fwd, p, c), p, c);
    }
    data[off] = v;
  }
}

__global__ void pointwise_kernel(uint64_t *__restrict__ a, const uint64_t *__restrict__ b, int logN,
                                 PrimeConst p0, PrimeConst p1, PrimeConst p2, int square) {
  const uint64_t n = static_cast<uint64_t>(kPrimes) << logN;
  const uint64_t stride = static_cast<uint64_t>(gridDim.x) * blockDim.x;
  for (uint64_t i = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += stride) {
    const int pr = static_cast<int>(i >> logN);
    const PrimeConst pc = pr == 0 ? p0 : (pr == 1 ? p1 : p2);
    const uint64_t x = a[i];
    const uint64_t y = square ? x : b[i];
    // x * y * 2^-64: the 2^64 is folded into the reconstruction constants.
    a[i] = mont_mul(x, y, pc.p, pc.c);
  }
}

__global__ void scale_kernel(uint64_t *a, uint64_t n, uint64_t f, uint64_t p, uint32_t c) {
  const uint64_t stride = static_cast<uint64_t>(gridDim.x) * blockDim.x;
  for (uint64_t i = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += stride)
    a[i] = mont_mul(a[i], f, p, c);
}

}  // namespace

cudaError_t launch_ntt_pass(const PassArgs &a, bool inverse, cudaStream_t st) {
  const int T = a.logT;
  const int nthr = T >= 4 ? (1 << (T - 4)) : 1;
  const size_t smem = (sizeof(uint64_t) << T) + (sizeof(uint64_t) << (a.logR - 1));
  const uint64_t grid = a.tiles * static_cast<uint64_t>(a.nops) * static_cast<uint64_t>(a.nprimes);
  if (grid == 0 || grid > 0x7fffffffull) return cudaErrorInvalidValue;
  if (inverse)
    ntt_pass_kernel<true><<<static_cast<unsigned>(grid), nthr, smem, st>>>(a);
  else
    ntt_pass_kernel<false><<<static_cast<unsigned>(grid), nthr, smem, st>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_pointwise(uint64_t *a, const uint64_t *b, int logN, const PrimeConst *pc, bool square,
                             cudaStream_t st) {
  const uint64_t n = static_cast<uint64_t>(kPrimes) << logN;
  const int threads = 256;
  uint64_t blocks = (n + threads - 1) / threads;
  if (blocks > 152ull * 16) blocks = 152ull * 16;
  pointwise_kernel<<<static_cast<unsigned>(blocks), threads, 0, st>>>(a, b, logN, pc[0], pc[1], pc[2],
                                                                       square ? 1 : 0);
  return cudaGetLastError();
}

cudaError_t launch_scale(uint64_t *a, uint64_t n, uint64_t f, PrimeConst pc, cudaStream_t st) {
  const int threads = 256;
  uint64_t blocks = (n + threads - 1) / threads;
  if (blocks > 152ull * 16) blocks = 152ull * 16;
  if (blocks == 0) return cudaSuccess;
  scale_kernel<<<static_cast<unsigned>(blocks), threads, 0, st>>>(a, n, f, pc.p, pc.c);
  return cudaGetLastError();
}

}  // namespace hg
