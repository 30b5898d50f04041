// hg_ntt_contig.cu -- the contiguous NTT pass and the middle of a product.
//
// The last T <= 12 forward stages of the reference's transform (ntt-forward,
// src/number-theoretic-transform.lisp:40-90) and the first T inverse stages
// (ntt-reverse, :93-143) act on contiguous blocks of 2^T residues.  One CTA
// owns one block.  Modes:
//   kFwd  the forward stages only (spectrum hook; bit-reversed output),
//   kInv  the inverse stages only (spectrum hook),
//   kMul  both operands' forward stages, the pointwise product
//         (multiply-pointwise!, src/ntt-multiply.lisp:88-99) and the
//         inverse stages: the block is read once per operand, written once,
//   kSqr  the same for one operand squared (src/ntt-multiply.lisp:136-144),
//   kMulSpec  operand 0's forward stages, the pointwise product with a
//         finished spectrum that every product of the launch shares, and the
//         inverse stages (the chunks of an unbalanced product).
// For transforms of at most 2^12 points this is the whole product's NTT work,
// and the kernel reads the limbs and reduces them itself.
//
// The block runs in rounds of up to four stages on 16 registers per thread,
// with one trip through shared memory between rounds; the stages of the low
// row group use compile-time twiddles, and multiplications by 1 are skipped.
// Transforms below 16 points run in ntt_tiny_kernel, one thread per prime.
#include "hg_ntt_rounds.cuh"

namespace hg {
namespace {

using namespace rounds;

constexpr int kFwd = 0, kInv = 1, kMul = 2, kSqr = 3, kMulSpec = 4;

// Register block of row group g in a 2^T block: groups of four row bits from
// the bottom; the top group may be partial and then shares its register
// block with the bits below it.
template <int T>
struct Groups {
  static constexpr int G = (T + 3) / 4;
  static constexpr int NBTOP = T - 4 * (G - 1);
  template <int g>
  __host__ __device__ static constexpr int A() { return g == G - 1 ? T - 4 : 4 * g; }
  template <int g>
  __host__ __device__ static constexpr int NB() { return g == G - 1 ? NBTOP : 4; }
  template <int g>
  __host__ __device__ static constexpr int JG() { return 4 - NB<g>(); }
};

template <int T, int g, bool INV, bool EDGE = false>
__device__ __forceinline__ void round_g(uint64_t (&v)[16], const ulonglong2 *tw, uint32_t xt, uint64_t p, uint32_t c) {
  using Gr = Groups<T>;
  constexpr int A = Gr::template A<g>();
  constexpr int NB = Gr::template NB<g>();
  constexpr int JG = Gr::template JG<g>();
  constexpr bool TZERO = (g == 0) && (A == 0) && (JG == 0);
  stages<NB, JG, A, 0, 4 * g, T, INV, TZERO, EDGE && TZERO>(v, tw, xt, p, c);
}

// Move the thread's registers from the layout of group g to that of group h
// through sm (two barriers: the buffer may still be read by the last round).
template <int T, int g, int h>
__device__ __forceinline__ void regroup(uint64_t (&v)[16], uint64_t *sm, uint32_t &xt, uint32_t tid) {
  using Gr = Groups<T>;
  constexpr int Ag = Gr::template A<g>(), Ah = Gr::template A<h>();
  if constexpr (Ag == Ah) return;
  __syncthreads();
  to_smem<Ag>(sm, v, xt);
  __syncthreads();
  xt = thread_base<Ah>(tid);
  from_smem<Ah>(v, sm, xt);
}

// All forward rounds, from the top group down to group 0.
template <int T>
__device__ __forceinline__ void forward_rounds(uint64_t (&v)[16], uint64_t *sm, const ulonglong2 *tw, uint32_t &xt,
                                               uint32_t tid, uint64_t p, uint32_t c) {
  constexpr int G = Groups<T>::G;
  if constexpr (G == 3) {
    round_g<T, 2, false>(v, tw, xt, p, c);
    regroup<T, 2, 1>(v, sm, xt, tid);
    round_g<T, 1, false>(v, tw, xt, p, c);
    regroup<T, 1, 0>(v, sm, xt, tid);
    round_g<T, 0, false>(v, tw, xt, p, c);
  } else if constexpr (G == 2) {
    round_g<T, 1, false>(v, tw, xt, p, c);
    regroup<T, 1, 0>(v, sm, xt, tid);
    round_g<T, 0, false>(v, tw, xt, p, c);
  } else {
    round_g<T, 0, false>(v, tw, xt, p, c);
  }
}

// All inverse rounds, from group 0 up to the top group.  CANON_IN: the
// residues come from the pointwise product, in [0, p).
template <int T, bool CANON_IN = false>
__device__ __forceinline__ void inverse_rounds(uint64_t (&v)[16], uint64_t *sm, const ulonglong2 *tw, uint32_t &xt,
                                               uint32_t tid, uint64_t p, uint32_t c) {
  constexpr int G = Groups<T>::G;
  round_g<T, 0, true, CANON_IN>(v, tw, xt, p, c);
  if constexpr (G >= 2) {
    regroup<T, 0, 1>(v, sm, xt, tid);
    round_g<T, 1, true>(v, tw, xt, p, c);
  }
  if constexpr (G == 3) {
    regroup<T, 1, 2>(v, sm, xt, tid);
    round_g<T, 2, true>(v, tw, xt, p, c);
  }
}

template <int A>
__device__ __forceinline__ void load_block(uint64_t (&v)[16], const uint64_t *data, const uint64_t *limbs, uint64_t nl,
                                           uint64_t base, uint32_t xt, uint64_t p) {
  if (limbs) {
#pragma unroll
    for (int i = 0; i < 16; ++i) {
      const uint64_t o = base + (xt | (static_cast<uint32_t>(i) << A));
      v[i] = o < nl ? reduce64(__ldg(limbs + o), p) : 0;
    }
  } else {
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = data[base + (xt | (static_cast<uint32_t>(i) << A))];
  }
}

__device__ __forceinline__ void zero16(uint64_t (&v)[16]) {
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = 0;
}

template <int A>
__device__ __forceinline__ void store_block(const uint64_t (&v)[16], uint64_t *data, uint64_t base, uint32_t xt) {
#pragma unroll
  for (int i = 0; i < 16; ++i) data[base + (xt | (static_cast<uint32_t>(i) << A))] = v[i];
}

// CTAs of 256 threads per SM: three (80 registers) where the rounds fit
// without spilling, two (128 registers) for the 9..11-bit blocks.
__host__ __device__ constexpr int contig_min_blocks(int T) { return (T >= 9 && T <= 11) ? 2 : 3; }

template <int T, int MODE>
__global__ void __launch_bounds__(kTileThreads, contig_min_blocks(T)) ntt_contig_kernel(const PassArgs P) {
  using Gr = Groups<T>;
  constexpr int ATOP = Gr::template A<Gr::G - 1>();
  constexpr int A0 = Gr::template A<0>();
  constexpr int LT = T - 4;                  // log2 threads per block
  constexpr int NT = kTileThreads;
  constexpr int BPC = 1 << (kTileBits - T);  // blocks per CTA: every CTA has 256 threads
  extern __shared__ uint64_t smem[];
  const uint32_t tid = threadIdx.x;
  const uint32_t lt = tid & ((1u << LT) - 1u);  // thread within its block
  const uint32_t lb = tid >> LT;                // block within the CTA
  const int prime = P.prime_lo + static_cast<int>(blockIdx.y);
  const uint64_t nblk = P.nprod * P.tiles;      // blocks of this prime
  const uint64_t gb = static_cast<uint64_t>(blockIdx.x) * BPC + lb;
  const bool valid = gb < nblk;                 // idle block slots still take part in barriers
  const uint64_t prod = valid ? gb / P.tiles : 0;
  const uint64_t tile = valid ? gb % P.tiles : 0;
  const uint64_t p = P.pc[prime].p;
  const uint32_t c = P.pc[prime].c;
  const NttTables tb = P.tb[prime];
  const uint64_t poff = prod * P.ws_stride + static_cast<uint64_t>(prime - P.prime_lo) * P.prime_stride;
  const uint64_t base = tile << T;

  constexpr bool TWO = (MODE == kMul);
  uint64_t *smA = smem + (lb << T);
  uint64_t *smB = smem + ((BPC + lb) << T);
  // The (twiddle, companion) pairs of the 2^T-point sub-transform, read from
  // the swizzled device tables (small, and shared by every CTA: they stay in
  // L1), forward first, inverse after the pointwise product.
  const ulonglong2 *tw = swz_table(tb, T, MODE == kInv);
  uint64_t nl0 = 0, nl1 = 0;
  const uint64_t *limbs0 = pass_limbs(P, prod, 0, nl0);
  const uint64_t *limbs1 = TWO ? pass_limbs(P, prod, 1, nl1) : nullptr;

  uint64_t v[16];
  uint32_t xt;
  if constexpr (MODE == kInv) {
    xt = thread_base<A0>(lt);
    if (valid) load_block<A0>(v, P.data[0] + poff, nullptr, 0, base, xt, p);
    else zero16(v);
    inverse_rounds<T>(v, smA, tw, xt, lt, p, c);
    if (valid) store_block<ATOP>(v, P.data[0] + poff, base, xt);
    return;
  } else if constexpr (MODE == kFwd) {
    xt = thread_base<ATOP>(lt);
    if (valid) load_block<ATOP>(v, P.data[0] + poff, limbs0, nl0, base, xt, p);
    else zero16(v);
    forward_rounds<T>(v, smA, tw, xt, lt, p, c);
    if (valid) store_block<A0>(v, P.data[0] + poff, base, xt);
    return;
  } else if constexpr (MODE == kMulSpec) {
    xt = thread_base<ATOP>(lt);
    if (valid) load_block<ATOP>(v, P.data[0] + poff, limbs0, nl0, base, xt, p);
    else zero16(v);
    forward_rounds<T>(v, smA, tw, xt, lt, p, c);
    // The shared spectrum sits where kFwd stores it, without a product offset.
    if (valid) {
      const uint64_t *spec = P.data[1] + static_cast<uint64_t>(prime - P.prime_lo) * P.prime_stride + base;
#pragma unroll
      for (int i = 0; i < 16; ++i) v[i] = mont_mul(v[i], __ldg(spec + (xt | (static_cast<uint32_t>(i) << A0))), p, c);
    }
    inverse_rounds<T, true>(v, smA, swz_table(tb, T, true), xt, lt, p, c);
    if (valid) store_block<ATOP>(v, P.data[0] + poff, base, xt);
    return;
  } else {
    {
      // The operands' forward transforms share one copy of the round code (a
      // loop, not unrolled): operand 0's spectrum is parked in smA (each
      // thread rereads only its own words), operand 1 transforms through smB.
      constexpr int nop = TWO ? 2 : 1;
#pragma unroll 1
      for (int op = 0; op < nop; ++op) {
        xt = thread_base<ATOP>(lt);
        if (valid) load_block<ATOP>(v, P.data[op] + poff, op ? limbs1 : limbs0, op ? nl1 : nl0, base, xt, p);
        else zero16(v);
        forward_rounds<T>(v, op ? smB : smA, tw, xt, lt, p, c);
        if (TWO && op == 0) {
          __syncthreads();
          to_smem<A0>(smA, v, xt);
        }
      }
    }
    {
      if constexpr (MODE == kMul) {
        const uint32_t sx = swz(xt);
#pragma unroll
        for (int i = 0; i < 16; ++i) v[i] = mont_mul(smA[sx ^ swz(static_cast<uint32_t>(i) << A0)], v[i], p, c);
      } else {
#pragma unroll
        for (int i = 0; i < 16; ++i) v[i] = mont_mul(v[i], v[i], p, c);
      }
      // The product is x*y*2^-64; the reconstruction constants absorb 2^64.
      inverse_rounds<T, true>(v, smA, swz_table(tb, T, true), xt, lt, p, c);
      if (valid) store_block<ATOP>(v, P.data[0] + poff, base, xt);
    }
  }
}

// Transforms of 2, 4 or 8 points: the reference's loops, one thread per
// (product, prime).
__global__ void ntt_tiny_kernel(const PassArgs P, int mode) {
  const uint64_t prod = blockIdx.x;
  const int prime = P.prime_lo + static_cast<int>(blockIdx.y);
  const uint64_t p = P.pc[prime].p;
  const uint32_t c = P.pc[prime].c;
  const NttTables tb = P.tb[prime];
  const uint64_t poff = prod * P.ws_stride + static_cast<uint64_t>(prime - P.prime_lo) * P.prime_stride;
  const int L = P.logN;
  const int n = 1 << L;
  uint64_t a[2][8];
  const int nops = mode == kMul ? 2 : 1;
  for (int op = 0; op < nops; ++op) {
    uint64_t nl = 0;
    const uint64_t *limbs = pass_limbs(P, prod, op, nl);
    for (int i = 0; i < n; ++i)
      a[op][i] = limbs ? (static_cast<uint64_t>(i) < nl ? reduce64(limbs[i], p) : 0) : P.data[op][poff + i];
  }
  if (mode != kInv) {
    for (int op = 0; op < nops; ++op)
      for (int ls = L; ls >= 1; --ls) {  // DIF, subn = 2^ls
        const int half = 1 << (ls - 1);
        for (int j = 0; j < half; ++j) {
          const ulonglong2 w = tb.sub_fwd[static_cast<uint64_t>(j) << (kTileBits - ls)];
          for (int r = 0; r < n; r += 2 * half) {
            const uint64_t u = a[op][r + j], x = a[op][r + j + half];
            a[op][r + j] = add_mod(u, x, p);
            a[op][r + j + half] = shoup_mul(u - x + p, w.x, w.y, p, c);
          }
        }
      }
  }
  if (mode == kMul || mode == kSqr)
    for (int i = 0; i < n; ++i) a[0][i] = mont_mul(a[0][i], a[mode == kMul ? 1 : 0][i], p, c);
  if (mode != kFwd) {
    for (int ls = 1; ls <= L; ++ls) {  // DIT, subn = 2^ls
      const int half = 1 << (ls - 1);
      for (int j = 0; j < half; ++j) {
        const ulonglong2 w = tb.sub_inv[static_cast<uint64_t>(j) << (kTileBits - ls)];
        for (int r = 0; r < n; r += 2 * half) {
          const uint64_t u = a[0][r + j], t = shoup_mul(a[0][r + j + half], w.x, w.y, p, c);
          a[0][r + j] = add_mod(u, t, p);
          a[0][r + j + half] = sub_mod(u, t, p);
        }
      }
    }
  }
  for (int i = 0; i < n; ++i) P.data[0][poff + i] = a[0][i];
}

__global__ void scale_kernel(uint64_t *a, uint64_t n, uint64_t f, uint64_t p, uint32_t c) {
  const uint64_t stride = static_cast<uint64_t>(gridDim.x) * blockDim.x;
  for (uint64_t i = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += stride)
    a[i] = mont_mul(a[i], f, p, c);
}

template <int T, int MODE>
cudaError_t launch_tm(const PassArgs &a, uint64_t nblk, cudaStream_t st) {
  constexpr uint64_t bpc = uint64_t(1) << (kTileBits - T);
  constexpr size_t bytes = static_cast<size_t>(MODE == kMul ? 2 : 1) * (1u << kTileBits) * sizeof(uint64_t);
  const uint64_t gx = (nblk + bpc - 1) / bpc;
  if (gx == 0 || gx > 0x7fffffffull) return cudaErrorInvalidValue;
  const dim3 grid(static_cast<unsigned>(gx), static_cast<unsigned>(a.nprimes));
  // Raise the dynamic shared-memory limit once per instantiation (not on
  // every launch, so that launches can be captured in a CUDA graph).
  static bool raised = false;
  if (bytes > 48 * 1024 && !raised) {
    cudaError_t e = cudaFuncSetAttribute(ntt_contig_kernel<T, MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         static_cast<int>(bytes));
    if (e != cudaSuccess) return e;
    raised = true;
  }
  ntt_contig_kernel<T, MODE><<<grid, kTileThreads, bytes, st>>>(a);
  return cudaGetLastError();
}

template <int MODE>
cudaError_t launch_mode(const PassArgs &a, uint64_t nblk, cudaStream_t st) {
  switch (a.logT) {
    case 4: return launch_tm<4, MODE>(a, nblk, st);
    case 5: return launch_tm<5, MODE>(a, nblk, st);
    case 6: return launch_tm<6, MODE>(a, nblk, st);
    case 7: return launch_tm<7, MODE>(a, nblk, st);
    case 8: return launch_tm<8, MODE>(a, nblk, st);
    case 9: return launch_tm<9, MODE>(a, nblk, st);
    case 10: return launch_tm<10, MODE>(a, nblk, st);
    case 11: return launch_tm<11, MODE>(a, nblk, st);
    case 12: return launch_tm<12, MODE>(a, nblk, st);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace

cudaError_t launch_ntt_contig(const PassArgs &a, int mode, cudaStream_t st) {
  const uint64_t nblk = a.tiles * a.nprod;  // blocks per prime
  if (nblk == 0 || a.logS != 0 || a.logR != a.logT || a.nprimes < 1 || a.nprimes > kPrimes)
    return cudaErrorInvalidValue;
  if (a.logT < 4) {
    if (mode == kMulSpec || a.logT < 1 || a.logT != a.logN || a.tiles != 1 || a.nprod > 0x7fffffffull) return cudaErrorInvalidValue;
    ntt_tiny_kernel<<<dim3(static_cast<unsigned>(a.nprod), static_cast<unsigned>(a.nprimes)), 1, 0, st>>>(a, mode);
    return cudaGetLastError();
  }
  switch (mode) {
    case kFwd: return launch_mode<kFwd>(a, nblk, st);
    case kInv: return launch_mode<kInv>(a, nblk, st);
    case kMul: return launch_mode<kMul>(a, nblk, st);
    case kSqr: return launch_mode<kSqr>(a, nblk, st);
    case kMulSpec: return launch_mode<kMulSpec>(a, nblk, st);
    default: return cudaErrorInvalidValue;
  }
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
