// hg_ntt_strided.cu -- strided NTT passes.
//
// The reference's forward transform is a sequence of radix-2 DIF stages
// (ntt-forward, src/number-theoretic-transform.lisp:40-90); the inverse, DIT
// stages (ntt-reverse, :93-143).  A strided pass performs the stages
// subn = M .. 2S (M = R*S, R = 2^LOGR rows, 4 <= LOGR <= 8) on every block of
// M residues.  Those stages equal an R-point transform down each of the S
// columns, bit-reversed output, with row r of column s then multiplied by
// w_M^(s * bitrev(r)); the inverse pass mirrors it.  Every residue stays
// canonical, so the pass leaves in memory exactly what the reference's
// stages leave.
//
// A CTA of 256 threads owns a tile of 4096 residues: R rows x 4096/R
// consecutive columns (>= 16 columns, so every row segment is >= 128 bytes).
// Each thread loads 16 residues straight into registers (coalesced: lanes
// run along columns), runs the stages of the top row bits, exchanges the tile
// once through shared memory, runs the stages of the low four row bits, and
// applies the inter-pass twiddle to its 16 rows of one column as a geometric
// sequence beta * gamma^k before storing from registers.
#include <algorithm>

#include "hg_ntt_rounds.cuh"

namespace hg {
namespace {

using namespace rounds;

// Four CTAs of 256 threads per SM (64 registers, a few spilled words): on
// the 2^25-point passes faster than three (80 registers), two (128) or five
// (48).
template <int LOGR, bool INV>
__global__ void __launch_bounds__(kTileThreads, 4) ntt_strided_kernel(const PassArgs P) {
  constexpr int T = kTileBits;
  constexpr int LOGTC = T - LOGR;  // log2 columns per tile
  constexpr int ROWOFF = LOGTC;    // tile bit of row bit 0
  constexpr int A0 = ROWOFF;       // register block of the low row group
  constexpr int A1 = T - 4;        // register block of the top row group
  constexpr int G = (LOGR + 3) / 4;
  constexpr int NB1 = LOGR - 4;  // row bits of the top group (when G == 2)
  static_assert(LOGR >= 4 && LOGR <= 8, "strided passes have 4..8 row bits");
  __shared__ ulonglong2 tw[1 << (LOGR - 1)];
  __shared__ uint64_t sm[G == 2 ? (1 << T) : 1];

  const uint32_t tid = threadIdx.x;
  uint64_t bid = blockIdx.x;
  const int prime = P.prime_lo + static_cast<int>(bid % P.nprimes);
  bid /= P.nprimes;
  const int op = static_cast<int>(bid % P.nops);
  bid /= P.nops;
  const uint64_t prod = bid / P.tiles;
  const uint64_t tile = P.tile_lo + bid % P.tiles;

  const uint64_t p = P.pc[prime].p;
  const uint32_t c = P.pc[prime].c;
  const NttTables tb = P.tb[prime];
  uint64_t *data = P.data[op] + prod * P.ws_stride + static_cast<uint64_t>(prime - P.prime_lo) * P.prime_stride;
  const int logS = P.logS;
  const int logM = LOGR + logS;
  const uint64_t ncg = 1ull << (logS - LOGTC);
  const uint64_t blk = tile / ncg, cg = tile % ncg;
  const uint64_t base = (blk << logM) + (cg << LOGTC);
  const uint64_t s0 = cg << LOGTC;

  load_sub_twiddles(tw, INV ? tb.sub_inv : tb.sub_fwd, LOGR, tid, kTileThreads);

  // Global offset of the thread's register 0 in layout A, and the stride
  // between consecutive registers (register bits are row bits).
  auto offsets = [&](uint32_t xt, int a, uint64_t &off0, uint64_t &step) {
    off0 = base + (static_cast<uint64_t>(xt >> ROWOFF) << logS) + (xt & ((1u << LOGTC) - 1u));
    step = 1ull << (logS + (a - ROWOFF));
  };
  // The inter-pass twiddles of the thread's 16 rows r = rhi * 16 + i of one
  // column s (layout A0): from the pass table when there is one, else as the
  // geometric sequence beta * gamma^bitrev4(i) from the two-level tables.
  auto inter_pass = [&](uint64_t (&v)[16], uint32_t xt, const uint64_t *hi, const uint64_t *lo) {
    const uint64_t s = s0 + (xt & ((1u << LOGTC) - 1u));
    const uint32_t rhi = (xt >> (ROWOFF + 4)) & ((1u << (LOGR - 4)) - 1u);
    if (P.ptw) {
      const uint64_t *t = P.ptw + (static_cast<uint64_t>(prime) << logM) +
                          (static_cast<uint64_t>(rhi) << (4 + logS)) + s;
#pragma unroll
      for (int i = 0; i < 16; ++i) v[i] = mont_mul(v[i], __ldg(t + (static_cast<uint64_t>(i) << logS)), p, c);
      return;
    }
    uint32_t rrev = 0;
    if constexpr (LOGR > 4) rrev = bitrev(rhi, LOGR - 4);
    const uint64_t beta = table_twiddle(s * rrev, logM, hi, lo, p, c);
    const uint64_t gamma = table_twiddle(s << (LOGR - 4), logM, hi, lo, p, c);
    geometric_twiddle(v, beta, gamma, p, c);
  };

  uint64_t v[16];
  if (!INV) {
    constexpr int AL = (G == 2) ? A1 : A0;
    uint32_t xt = thread_base<AL>(tid);
    uint64_t off, step;
    offsets(xt, AL, off, step);
    uint64_t nl = 0;
    const uint64_t *limbs = pass_limbs(P, prod, op, nl);
    if (limbs) {
#pragma unroll
      for (int i = 0; i < 16; ++i) {
        const uint64_t o = off + i * step;
        v[i] = o < nl ? reduce64(__ldg(limbs + o), p) : 0;
      }
    } else {
#pragma unroll
      for (int i = 0; i < 16; ++i) v[i] = data[off + i * step];
    }
    __syncthreads();  // twiddle table ready
    if constexpr (G == 2) {
      stages<NB1, 4 - NB1, A1, ROWOFF, 4, LOGR, false, false>(v, tw, xt, p, c);
      to_smem<A1>(sm, v, xt);
      __syncthreads();
      xt = thread_base<A0>(tid);
      from_smem<A0>(v, sm, xt);
    }
    stages<4, 0, A0, ROWOFF, 0, LOGR, false, true, true>(v, tw, xt, p, c);  // then the inter-pass twiddle
    inter_pass(v, xt, tb.hi_fwd, tb.lo_fwd);
    offsets(xt, A0, off, step);
#pragma unroll
    for (int i = 0; i < 16; ++i) data[off + i * step] = v[i];
  } else {
    uint32_t xt = thread_base<A0>(tid);
    uint64_t off, step;
    offsets(xt, A0, off, step);
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = data[off + i * step];
    inter_pass(v, xt, tb.hi_inv, tb.lo_inv);
    __syncthreads();  // twiddle table ready
    stages<4, 0, A0, ROWOFF, 0, LOGR, true, true, true>(v, tw, xt, p, c);  // after the inter-pass twiddle
    if constexpr (G == 2) {
      to_smem<A0>(sm, v, xt);
      __syncthreads();
      xt = thread_base<A1>(tid);
      from_smem<A1>(v, sm, xt);
      stages<NB1, 4 - NB1, A1, ROWOFF, 4, LOGR, true, false>(v, tw, xt, p, c);
      offsets(xt, A1, off, step);
    }
#pragma unroll
    for (int i = 0; i < 16; ++i) data[off + i * step] = v[i];
  }
}

__global__ void pass_twiddles_kernel(uint64_t *out, int logM, int logR, bool inverse, NttTables t0, NttTables t1,
                                     NttTables t2, PrimeConst c0, PrimeConst c1, PrimeConst c2) {
  const uint64_t M = uint64_t(1) << logM;
  const int j = static_cast<int>(blockIdx.y);
  const NttTables &t = j == 0 ? t0 : (j == 1 ? t1 : t2);
  const PrimeConst &pc = j == 0 ? c0 : (j == 1 ? c1 : c2);
  const int logS = logM - logR;
  for (uint64_t e = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; e < M;
       e += static_cast<uint64_t>(gridDim.x) * blockDim.x) {
    const uint64_t r = e >> logS, s = e & ((uint64_t(1) << logS) - 1);
    const uint64_t E = (s * bitrev(static_cast<uint32_t>(r), logR)) & (M - 1);
    out[static_cast<uint64_t>(j) * M + e] =
        table_twiddle(E, logM, inverse ? t.hi_inv : t.hi_fwd, inverse ? t.lo_inv : t.lo_fwd, pc.p, pc.c);
  }
}

template <int LOGR>
cudaError_t launch_r(const PassArgs &a, bool inverse, unsigned grid, cudaStream_t st) {
  if (inverse)
    ntt_strided_kernel<LOGR, true><<<grid, kTileThreads, 0, st>>>(a);
  else
    ntt_strided_kernel<LOGR, false><<<grid, kTileThreads, 0, st>>>(a);
  return cudaGetLastError();
}

}  // namespace

cudaError_t launch_pass_twiddles(uint64_t *out, int logM, int logR, bool inverse, const NttTables *tb,
                                 const PrimeConst *pc, int nprimes, cudaStream_t st) {
  if (nprimes < 1 || nprimes > kPrimes || logR < 1 || logR > 8 || logM <= logR || logM > kLogNmax)
    return cudaErrorInvalidValue;
  const uint64_t M = uint64_t(1) << logM;
  const unsigned gx = static_cast<unsigned>(std::min<uint64_t>((M + 255) / 256, 152 * 64));
  pass_twiddles_kernel<<<dim3(gx, static_cast<unsigned>(nprimes)), 256, 0, st>>>(
      out, logM, logR, inverse, tb[0], tb[nprimes > 1 ? 1 : 0], tb[nprimes > 2 ? 2 : 0], pc[0],
      pc[nprimes > 1 ? 1 : 0], pc[nprimes > 2 ? 2 : 0]);
  return cudaGetLastError();
}

cudaError_t launch_ntt_strided(const PassArgs &a, bool inverse, cudaStream_t st) {
  const uint64_t grid = a.tiles * a.nprod * static_cast<uint64_t>(a.nops) * static_cast<uint64_t>(a.nprimes);
  if (grid == 0 || grid > 0x7fffffffull || a.logT != kTileBits || a.logS < kTileBits - a.logR)
    return cudaErrorInvalidValue;
  const unsigned g = static_cast<unsigned>(grid);
  switch (a.logR) {
    case 4: return launch_r<4>(a, inverse, g, st);
    case 5: return launch_r<5>(a, inverse, g, st);
    case 6: return launch_r<6>(a, inverse, g, st);
    case 7: return launch_r<7>(a, inverse, g, st);
    case 8: return launch_r<8>(a, inverse, g, st);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace hg
