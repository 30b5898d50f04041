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
//
// Passes over residues (every pass but the first forward one, which reads and
// reduces the limbs) stage the tile through shared memory with TMA instead:
// one bulk tensor copy brings the tile's R rows of C residues in (and the
// same box of the pass's inter-pass twiddle table beside it), threads read
// their 16 residues with constant shared-memory offsets, and after the
// stages one bulk copy writes the tile back.  No thread computes a global
// address or issues a global load or store for the residues.
#include <algorithm>
#include <cudaTypedefs.h>
#include <mutex>

#include "hg_ntt_bodies.cuh"
#include "hg_tma.cuh"

namespace hg {
namespace {

using namespace rounds;
using namespace bodies;

// Four CTAs of 256 threads per SM (64 registers, a few spilled words): on
// the 2^25-point passes faster than three (80 registers), two (128) or five
// (48).
template <int LOGR, bool INV>
__global__ void __launch_bounds__(kTileThreads, 4) ntt_strided_kernel(const PassArgs P) {
  __shared__ ulonglong2 tw[1 << (LOGR - 1)];
  __shared__ uint64_t sm[LOGR > 4 ? (1 << kTileBits) : 1];
  strided_ldg_body<LOGR, INV>(P, blockIdx.x, tw, sm);
}

// Tensor maps of one TMA-staged pass: the box each CTA loads (residues, or
// the limbs of a first forward pass) and stores, per operand, and the box of
// the inter-pass twiddle table.
struct TmaMaps {
  CUtensorMap in[2];
  CUtensorMap out[2];
  CUtensorMap tw;
};

// A first forward pass's limbs per operand: the complete rows of S limbs the
// load map covers, the limbs of the partial row after them, and (bit op of
// ztop) whether every limb lies in the lower half of the block.
struct TmaLimbs {
  const uint64_t *limbs[2];
  uint64_t full_rows[2];
  uint64_t tail[2];
  uint32_t ztop;
};

// A strided pass with the tile staged by TMA.  Shared memory: the tile
// [R][C] (row-major, exactly the tile position x = r C + c), then, with
// TABLE, the same box of the inter-pass twiddle table.  Three CTAs of 256
// threads per SM (66 KB of shared memory each) with the table, four
// without; 64 registers (the table variants do not spill; measured 0.3%
// faster than with 80).
//
// LIMBS (forward only): the pass reads the operand's limbs, viewed as rows
// of S limbs (a 2-D map over the rows that are complete; the copy fills the
// rows past them with zeros) and patches the partial row past the last
// complete one with plain loads before reducing every limb modulo p.  When
// the upper half of the block lies past the limbs (P.ztop bit op), the first
// stage skips its zero inputs.
template <int LOGR, bool INV, bool TABLE, bool LIMBS>
__global__ void __launch_bounds__(kTileThreads, 4)
    ntt_strided_tma_kernel(const __grid_constant__ TmaMaps maps, const PassArgs P, const TmaLimbs L) {
  constexpr int T = kTileBits;
  constexpr int LOGTC = T - LOGR;
  constexpr int ROWOFF = LOGTC;
  constexpr int A0 = ROWOFF;
  constexpr int A1 = T - 4;
  constexpr int G = (LOGR + 3) / 4;
  constexpr int NB1 = LOGR - 4;
  constexpr uint32_t kTileBytes = (1u << T) * sizeof(uint64_t);
  static_assert(LOGR >= 4 && LOGR <= 8, "strided passes have 4..8 row bits");
  static_assert(!LIMBS || !INV, "only a forward pass reads limbs");
  extern __shared__ __align__(128) uint64_t tile[];  // [1 << T] residues, then [1 << T] twiddles
  __shared__ ulonglong2 tw[1 << (LOGR - 1)];
  __shared__ __align__(8) uint64_t bar;

  const uint32_t tid = threadIdx.x;
  uint64_t bid = blockIdx.x;
  const int prime = P.prime_lo + static_cast<int>(bid % P.nprimes);
  bid /= P.nprimes;
  const int op = static_cast<int>(bid % P.nops);
  bid /= P.nops;
  const uint64_t prod = bid / P.tiles;
  const uint64_t t = P.tile_lo + bid % P.tiles;
  const uint64_t p = P.pc[prime].p;
  const uint32_t c = P.pc[prime].c;
  const NttTables tb = P.tb[prime];
  const int logS = P.logS;
  const uint64_t ncg = 1ull << (logS - LOGTC);
  const int blk = static_cast<int>(t / ncg);
  const int s0 = static_cast<int>((t % ncg) << LOGTC);
  uint64_t *twt = tile + (1u << T);

  if (tid == 0) {
    tma::mbar_init(&bar, 1);
    tma::fence_barrier_init();
  }
  __syncthreads();
  if (tid == 0) {
    tma::mbar_arrive_expect_tx(&bar, TABLE ? 2 * kTileBytes : kTileBytes);
    if constexpr (LIMBS)
      tma::load_2d(tile, &maps.in[op], &bar, s0, blk << LOGR);
    else
      tma::load_5d(tile, &maps.in[op], &bar, s0, 0, blk, prime - P.prime_lo, static_cast<int>(prod));
    if (TABLE) tma::load_3d(twt, &maps.tw, &bar, s0, 0, prime);
  }
  load_sub_twiddles(tw, INV ? tb.sub_inv : tb.sub_fwd, LOGR, tid, kTileThreads);
  const bool landed = tma::mbar_wait_bounded(&bar, 0);
  if (!__syncthreads_and(landed)) {  // also orders the sub-twiddle table
    if (tid == 0) latch_error(P.err, kDevCopyTimeout);
    return;
  }

  // The inter-pass twiddles of the thread's 16 rows r = rhi * 16 + i of one
  // column (layout A0): from the table's box, or as a geometric sequence.
  auto inter_pass = [&](uint64_t (&v)[16], uint32_t xt, const uint64_t *hi, const uint64_t *lo) {
    if constexpr (TABLE) {
#pragma unroll
      for (int i = 0; i < 16; ++i) v[i] = mont_mul(v[i], twt[xt | (static_cast<uint32_t>(i) << A0)], p, c);
    } else {
      const uint64_t s = static_cast<uint64_t>(s0) + (xt & ((1u << LOGTC) - 1u));
      const uint32_t rhi = (xt >> (ROWOFF + 4)) & ((1u << (LOGR - 4)) - 1u);
      const int logM = LOGR + logS;
      uint32_t rrev = 0;
      if constexpr (LOGR > 4) rrev = bitrev(rhi, LOGR - 4);
      const uint64_t beta = table_twiddle(s * rrev, logM, hi, lo, p, c);
      const uint64_t gamma = table_twiddle(s << (LOGR - 4), logM, hi, lo, p, c);
      geometric_twiddle(v, beta, gamma, p, c);
    }
  };

  uint64_t v[16];
  uint32_t xt;
  if (!INV) {
    constexpr int AL = (G == 2) ? A1 : A0;
    xt = thread_base<AL>(tid);
    if constexpr (LIMBS) {
      // Row tr (in the limbs' rows of S) is the partial one: limbs
      // [tr S, tr S + tail) exist past the complete rows the map covers.
      const uint64_t tr = op ? L.full_rows[1] : L.full_rows[0];
      const uint64_t tail = op ? L.tail[1] : L.tail[0];
      const uint64_t *lp = op ? L.limbs[1] : L.limbs[0];
      const uint64_t row0 = static_cast<uint64_t>(blk) << LOGR;
      const bool has_tail = tail != 0 && tr >= row0 && tr < row0 + (1u << LOGR);
      auto limb = [&](int i) {
        const uint32_t x = xt | (static_cast<uint32_t>(i) << AL);
        uint64_t w = tile[x];
        if (has_tail && row0 + (x >> ROWOFF) == tr && s0 + (x & ((1u << LOGTC) - 1u)) < tail)
          w = __ldg(lp + tr * (uint64_t(1) << logS) + s0 + (x & ((1u << LOGTC) - 1u)));
        return reduce64(w, p);
      };
      if (G == 2 && ((L.ztop >> op) & 1)) {
        // Registers 8..15 hold the top row bit's upper half, past the limbs:
        // zeros that the first stage (ZTOP) never reads, so neither read nor
        // reduced here.
#pragma unroll
        for (int i = 0; i < 8; ++i) v[i] = limb(i);
        if constexpr (G == 2) stages<NB1, 4 - NB1, A1, ROWOFF, 4, LOGR, false, false, false, true>(v, tw, xt, p, c);
      } else {
#pragma unroll
        for (int i = 0; i < 16; ++i) v[i] = limb(i);
        if constexpr (G == 2) stages<NB1, 4 - NB1, A1, ROWOFF, 4, LOGR, false, false>(v, tw, xt, p, c);
      }
    } else {
#pragma unroll
      for (int i = 0; i < 16; ++i) {
        v[i] = tile[xt | (static_cast<uint32_t>(i) << AL)];
        check_below(v[i], p);  // forward input: canonical residues
      }
    }
    if constexpr (G == 2) {
      if constexpr (!LIMBS) stages<NB1, 4 - NB1, A1, ROWOFF, 4, LOGR, false, false>(v, tw, xt, p, c);
      __syncthreads();  // every thread has its values out of the tile
      to_smem<A1>(tile, v, xt);
      __syncthreads();
      xt = thread_base<A0>(tid);
      from_smem<A0>(v, tile, xt);
    }
    stages<4, 0, A0, ROWOFF, 0, LOGR, false, true, true>(v, tw, xt, p, c);
    inter_pass(v, xt, tb.hi_fwd, tb.lo_fwd);
    __syncthreads();
#pragma unroll
    for (int i = 0; i < 16; ++i) {
      check_below(v[i], p);  // after the Montgomery inter-pass twiddle
      tile[xt | (static_cast<uint32_t>(i) << A0)] = v[i];
    }
  } else {
    xt = thread_base<A0>(tid);
#pragma unroll
    for (int i = 0; i < 16; ++i) {
      v[i] = tile[xt | (static_cast<uint32_t>(i) << A0)];
      check_below(v[i], 2 * p);  // inverse residues live in [0, 2p)
    }
    inter_pass(v, xt, tb.hi_inv, tb.lo_inv);
    stages<4, 0, A0, ROWOFF, 0, LOGR, true, true, true>(v, tw, xt, p, c);
    constexpr int AS = (G == 2) ? A1 : A0;
    if constexpr (G == 2) {
      __syncthreads();
      to_smem<A0>(tile, v, xt);
      __syncthreads();
      xt = thread_base<A1>(tid);
      from_smem<A1>(v, tile, xt);
      stages<NB1, 4 - NB1, A1, ROWOFF, 4, LOGR, true, false>(v, tw, xt, p, c);
    }
    __syncthreads();
#pragma unroll
    for (int i = 0; i < 16; ++i) {
      check_below(v[i], 2 * p);
      tile[xt | (static_cast<uint32_t>(i) << AS)] = v[i];
    }
  }
  tma::fence_async_smem();
  __syncthreads();
  if (tid == 0) {
    tma::store_5d(&maps.out[op], tile, s0, 0, blk, prime - P.prime_lo, static_cast<int>(prod));
    tma::store_wait_read();
  }
}

// The inter-pass twiddles w_M^(s * bitrev(r)) of one (M, R, direction) in
// Montgomery form, [prime][r][s]; with scale[j] != 0 (a Montgomery-form
// factor) every entry of prime j is multiplied by it.
__global__ void pass_twiddles_kernel(uint64_t *out, int logM, int logR, bool inverse, NttTables t0, NttTables t1,
                                     NttTables t2, PrimeConst c0, PrimeConst c1, PrimeConst c2, uint64_t s0,
                                     uint64_t s1, uint64_t s2) {
  const uint64_t M = uint64_t(1) << logM;
  const int j = static_cast<int>(blockIdx.y);
  const NttTables &t = j == 0 ? t0 : (j == 1 ? t1 : t2);
  const PrimeConst &pc = j == 0 ? c0 : (j == 1 ? c1 : c2);
  const uint64_t scale = j == 0 ? s0 : (j == 1 ? s1 : s2);
  const int logS = logM - logR;
  for (uint64_t e = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; e < M;
       e += static_cast<uint64_t>(gridDim.x) * blockDim.x) {
    const uint64_t r = e >> logS, s = e & ((uint64_t(1) << logS) - 1);
    const uint64_t E = (s * bitrev(static_cast<uint32_t>(r), logR)) & (M - 1);
    uint64_t w = table_twiddle(E, logM, inverse ? t.hi_inv : t.hi_fwd, inverse ? t.lo_inv : t.lo_fwd, pc.p, pc.c);
    if (scale) w = mont_mul(w, scale, pc.p, pc.c);
    out[static_cast<uint64_t>(j) * M + e] = w;
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

// ---- tensor maps ----------------------------------------------------------

PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void *f = nullptr;
    cudaDriverEntryPointQueryResult q{};
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(f);
    else
      cudaGetLastError();
  });
  return fn;
}

cudaError_t encode(CUtensorMap *m, const void *base, int rank, const cuuint64_t *dims, const cuuint64_t *strides,
                   const cuuint32_t *box) {
  PFN_cuTensorMapEncodeTiled_v12000 fn = encode_fn();
  if (!fn) return cudaErrorNotSupported;
  const cuuint32_t estr[5] = {1, 1, 1, 1, 1};
  const CUresult r = fn(m, CU_TENSOR_MAP_DATA_TYPE_UINT64, static_cast<cuuint32_t>(rank), const_cast<void *>(base),
                        dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                        CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS ? cudaSuccess : cudaErrorInvalidValue;
}

// The residue arrays of one operand as a 5-D tensor: column s (S), row r (R),
// block (N / M), prime (nprimes, prime_stride apart), product (nprod,
// ws_stride apart); the box is one tile, C columns by R rows.
cudaError_t residue_map(CUtensorMap *m, const uint64_t *base, const PassArgs &a) {
  const uint64_t S = uint64_t(1) << a.logS, R = uint64_t(1) << a.logR, M = R * S;
  const uint64_t N = uint64_t(1) << a.logN;
  const cuuint64_t dims[5] = {S, R, N / M, static_cast<cuuint64_t>(a.nprimes), a.nprod};
  const uint64_t pstride = a.nprimes > 1 ? a.prime_stride : N;
  const uint64_t wstride = a.nprod > 1 ? a.ws_stride : N * static_cast<uint64_t>(a.nprimes);
  const cuuint64_t strides[4] = {S * 8, M * 8, pstride * 8, wstride * 8};
  const cuuint32_t box[5] = {static_cast<cuuint32_t>((uint64_t(1) << kTileBits) / R), static_cast<cuuint32_t>(R), 1,
                             1, 1};
  return encode(m, base, 5, dims, strides, box);
}

// The pass's inter-pass twiddle table [prime][r][s] (M words per prime, every
// prime of the scheme) as a 3-D tensor with the same box.
cudaError_t twiddle_map(CUtensorMap *m, const uint64_t *ptw, const PassArgs &a) {
  const uint64_t S = uint64_t(1) << a.logS, R = uint64_t(1) << a.logR;
  const cuuint64_t dims[3] = {S, R, static_cast<cuuint64_t>(kPrimes)};
  const cuuint64_t strides[2] = {S * 8, R * S * 8};
  const cuuint32_t box[3] = {static_cast<cuuint32_t>((uint64_t(1) << kTileBits) / R), static_cast<cuuint32_t>(R), 1};
  return encode(m, ptw, 3, dims, strides, box);
}

template <int LOGR, bool INV, bool TABLE, bool LIMBS>
cudaError_t launch_tma_v(const TmaMaps &m, const PassArgs &a, const TmaLimbs &l, unsigned grid, cudaStream_t st) {
  constexpr size_t bytes = (TABLE ? 2 : 1) * (size_t(1) << kTileBits) * sizeof(uint64_t);
  // Raise the dynamic shared-memory limit once per instantiation (not on
  // every launch, so that launches can be captured in a CUDA graph).
  static bool raised = false;
  if (bytes > 48 * 1024 && !raised) {
    cudaError_t e = cudaFuncSetAttribute(ntt_strided_tma_kernel<LOGR, INV, TABLE, LIMBS>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(bytes));
    if (e != cudaSuccess) return e;
    raised = true;
  }
  ntt_strided_tma_kernel<LOGR, INV, TABLE, LIMBS><<<grid, kTileThreads, bytes, st>>>(m, a, l);
  return cudaGetLastError();
}

template <int LOGR>
cudaError_t launch_tma_r(const TmaMaps &m, const PassArgs &a, const TmaLimbs &l, bool inverse, bool limbs,
                         unsigned grid, cudaStream_t st) {
  const bool table = a.ptw != nullptr;
  if (inverse)
    return table ? launch_tma_v<LOGR, true, true, false>(m, a, l, grid, st)
                 : launch_tma_v<LOGR, true, false, false>(m, a, l, grid, st);
  if (limbs)
    return table ? launch_tma_v<LOGR, false, true, true>(m, a, l, grid, st)
                 : launch_tma_v<LOGR, false, false, true>(m, a, l, grid, st);
  return table ? launch_tma_v<LOGR, false, true, false>(m, a, l, grid, st)
               : launch_tma_v<LOGR, false, false, false>(m, a, l, grid, st);
}

// The limbs of a single product's operand as rows of S limbs: a 2-D map
// over the complete rows (none when the operand is shorter than a row).
cudaError_t limb_map(CUtensorMap *m, const uint64_t *limbs, uint64_t nl, const PassArgs &a) {
  const uint64_t S = uint64_t(1) << a.logS, R = uint64_t(1) << a.logR;
  const cuuint64_t dims[2] = {S, nl / S};
  const cuuint64_t strides[1] = {S * 8};
  const cuuint32_t box[2] = {static_cast<cuuint32_t>((uint64_t(1) << kTileBits) / R), static_cast<cuuint32_t>(R)};
  return encode(m, limbs, 2, dims, strides, box);
}

bool reads_limbs(const PassArgs &a) {
  if (a.batch) return a.read_limbs != 0;
  return a.limbs[0] != nullptr || (a.nops > 1 && a.limbs[1] != nullptr);
}

// A first forward pass of one product (not a batch, not chunks) whose block
// is the whole transform reads its limbs through TMA: each operand's limbs
// fill at least one row of S, start on a 16-byte boundary and lie in the
// pass's single block.
bool tma_limbs_ok(const PassArgs &a) {
  if (a.batch || a.chunk || a.nprod != 1 || a.logS + a.logR != a.logN) return false;
  for (int op = 0; op < a.nops; ++op) {
    if (!a.limbs[op] || (reinterpret_cast<uintptr_t>(a.limbs[op]) & 15u)) return false;
    if ((a.nlimbs[op] >> a.logS) == 0 || a.nlimbs[op] > (uint64_t(1) << a.logN)) return false;
  }
  return true;
}

// TMA copies need 16-byte aligned arrays; the spectrum entry points take a
// caller's pointer, which may sit at any 8-byte offset.
bool tma_aligned(const PassArgs &a) {
  const auto al = [](const void *q) { return (reinterpret_cast<uintptr_t>(q) & 15u) == 0; };
  return al(a.data[0]) && (a.nops < 2 || al(a.data[1])) && (!a.ptw || al(a.ptw)) && (a.prime_stride & 1) == 0 &&
         (a.ws_stride & 1) == 0;
}

}  // namespace

#if HG_CHECKED
HG_CHECKED_READER(checked_fault_strided)
#endif

cudaError_t launch_pass_twiddles(uint64_t *out, int logM, int logR, bool inverse, const NttTables *tb,
                                 const PrimeConst *pc, int nprimes, cudaStream_t st, const uint64_t *scale) {
  if (nprimes < 1 || nprimes > kPrimes || logR < 1 || logR > 8 || logM <= logR || logM > kLogNmax)
    return cudaErrorInvalidValue;
  const uint64_t M = uint64_t(1) << logM;
  const unsigned gx = static_cast<unsigned>(std::min<uint64_t>((M + 255) / 256, 152 * 64));
  const int j1 = nprimes > 1 ? 1 : 0, j2 = nprimes > 2 ? 2 : 0;
  pass_twiddles_kernel<<<dim3(gx, static_cast<unsigned>(nprimes)), 256, 0, st>>>(
      out, logM, logR, inverse, tb[0], tb[j1], tb[j2], pc[0], pc[j1], pc[j2], scale ? scale[0] : 0,
      scale ? scale[j1] : 0, scale ? scale[j2] : 0);
  return cudaGetLastError();
}

cudaError_t launch_ntt_strided(const PassArgs &a, bool inverse, cudaStream_t st) {
  const uint64_t grid = a.tiles * a.nprod * static_cast<uint64_t>(a.nops) * static_cast<uint64_t>(a.nprimes);
  if (grid == 0 || grid > 0x7fffffffull || a.logT != kTileBits || a.logS < kTileBits - a.logR)
    return cudaErrorInvalidValue;
  const unsigned g = static_cast<unsigned>(grid);
  const bool limbs = reads_limbs(a);
  if (tma_aligned(a) && (!limbs || tma_limbs_ok(a))) {
    TmaMaps m;
    TmaLimbs l{};
    cudaError_t e = cudaSuccess;
    for (int op = 0; op < 2 && e == cudaSuccess; ++op) {
      const uint64_t *d = (op < a.nops) ? a.data[op] : a.data[0];
      e = residue_map(&m.out[op], d, a);
      if (e != cudaSuccess) break;
      if (!limbs) {
        m.in[op] = m.out[op];
        continue;
      }
      const int lo = op < a.nops ? op : 0;
      l.limbs[op] = a.limbs[lo];
      l.full_rows[op] = a.nlimbs[lo] >> a.logS;
      l.tail[op] = a.nlimbs[lo] & ((uint64_t(1) << a.logS) - 1);
      // Every limb lies in the lower half of the block: the first stage's
      // upper inputs are zero.
      if (a.nlimbs[lo] <= (uint64_t(1) << (a.logS + a.logR - 1))) l.ztop |= 1u << op;
      e = limb_map(&m.in[op], a.limbs[lo], a.nlimbs[lo], a);
    }
    if (e == cudaSuccess) e = a.ptw ? twiddle_map(&m.tw, a.ptw, a) : residue_map(&m.tw, a.data[0], a);
    if (e != cudaSuccess) return e;
    switch (a.logR) {
      case 4: return launch_tma_r<4>(m, a, l, inverse, limbs, g, st);
      case 5: return launch_tma_r<5>(m, a, l, inverse, limbs, g, st);
      case 6: return launch_tma_r<6>(m, a, l, inverse, limbs, g, st);
      case 7: return launch_tma_r<7>(m, a, l, inverse, limbs, g, st);
      case 8: return launch_tma_r<8>(m, a, l, inverse, limbs, g, st);
      default: return cudaErrorInvalidValue;
    }
  }
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
