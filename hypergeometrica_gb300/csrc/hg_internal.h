// hg_internal.h -- structures shared by the kernels and the host driver.
#pragma once

#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

#include "hg_common.cuh"

namespace hg {

// Device twiddle tables of one prime.
struct NttTables {
  const ulonglong2 *sub_fwd;  // (w_4096^e, Shoup companion), e < 2048: sub-transform twiddles, any R <= 4096
  const ulonglong2 *sub_inv;  // (w_4096^-e, companion)
  const uint64_t *hi_fwd;     // w_{2^30}^(e * 2^15), e < 2^15, Montgomery form
  const uint64_t *lo_fwd;     // w_{2^30}^e,          e < 2^15, Montgomery form
  const uint64_t *hi_inv;
  const uint64_t *lo_inv;
  // Sub-transform tables of every block size R = 2^T, T = 1..12, in the
  // contiguous pass's padded order: entry tw_pos(e) of the table of T is
  // (w_R^e, companion), e < R / 2.  The forward table of T starts at entry
  // tw_base(T), its inverse kTwInverse entries later.
  const ulonglong2 *swz;
};

// Padded position of entry e of a contiguous pass's twiddle table: one gap
// entry after every 8, 64 and 512, so that 8 lanes reading 16-byte entries
// at a power-of-two stride of up to 2^8 entries hit 8 different bank quads.
// Additive over disjoint bits (tw_pos(a | b) = tw_pos(a) + tw_pos(b) when
// a & b = 0), so a thread's part and a register's compile-time part of an
// index combine by an addition the load instruction's offset absorbs.  The
// 12-bit middle kernel ran 1.2% faster than with an XOR swizzle of the same
// bank property (no gaps, but an XOR per load), and spilled less.
__host__ __device__ __forceinline__ constexpr uint32_t tw_pos(uint32_t e) {
  return e + (e >> 3) + (e >> 6) + (e >> 9);
}

// First entry of the padded table of block size 2^T (T = 1..13; 13 gives
// the entries of all forward tables).
__host__ __device__ __forceinline__ constexpr uint32_t tw_base(int T) {
  uint32_t b = 0;
  for (int t = 1; t < T; ++t) b += tw_pos((1u << (t - 1)) - 1u) + 1u;
  return b;
}

constexpr uint32_t kTwInverse = tw_base(kTileBits + 1);  // entries in all forward tables

// Shared-memory word of position x of a contiguous pass's block: bits 4..7
// XORed into bits 0..3, so that 16 lanes reading 8-byte words at a
// power-of-two stride of up to 128 positions hit 16 different bank pairs.
// Not padded: a gap word per 16 takes three middle-kernel CTAs past the
// 196 KB shared-memory carveout, which leaves the SM 28 KB of L1 for the
// twiddle tables instead of 60 KB (measured 2.3% slower).
__host__ __device__ __forceinline__ constexpr uint32_t data_swz(uint32_t x) { return x ^ ((x >> 4) & 15u); }

__host__ __device__ __forceinline__ const ulonglong2 *swz_table(const NttTables &t, int T, bool inverse) {
  return t.swz + (inverse ? kTwInverse : 0u) + tw_base(T);
}

// One product of a batch, as the kernels read it.  y == nullptr squares x.
struct ProductDesc {
  const uint64_t *x, *y;
  uint64_t nx, ny;
  uint64_t *out;
  uint64_t nout;
};

// One NTT pass over the residue arrays of nprod products x nops operands x
// nprimes primes.  The N residues of an array form blocks of M = R*S; the
// pass performs the reference's radix-2 stages subn = M .. 2S, i.e. an
// R-point transform down each of the S columns of every block, followed
// (forward) or preceded (inverse) by the twiddle w_M^(s * bitrev(r)).
// Product k's arrays start at data[op] + k * ws_stride; prime i's at a
// further (i - prime_lo) * prime_stride.
struct PassArgs {
  uint64_t *data[2];           // residues per operand
  const uint64_t *limbs[2];    // single product: this pass reads and reduces limbs
  uint64_t nlimbs[2];
  const ProductDesc *batch;    // batch: operands of product k are batch[k].x / .y
  uint64_t chunk;              // single product cut into chunks: product k reads
                               // operand 0's limbs [k * chunk, (k + 1) * chunk)
  int read_limbs;              // batch: this pass reads and reduces limbs
  int nops;                    // operands handled by this launch
  int logN;
  int logR;                    // log2 rows (transform points) of this pass
  int logS;                    // log2 stride; 0 = contiguous pass
  int logT;                    // log2 residues per tile
  int prime_lo, nprimes;
  uint64_t prime_stride;       // words between the arrays of consecutive primes
  uint64_t nprod;              // products in the launch
  uint64_t ws_stride;          // words between consecutive products' arrays
  uint64_t tiles;              // tiles per (product, operand, prime) in this launch
  uint64_t tile_lo;            // strided passes: the launch covers tiles [tile_lo, tile_lo + tiles)
  PrimeConst pc[kPrimes];
  NttTables tb[kPrimes];
  // Strided passes: the inter-pass twiddles w_M^(+-s * bitrev r) of this
  // (M, R, direction), Montgomery form, [prime][r][s] with M words per prime
  // (all primes of the scheme), or null to form them from tb.
  const uint64_t *ptw;
  int *err;                    // device error word (a tile copy that did not land)
};

// Limbs a pass reads for (product, operand), or nullptr when it reads residues.
__host__ __device__ __forceinline__ const uint64_t *pass_limbs(const PassArgs &P, uint64_t prod, int op,
                                                               uint64_t &nl) {
  if (P.batch) {
    if (!P.read_limbs) return nullptr;
    const ProductDesc &d = P.batch[prod];
    nl = op ? d.ny : d.nx;
    return op ? d.y : d.x;
  }
  nl = P.nlimbs[op];
  if (P.chunk && op == 0 && P.limbs[0]) {
    const uint64_t o = prod * P.chunk;
    nl = nl > o ? (nl - o < P.chunk ? nl - o : P.chunk) : 0;
    return P.limbs[0] + o;
  }
  return P.limbs[op];
}

// Constants of the Garner reconstruction for one transform length.
// Each constant is a (value, Shoup companion) pair.  The residues are
// N c 2^-64 mod p_j for the coefficient c (the inverse transform is
// unscaled, the pointwise product Montgomery), unless `prescaled`: then the
// product's last inverse pass read an inter-pass table multiplied by
// N^-1 2^64 mod p_j, and the residues are c mod p_j (in [0, 2p_j)).
struct CrtConst {
  PrimeConst pc[kPrimes];
  ulonglong2 k0;            // N^-1 2^64                                         mod p0
  ulonglong2 k1a, k1b;      // N^-1 2^64 p0^-1, p0^-1                            mod p1
  ulonglong2 k2a, k2b, k2c; // N^-1 2^64 (p0p1)^-1, (p0p1)^-1, p1^-1            mod p2
  uint64_t p01_lo, p01_hi;  // p0 * p1
  uint32_t prescaled;
  uint32_t pad;
};

// Carry launch state: tile tickets and the tiles' published aggregates.
struct ScanState {
  unsigned long long *ticket;  // monotonically increasing tile ticket
  unsigned long long ticket_base;
  unsigned long long *flags;   // one word per tile
  uint32_t epoch;              // distinguishes launches sharing `flags`
  int *err;                    // device error word
};

// Kernel launchers.
// Strided pass (hg_ntt_strided.cu): 4 <= logR <= 8, logT = 12.
cudaError_t launch_ntt_strided(const PassArgs &a, bool inverse, cudaStream_t st);
// Contiguous pass (hg_ntt_contig.cu), mode: 0 forward, 1 inverse, 2 product
// of operands 0 and 1, 3 square of operand 0, 4 product of operand 0 with a
// finished spectrum at data[1] that every product of the launch shares;
// logR == logT <= 12.
constexpr int kContigFwd = 0, kContigInv = 1, kContigMul = 2, kContigSqr = 3, kContigMulSpec = 4;
cudaError_t launch_ntt_contig(const PassArgs &a, int mode, cudaStream_t st);
cudaError_t launch_crt_carry(const uint64_t *res, int logN, const CrtConst &cc, uint64_t *out, uint64_t nout,
                             const ScanState &ss, cudaStream_t st, uint64_t *tiles_used);
// Reconstruction + carry for nprod products of transform length 2^logN whose
// residues start ws_stride words apart at res.
cudaError_t launch_crt_carry_batch(const uint64_t *res, uint64_t ws_stride, int logN, const CrtConst &cc,
                                   const ProductDesc *batch, uint64_t nprod, const ScanState &ss, cudaStream_t st);
// Reconstruction + carry of a product computed in chunks: chunk k's
// residues ([3][2^logN], unscaled inverse) start k * ws_stride words past
// res and hold the product of limbs [k * chunk, (k + 1) * chunk) of the long
// operand with the short one; position i of the result sums chunk i / chunk
// at i % chunk and the chunk before it at i % chunk + chunk.  Writes
// out[0, nproc).  Needs 2^(logN-1) <= chunk, chunk a multiple of 8.
cudaError_t launch_crt_carry_chunks(const uint64_t *res, uint64_t ws_stride, int logN, uint64_t chunk,
                                    uint64_t nchunks, const CrtConst &cc, uint64_t *out, uint64_t nproc,
                                    const ScanState &ss, cudaStream_t st, uint64_t *tiles_used);
// sa |a| + sb |b| into out[0, n + 1) (n = max(na, nb); out[0, n) when the
// signs differ) over the whole GPU, with the carry scan of the products;
// result = (sign, size).  top is one device word of scratch.
cudaError_t launch_large_sum(const uint64_t *a, uint64_t na, int64_t sa, const uint64_t *b, uint64_t nb, int64_t sb,
                             uint64_t *out, long long *top, int64_t *result, const ScanState &ss, cudaStream_t st);
// Zero out[N, nout) of every product (out[0, nout) when N == 0).
cudaError_t launch_zero_tails(const ProductDesc *batch, uint64_t nprod, uint64_t N, cudaStream_t st);
cudaError_t launch_schoolboy_carry(const uint64_t *x, uint64_t nx, const uint64_t *y, uint64_t ny, uint64_t *out,
                                   uint64_t nout, const ScanState &ss, cudaStream_t st, uint64_t *tiles_used);
cudaError_t launch_digit_carry(const uint64_t *x, uint64_t nx, uint64_t d, uint64_t *out, uint64_t nout,
                               const ScanState &ss, cudaStream_t st, uint64_t *tiles_used);
cudaError_t launch_scale(uint64_t *a, uint64_t n, uint64_t mont_factor, PrimeConst pc, cudaStream_t st);

// Fill out[j * M + r * S + s] = w_M^(+-s * bitrev_R(r)) (Montgomery form) for
// the primes j = 0 .. nprimes - 1 of tb, M = 2^logM, R = 2^logR, S = M / R.
cudaError_t launch_pass_twiddles(uint64_t *out, int logM, int logR, bool inverse, const NttTables *tb,
                                 const PrimeConst *pc, int nprimes, cudaStream_t st, const uint64_t *scale = nullptr);

// Tiles a carry-scan launch over n positions uses.
uint64_t carry_tiles(uint64_t n);

#if HG_CHECKED
// The fault word of each translation unit with kernels (checked builds),
// read and cleared: 0, a DevErr code, or -1 when the read failed.
int checked_fault_strided();
int checked_fault_contig();
int checked_fault_crt();
int checked_fault_persist();
int checked_fault_peak();
int checked_fault_sum();
int checked_fault_series();
#endif

// ---- one persistent launch for a batch (hg_persist.cu) --------------------
//
// A phase is one launch of the per-pass schedule; each of its items covers
// `per` consecutive units (CTAs of that launch).  Items of a phase with
// dep >= 0 start once phase dep has counted all its items done.
enum PersistKind : int {
  kPhaseZero = 0,     // out[n, nout) of products batch[0, count) (all of out when n == 0)
  kPhaseStrided = 1,  // sel = logR | inverse << 4
  kPhaseContig = 2,   // sel = T | mode << 4 (kContigMul or kContigSqr); item = by * gx + bx
  kPhaseTiny = 3,     // sel = mode; 256 (product, prime) pairs per item
  kPhaseCarry = 4,    // one carry tile of the persistent kernel per item
  kPhaseFix = 5,      // eight carry tiles per item, one per warp
};

struct PersistPhase {
  int kind, sel, dep, pad;
  uint64_t first, count, gx;
  uint64_t units, per;  // the launch's CTAs (warps for kPhaseFix, 256-pair groups for kPhaseTiny); per item
  PassArgs a;
  // reconstruction, carry and zeroing
  const uint64_t *res;
  uint64_t n, ws_stride, tpp, tiles;
  CrtConst cc;
  const ProductDesc *batch;
  ScanState ss;
};

constexpr int kPersistMaxPhases = 512;
constexpr size_t kPersistSmemBytes = 2 * (size_t(1) << kTileBits) * sizeof(uint64_t);

// The work counter, the abort word and one completion count per phase.
struct PersistState {
  unsigned long long next;
  unsigned abort, pad;
  unsigned done[1];
};
__host__ __device__ constexpr size_t persist_state_bytes(int nphases) {
  return sizeof(PersistState) + sizeof(unsigned) * static_cast<size_t>(nphases);
}

// CTAs of the persistent grid (SMs x resident CTAs per SM), 0 if unavailable.
int persist_grid();
// Carry tiles of the persistent kernel over n positions.
uint64_t persist_carry_tiles(uint64_t n);
// Clear the state and launch; phases and state are device memory.
cudaError_t launch_persist(const PersistPhase *phases, int nphases, uint64_t total, PersistState *state, int *err,
                           cudaStream_t st);

}  // namespace hg
