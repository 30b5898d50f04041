// hg_ntt_rounds.cuh -- register rounds shared by the NTT kernels.
//
// A CTA owns a tile of 2^T residues (T <= 12).  Tile position x holds row r
// of column c: strided tiles keep the column in the low bits (x = r << ROWOFF
// | c), contiguous blocks have ROWOFF = 0.  In a round, each thread holds 16
// residues whose tile positions differ only in the four bits [A, A+4): the
// residue of register i sits at xt | (i << A), where xt deposits the thread
// index into the other bits.  Up to four radix-2 stages run on those
// registers; between rounds the tile goes through shared memory once.
//
// Every shape (A, ROWOFF, which row bits a round owns) is a template
// argument, so all index arithmetic folds to constants except one thread
// offset per stage.
#pragma once

#include "hg_internal.h"

namespace hg {
namespace rounds {

// A residue a contiguous pass reads once: not allocated in L1, which keeps
// L1 for the twiddle tables (the 2^25-point middle kernel 2.335 -> 2.319
// ms; marking the tables' loads evict-last as well measured 2.334 ms).
__device__ __forceinline__ uint64_t ld_once(const uint64_t *p) {
  uint64_t v;
  asm("ld.global.L1::no_allocate.u64 %0, [%1];" : "=l"(v) : "l"(p));
  return v;
}

__device__ __forceinline__ uint32_t bitrev(uint32_t r, int bits) { return __brev(r) >> (32 - bits); }

// Thread part of the tile position for register block [A, A+4).
template <int A>
__device__ __forceinline__ uint32_t thread_base(uint32_t tid) {
  return (tid & ((1u << A) - 1u)) | ((tid >> A) << (A + 4));
}

// (w_R^e, companion), e < R/2, loaded into shared memory at entry e.  A
// strided pass's lanes run along columns, so the 8 lanes of one 16-byte
// access read the same entry.
__device__ __forceinline__ void load_sub_twiddles(ulonglong2 *tw, const ulonglong2 *src, int logR, int tid, int nthr) {
  const int half = 1 << (logR - 1);
  for (int e = tid; e < half; e += nthr) tw[e] = __ldg(src + (static_cast<uint64_t>(e) << (kTileBits - logR)));
}

// Twiddle w_M^E (E < M = 2^logM) in Montgomery form from the two-level tables
// of w_{2^30}.
__device__ __forceinline__ uint64_t table_twiddle(uint64_t E, int logM, const uint64_t *hi, const uint64_t *lo,
                                                  uint64_t p, uint32_t c) {
  const uint64_t e = E << (kLogNmax - logM);
  const uint64_t th = __ldg(hi + (e >> kTwLevelBits));
  const uint64_t tl = __ldg(lo + (e & ((1u << kTwLevelBits) - 1)));
  return mont_mul(th, tl, p, c);
}

// NB radix-2 stages on register bits [JG, JG+NB) = row bits [BLO, BLO+NB).
// The stage on row bit b multiplies by w_{2^(b+1)}^(r mod 2^b), read from the
// R/2-entry table of w_R at (r mod 2^b) << (LOGR-1-b).  r mod 2^b splits into
// the thread's row bits below b (runtime, zero when TZERO) and the register's
// (compile time).  With TZERO, butterflies whose twiddle is 1 skip the
// multiplication.
//
// Forward (DIF) butterflies keep every residue in [0, p), as ntt-forward
// does.  Inverse (DIT) butterflies take and leave [0, 2p) (2p < 2^64): u is
// folded once, v w is a corrected Shoup product (v folded when w = 1), and
// u + t, u - t + p need no correction.  Every consumer of an inverse
// residue accepts [0, 2p): the next pass's Montgomery pre-twiddle, the 1/N
// scaling and the reconstruction's Shoup products.
//
// EDGE marks the stage on row bit 0 (BLO = 0, twiddle 1) of a pass whose
// neighbour is a Montgomery product: forward, it is the last stage and its
// u + v, u - v + p go uncorrected ([0, 2p)) into the inter-pass twiddle;
// inverse, it is the first stage and its inputs are already in [0, p).
//
// ZTOP (forward only) marks a first stage whose upper inputs are all zero
// (the zero padding above an operand's limbs): u + 0 and (u - 0) w need
// neither the sum's correction nor the difference, only the product.
//
// CONTIG: the twiddle table is in a contiguous pass's padded order (tw_pos;
// its lanes have different row bits); otherwise entry e sits at e (a
// strided pass's lanes share their row bits).  Either way a twiddle's index
// is the thread's part plus a compile-time part: the thread's table pointer
// is formed once per stage, and each load takes the register's part as its
// address offset.  Dropping the XOR swizzle of the strided passes' tables
// and tiles took the forward strided pass from 0.996 to 0.980 ms and the
// inverse from 0.496 to 0.484 ms (2^25 points).
template <int NB, int JG, int A, int ROWOFF, int BLO, int LOGR, bool INV, bool TZERO, bool EDGE = false,
          bool ZTOP = false, bool CONTIG = false>
__device__ __forceinline__ void stages(uint64_t (&v)[16], const ulonglong2 *__restrict__ tw, uint32_t xt, uint64_t p,
                                       uint32_t c) {
  static_assert(!EDGE || (TZERO && BLO == 0), "the edge stage is the twiddle-free stage on row bit 0");
  static_assert(!ZTOP || !INV, "zero upper inputs only in a forward pass");
#pragma unroll
  for (int s = 0; s < NB; ++s) {
    const int jj = INV ? s : NB - 1 - s;
    const int j = JG + jj;
    const int b = BLO + jj;
    const int sh = LOGR - 1 - b;
    const uint32_t lowmask = (1u << b) - 1u;
    const uint32_t te = TZERO ? 0u : ((xt >> ROWOFF) & lowmask) << sh;
    const ulonglong2 *__restrict__ tws = tw + (CONTIG ? tw_pos(te) : te);
    auto at = [&](uint32_t k) { return CONTIG ? __ldg(tws + tw_pos(k)) : tws[k]; };
#pragma unroll
    for (int i = 0; i < 16; ++i) {
      if (i & (1 << j)) continue;
      const uint32_t rp = ((static_cast<uint32_t>(i) << A) >> ROWOFF) & lowmask;
      const bool trivial = TZERO && rp == 0;
      const uint64_t u = v[i], w = v[i | (1 << j)];
      if (EDGE && jj == 0) {  // twiddle 1, inputs in [0, p): outputs in [0, 2p)
        v[i] = u + w;
        v[i | (1 << j)] = u - w + p;
        continue;
      }
      if (ZTOP && s == 0) {  // w = 0: v[i] keeps u
        if (trivial) {
          v[i | (1 << j)] = u;
        } else {
          const ulonglong2 t = at(rp << sh);
          v[i | (1 << j)] = shoup_mul(u, t.x, t.y, p, c);
        }
        continue;
      }
      if (!INV) {
        v[i] = add_mod(u, w, p);
        if (trivial) {
          v[i | (1 << j)] = sub_mod(u, w, p);
        } else {
          const ulonglong2 t = at(rp << sh);
          v[i | (1 << j)] = shoup_mul(u - w + p, t.x, t.y, p, c);  // u - w + p in (0, 2p)
        }
      } else {
        const uint64_t uu = fold_p(u, p);
        uint64_t t;
        if (trivial) {
          t = fold_p(w, p);
        } else {
          const ulonglong2 tt = at(rp << sh);
          t = shoup_mul(w, tt.x, tt.y, p, c);
        }
        v[i] = uu + t;               // [0, 2p)
        v[i | (1 << j)] = uu - t + p;  // (0, 2p)
      }
    }
  }
}

// Shared-memory word of tile position x: data_swz(x) in a contiguous pass
// (its lanes may run at a stride of 16 positions), x in a strided pass
// (lanes run along columns, one position apart; the thread's word pointer
// is formed once and each register's part is the access's address offset).
template <bool CONTIG>
struct SmemAt {
  uint64_t *s;
  uint32_t sx;
  __device__ __forceinline__ SmemAt(uint64_t *sm, uint32_t xt) : s(sm + (CONTIG ? 0u : xt)), sx(data_swz(xt)) {}
  __device__ __forceinline__ uint64_t &operator[](uint32_t k) const { return CONTIG ? s[sx ^ data_swz(k)] : s[k]; }
};

// Registers <-> shared memory for register block A.
template <int A, bool CONTIG = false>
__device__ __forceinline__ void to_smem(uint64_t *sm, const uint64_t (&v)[16], uint32_t xt) {
  const SmemAt<CONTIG> s(sm, xt);
#pragma unroll
  for (int i = 0; i < 16; ++i) s[static_cast<uint32_t>(i) << A] = v[i];
}
template <int A, bool CONTIG = false>
__device__ __forceinline__ void from_smem(uint64_t (&v)[16], uint64_t *sm, uint32_t xt) {
  const SmemAt<CONTIG> s(sm, xt);
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = s[static_cast<uint32_t>(i) << A];
}

// Multiply register i by beta * gamma^bitrev4(i) (Montgomery-form beta, gamma):
// the twiddle w_M^(s * bitrev_R(r)) of the 16 rows r = rhi*16 + i of one
// column, with beta = w_M^(s * bitrev(rhi)), gamma = w_M^(s * R/16).
__device__ __forceinline__ void geometric_twiddle(uint64_t (&v)[16], uint64_t beta, uint64_t gamma, uint64_t p,
                                                  uint32_t c) {
  uint64_t t = beta;
#pragma unroll
  for (int k = 0; k < 16; ++k) {
    const int i = ((k & 1) << 3) | ((k & 2) << 1) | ((k & 4) >> 1) | ((k & 8) >> 3);  // bitrev4(k)
    v[i] = mont_mul(v[i], t, p, c);
    if (k < 15) t = mont_mul(t, gamma, p, c);
  }
}

}  // namespace rounds
}  // namespace hg
