// hg_ntt_bodies.cuh -- the NTT pass bodies shared by the per-pass kernels
// and the persistent batch kernel (hg_persist.cu).
//
// Strided passes with per-thread global loads and stores (the pass that reads
// limbs from batch descriptors or chunks; every pass of the persistent
// kernel), contiguous passes and the middle of a product, and transforms
// below 16 points.  Each body is one CTA's (or one thread's) share of a
// per-pass launch, addressed by its block index; the persistent kernel calls
// the same bodies with the block index of a work item.
#pragma once

#include "hg_ntt_rounds.cuh"

namespace hg {
namespace bodies {

using namespace rounds;

constexpr int kFwd = 0, kInv = 1, kMul = 2, kSqr = 3, kMulSpec = 4;

// A strided pass over one 4096-residue tile (flattened block index bid) with
// per-thread global loads and stores; tw holds 2^(LOGR-1) (twiddle,
// companion) pairs and sm 4096 words of shared memory.  The pass that reads
// and reduces limbs from batch descriptors or chunks runs here.
template <int LOGR, bool INV>
__device__ __forceinline__ void strided_ldg_body(const PassArgs &P, uint64_t bid, ulonglong2 *tw, uint64_t *sm) {
  constexpr int T = kTileBits;
  constexpr int LOGTC = T - LOGR;  // log2 columns per tile
  constexpr int ROWOFF = LOGTC;    // tile bit of row bit 0
  constexpr int A0 = ROWOFF;       // register block of the low row group
  constexpr int A1 = T - 4;        // register block of the top row group
  constexpr int G = (LOGR + 3) / 4;
  constexpr int NB1 = LOGR - 4;  // row bits of the top group (when G == 2)
  static_assert(LOGR >= 4 && LOGR <= 8, "strided passes have 4..8 row bits");

  const uint32_t tid = threadIdx.x;
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
      for (int i = 0; i < 16; ++i) {
        const uint64_t o = off + i * step;
        v[i] = check_index(o, uint64_t(1) << P.logN) ? data[o] : 0;
        check_below(v[i], p);
      }
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
    for (int i = 0; i < 16; ++i) {
      const uint64_t o = off + i * step;
      check_below(v[i], p);
      if (check_index(o, uint64_t(1) << P.logN)) data[o] = v[i];
    }
  } else {
    uint32_t xt = thread_base<A0>(tid);
    uint64_t off, step;
    offsets(xt, A0, off, step);
#pragma unroll
    for (int i = 0; i < 16; ++i) {
      const uint64_t o = off + i * step;
      v[i] = check_index(o, uint64_t(1) << P.logN) ? data[o] : 0;
      check_below(v[i], 2 * p);
    }
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
    for (int i = 0; i < 16; ++i) {
      const uint64_t o = off + i * step;
      check_below(v[i], 2 * p);
      if (check_index(o, uint64_t(1) << P.logN)) data[o] = v[i];
    }
  }
}

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
  stages<NB, JG, A, 0, 4 * g, T, INV, TZERO, EDGE && TZERO, false, true>(v, tw, xt, p, c);
}

// Move the thread's registers from the layout of group g to that of group h
// through sm.  The barrier after the writes makes them visible; the one
// before them (wait) keeps the writes from overtaking threads that still
// read the buffer's last exchange, and is left out where no thread has read
// the buffer since the last barrier the whole CTA passed.
template <int T, int g, int h>
__device__ __forceinline__ void regroup(uint64_t (&v)[16], uint64_t *sm, uint32_t &xt, uint32_t tid,
                                        bool wait = true) {
  using Gr = Groups<T>;
  constexpr int Ag = Gr::template A<g>(), Ah = Gr::template A<h>();
  if constexpr (Ag == Ah) return;
  if (wait) __syncthreads();
  to_smem<Ag, true>(sm, v, xt);
  __syncthreads();
  xt = thread_base<Ah>(tid);
  from_smem<Ah, true>(v, sm, xt);
}

// Exchange buffers of a block's rounds: the first exchange goes through sm1,
// the second (three groups) through sm2; wait1 and wait2 as regroup's wait.
struct Exchanges {
  uint64_t *sm1, *sm2;
  bool wait1, wait2;
};
__device__ __forceinline__ Exchanges through(uint64_t *sm) { return Exchanges{sm, sm, true, true}; }

// All forward rounds, from the top group down to group 0.  EDGE_LAST: the
// last stage (twiddle 1) leaves its sums and differences uncorrected, in
// [0, 2p), for a consumer that takes them (the pointwise mont_mul_2p).
template <int T, bool EDGE_LAST = false>
__device__ __forceinline__ void forward_rounds(uint64_t (&v)[16], Exchanges x, const ulonglong2 *tw, uint32_t &xt,
                                               uint32_t tid, uint64_t p, uint32_t c) {
  constexpr int G = Groups<T>::G;
  if constexpr (G == 3) {
    round_g<T, 2, false>(v, tw, xt, p, c);
    regroup<T, 2, 1>(v, x.sm1, xt, tid, x.wait1);
    round_g<T, 1, false>(v, tw, xt, p, c);
    regroup<T, 1, 0>(v, x.sm2, xt, tid, x.wait2);
    round_g<T, 0, false, EDGE_LAST>(v, tw, xt, p, c);
  } else if constexpr (G == 2) {
    round_g<T, 1, false>(v, tw, xt, p, c);
    regroup<T, 1, 0>(v, x.sm1, xt, tid, x.wait1);
    round_g<T, 0, false, EDGE_LAST>(v, tw, xt, p, c);
  } else {
    round_g<T, 0, false, EDGE_LAST>(v, tw, xt, p, c);
  }
}

// All inverse rounds, from group 0 up to the top group.  CANON_IN: the
// residues come from the pointwise product, in [0, p).
template <int T, bool CANON_IN = false>
__device__ __forceinline__ void inverse_rounds(uint64_t (&v)[16], Exchanges x, const ulonglong2 *tw, uint32_t &xt,
                                               uint32_t tid, uint64_t p, uint32_t c) {
  constexpr int G = Groups<T>::G;
  round_g<T, 0, true, CANON_IN>(v, tw, xt, p, c);
  if constexpr (G >= 2) {
    regroup<T, 0, 1>(v, x.sm1, xt, tid, x.wait1);
    round_g<T, 1, true>(v, tw, xt, p, c);
  }
  if constexpr (G == 3) {
    regroup<T, 1, 2>(v, x.sm2, xt, tid, x.wait2);
    round_g<T, 2, true>(v, tw, xt, p, c);
  }
}

// Residues read here lie below `bound` (p for a forward input, 2p for an
// inverse one), checked in checked builds.
template <int A>
__device__ __forceinline__ void load_block(uint64_t (&v)[16], const uint64_t *data, const uint64_t *limbs, uint64_t nl,
                                           uint64_t base, uint32_t xt, uint64_t p, uint64_t bound = 0) {
  if (limbs) {
#pragma unroll
    for (int i = 0; i < 16; ++i) {
      const uint64_t o = base + (xt | (static_cast<uint32_t>(i) << A));
      v[i] = o < nl ? reduce64(__ldg(limbs + o), p) : 0;
    }
  } else {
#pragma unroll
    for (int i = 0; i < 16; ++i) {
      v[i] = ld_once(data + base + (xt | (static_cast<uint32_t>(i) << A)));
      check_below(v[i], bound ? bound : p);
    }
  }
}

__device__ __forceinline__ void zero16(uint64_t (&v)[16]) {
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = 0;
}

template <int A>
__device__ __forceinline__ void store_block(const uint64_t (&v)[16], uint64_t *data, uint64_t base, uint32_t xt,
                                            uint64_t bound = ~0ull) {
#pragma unroll
  for (int i = 0; i < 16; ++i) {
    check_below(v[i], bound);
    data[base + (xt | (static_cast<uint32_t>(i) << A))] = v[i];
  }
}

// CTAs of 256 threads per SM: three (80 registers) where the rounds fit
// without spilling, two (128 registers) for the 9..11-bit blocks.
__host__ __device__ constexpr int contig_min_blocks(int T) { return (T >= 9 && T <= 11) ? 2 : 3; }

// One CTA's blocks of a contiguous pass: CTA (bx, by) of the per-pass
// launch; smem holds (MODE == kMul ? 2 : 1) * 4096 words.
template <int T, int MODE>
__device__ __forceinline__ void contig_body(const PassArgs &P, uint64_t bx, int by, uint64_t *smem) {
#include "hg_contig_body.inc"
}

// Transforms of 2, 4 or 8 points: the reference's loops, one thread per
// (product, prime).
__device__ __forceinline__ void tiny_body(const PassArgs &P, int mode, uint64_t prod, int by) {
  const int prime = P.prime_lo + by;
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

}  // namespace bodies
}  // namespace hg
