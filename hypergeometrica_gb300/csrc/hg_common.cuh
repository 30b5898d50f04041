// hg_common.cuh -- shared definitions of the GB300 multiplication library.
//
// Arithmetic is modulo the reference's three NTT primes (default-moduli,
// src/moduli.lisp:257-264): p = c * 2^55 + 1 with c = 197, 174, 131.  That
// shape makes Montgomery reduction with R = 2^64 cheap: p^-1 mod 2^64 is
// 1 - c*2^55, and floor(m*p / 2^64) needs only a 64 x 8-bit product.  The
// reference's Barrett (m*/fast, src/modular-arithmetic.lisp:167-202) and
// Shoup (m*/fast2, :207-231) multiplications compute the same residues; only
// the instruction sequence differs.  Data stays in normal form; twiddles are
// stored in Montgomery form (w * 2^64 mod p), so mont_mul(x, w~) = x*w mod p.
#pragma once

#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

namespace hg {

constexpr int kPrimes = 3;      // moduli in the scheme
constexpr int kShift = 55;      // p = c * 2^kShift + 1
constexpr int kLogNmax = 30;    // largest transform: 2^30 limbs
constexpr int kTwLevelBits = 15;  // two-level twiddle tables: 2^15 entries per level
constexpr int kTileBits = 12;   // in-CTA transform tile: 2^12 residues
constexpr int kTileThreads = 256;
constexpr int kPerThread = 16;  // residues held in registers per thread

// Per-prime constants.
struct PrimeConst {
  uint64_t p;
  uint32_t c;  // p = c * 2^55 + 1
  uint32_t pad;
};

// Device error word codes (latched with atomicCAS; first error wins).
enum DevErr : int {
  kDevOk = 0,
  kDevCarryOverflow = 2,  // a carry left the top of the result
  kDevTicket = 3,         // a carry tile ticket fell outside its launch, or a tile aggregate of another launch
  kDevCopyTimeout = 4,    // a tile copy (TMA) did not land within its wait limit
  kDevQueueTimeout = 5,   // a persistent batch's item waited past its limit for the phase before it
  // Checked builds (HG_CHECKED) only:
  kDevRange = 6,          // a residue outside the range its pass guarantees (>= p, or >= 2p)
  kDevBounds = 7,         // a residue index outside its array; the access was skipped
  kDevProduct = 8,        // a modular product that differs from an exact 128-bit reduction
};

// ---- checked builds -------------------------------------------------------
//
// Built with -DHG_CHECKED=1 (libhg_gb300_checked.so), the kernels check what
// the reference checks under :hypergeometrica-safe and -paranoid
// (src/config.lisp:31-37): every residue a pass reads or writes lies in its
// range (ntt-forward asserts its inputs are below m,
// src/number-theoretic-transform.lisp:63-64), every residue index lies in
// its array, and every modular product equals an independent reduction of
// the full 128-bit product (m*/fast2 re-checks against bignum mod,
// src/modular-arithmetic.lisp:228-229).  A failed check latches a code in a
// fault word of the translation unit (one per .cu file, read and cleared by
// the host at hg_sync); an index out of range also skips the access.
#ifndef HG_CHECKED
#define HG_CHECKED 0
#endif

#if HG_CHECKED
static __device__ int g_checked_fault;
// Host: the fault word of this translation unit, cleared once read.
#define HG_CHECKED_READER(name)                                                     \
  int name() {                                                                      \
    int v = 0;                                                                      \
    if (cudaMemcpyFromSymbol(&v, g_checked_fault, sizeof v) != cudaSuccess) {       \
      cudaGetLastError();                                                           \
      return -1;                                                                    \
    }                                                                               \
    if (v) {                                                                        \
      const int z = 0;                                                              \
      cudaMemcpyToSymbol(g_checked_fault, &z, sizeof z);                            \
    }                                                                               \
    return v;                                                                       \
  }
#endif

__device__ __forceinline__ void checked_fault(int code) {
#if HG_CHECKED
  atomicCAS(&g_checked_fault, 0, code);
#else
  (void)code;
#endif
}

// x < bound, checked (checked builds only; nothing otherwise).
__device__ __forceinline__ void check_below(uint64_t x, uint64_t bound) {
#if HG_CHECKED
  if (x >= bound) checked_fault(kDevRange);
#else
  (void)x;
  (void)bound;
#endif
}

// Index o < n, checked: false (and a fault latched) when it is not.  Always
// true in unchecked builds.
__device__ __forceinline__ bool check_index(uint64_t o, uint64_t n) {
#if HG_CHECKED
  if (o >= n) {
    checked_fault(kDevBounds);
    return false;
  }
#else
  (void)o;
  (void)n;
#endif
  return true;
}

#if HG_CHECKED
// (a * b) mod p by binary long division of the 128-bit product, one bit at a
// time: the independent reduction checked builds compare every product with.
static __device__ __noinline__ uint64_t mulmod_exact(uint64_t a, uint64_t b, uint64_t p) {
  const uint64_t lo = a * b, hi = __umul64hi(a, b);
  uint64_t r = 0;  // r < p < 2^63, so 2r + 1 fits
  for (int i = 127; i >= 0; --i) {
    const uint64_t bit = i >= 64 ? (hi >> (i - 64)) & 1u : (lo >> i) & 1u;
    r = (r << 1) | bit;
    if (r >= p) r -= p;
  }
  return r;
}
#endif

// Latch `code` in the device error word (the first error wins).
__device__ __forceinline__ void latch_error(int *err, int code) {
  if (err) atomicCAS(err, 0, code);
}

// x - p when x >= p, else x, for x < 2p and p < 2^63 (all three primes).
// The butterflies' corrections select rather than add a sign mask (17.5
// against 19.3 ALU-pipe instructions per forward butterfly on a butterfly
// network).  The condition is the sign of d = x - p itself: for x >= p,
// d < p < 2^63; for x < p the difference wraps to 2^64 - (p - x) > 2^63.
// Measured on a register-only butterfly network: 3.0% more forward and
// 1.2% more inverse butterflies per second than taking the condition from
// the borrow of the subtraction (sub.cc/subc, then a predicate from it),
// and that one was 3-5% ahead of a separate 64-bit compare; the same
// residues.
__host__ __device__ __forceinline__ uint64_t fold_p(uint64_t x, uint64_t p) {
#ifdef __CUDA_ARCH__
  const uint64_t d = x - p;
  return static_cast<int64_t>(d) < 0 ? x : d;
#else
  return x >= p ? x - p : x;
#endif
}

// x - q when x >= q, else x, for any x < 2q (a modulus of any size).
__host__ __device__ __forceinline__ uint64_t fold_any(uint64_t x, uint64_t q) { return x >= q ? x - q : x; }

__host__ __device__ __forceinline__ uint64_t add_mod(uint64_t a, uint64_t b, uint64_t p) {
  return fold_p(a + b, p);  // a + b < 2p < 2^64
}

__host__ __device__ __forceinline__ uint64_t sub_mod(uint64_t a, uint64_t b, uint64_t p) {
  return a >= b ? a - b : a - b + p;
}

// sub_mod with the borrow of a - b selecting whether p is added.  Faster
// in the reconstruction (0.448 -> 0.425 ms per 2^25-limb carry launch pair),
// slower inside the butterfly kernels, which keep the compare form.
__device__ __forceinline__ uint64_t sub_mod_borrow(uint64_t a, uint64_t b, uint64_t p) {
  uint64_t r;
  asm("{\n\t.reg .u32 a0, a1, b0, b1, p0, p1, d0, d1, e0, e1, m;\n\t.reg .pred n;\n\t"
      "mov.b64 {a0, a1}, %1;\n\t"
      "mov.b64 {b0, b1}, %2;\n\t"
      "mov.b64 {p0, p1}, %3;\n\t"
      "sub.cc.u32 d0, a0, b0;\n\t"
      "subc.cc.u32 d1, a1, b1;\n\t"
      "subc.u32 m, 0, 0;\n\t"  // all ones when a < b
      "setp.ne.u32 n, m, 0;\n\t"
      "add.cc.u32 e0, d0, p0;\n\t"
      "addc.u32 e1, d1, p1;\n\t"
      "selp.u32 d0, e0, d0, n;\n\t"
      "selp.u32 d1, e1, d1, n;\n\t"
      "mov.b64 %0, {d0, d1};\n\t}"
      : "=l"(r)
      : "l"(a), "l"(b), "l"(p));
  return r;
}

__device__ __forceinline__ uint64_t mul_hi64(uint64_t a, uint64_t b) { return __umul64hi(a, b); }

// Montgomery product a * b * 2^-64 mod p, for any 64-bit a and b < p (WIDE:
// a, b < 2p), with p = c * 2^55 + 1.  Result is fully reduced in [0, p).
//   m = lo * p^-1 mod 2^64 = lo - ((lo * c) mod 2^9) * 2^55   (m1:m0 below)
//   floor(m * p / 2^64) = u * 2^23 + floor((t mod 2^32) / 2^9) with
//   t = m0 * c + floor(m / 2^55) and u = m1 * c + floor(t / 2^32) < 2^40;
// the last product and sum are formed with IMAD (mad.wide.u32), which keeps
// them off the integer ALU pipe that the butterflies' additions load.
template <bool WIDE = false>
__device__ __forceinline__ uint64_t mont_mul(uint64_t a, uint64_t b, uint64_t p, uint32_t c) {
  const uint64_t lo = a * b;
  const uint64_t hi = mul_hi64(a, b);  // < p because a < 2^64 and b < p (WIDE: a, b < 2p)
  const uint32_t m0 = static_cast<uint32_t>(lo);
  const uint32_t m1 = static_cast<uint32_t>(lo >> 32) - m0 * (c << 23);
  uint64_t t;
  asm("{\n\t.reg .u32 sh;\n\t.reg .u64 shw;\n\t"
      "shr.u32 sh, %2, 23;\n\t"
      "cvt.u64.u32 shw, sh;\n\t"
      "mad.wide.u32 %0, %1, %3, shw;\n\t}"
      : "=l"(t)
      : "r"(m0), "r"(m1), "r"(c));
  const uint64_t u = static_cast<uint64_t>(m1) * c + (t >> 32);
  uint64_t mph;
  asm("{\n\t.reg .u32 t9;\n\t.reg .u64 t9w;\n\t"
      "shr.u32 t9, %1, 9;\n\t"
      "cvt.u64.u32 t9w, t9;\n\t"
      "mad.wide.u32 %0, %2, 8388608, t9w;\n\t}"
      : "=l"(mph)
      : "r"(static_cast<uint32_t>(t)), "r"(static_cast<uint32_t>(u)));
  mph += static_cast<uint64_t>(static_cast<uint32_t>(u >> 32)) << 55;
  uint64_t r;
  if constexpr (WIDE)  // hi < (2p)^2 / 2^64 < 2p, so hi - mph lies in (-p, 2p)
    r = hi >= mph ? fold_p(hi - mph, p) : hi - mph + p;
  else
    r = hi >= mph ? hi - mph : hi - mph + p;  // low halves cancel exactly; hi, mph < p
#if HG_CHECKED
  // r 2^64 = a b (mod p), with 2^64 mod p = (2^32)^2 mod p
  if (r >= p || mulmod_exact(r, mulmod_exact(1ull << 32, 1ull << 32, p), p) != mulmod_exact(a, b, p))
    checked_fault(kDevProduct);
#endif
  return r;
}

// The Montgomery product of a, b < 2p (both factors left uncorrected by the
// last forward stage of the middle pass): one correction more.
__device__ __forceinline__ uint64_t mont_mul_2p(uint64_t a, uint64_t b, uint64_t p, uint32_t c) {
  return mont_mul<true>(a, b, p, c);
}

// Shoup product a * w mod p for any 64-bit a, w < p with companion
// wq = floor(w * 2^64 / p) (the reference's m*/fast2,
// src/modular-arithmetic.lisp:207-231).  q = floor(a * wq / 2^64) leaves
// r = a*w - q*p in [0, 2p).  r is formed as a*w + q*(2^64 - p) mod 2^64 by
// one chain of 32-bit multiply-adds (mul.wide, mad.wide, four mad.lo) on the
// FMA pipe, none on the integer ALU pipe that the butterflies' additions and
// selects keep busy.  The words of 2^64 - p come from p at run time, so the
// compiler keeps them as multiplications.  On a register-only butterfly
// network: 3-7% more forward and 2% more inverse butterflies per second than
// subtracting q*p mod 2^64 = q + ((q * c) mod 2^9) * 2^55 on the ALU pipe
// (the fold's subtraction and the additions moved onto IMAD measured slower).
__device__ __forceinline__ uint64_t shoup_mul(uint64_t a, uint64_t w, uint64_t wq, uint64_t p, uint32_t c) {
  (void)c;
  const uint64_t q = mul_hi64(a, wq);
  const uint64_t np = 0 - p;
  uint64_t r;
  asm("{\n\t.reg .u32 a0, a1, w0, w1, q0, q1, n0, n1, r0, r1;\n\t"
      "mov.b64 {a0, a1}, %1;\n\t"
      "mov.b64 {w0, w1}, %2;\n\t"
      "mov.b64 {q0, q1}, %3;\n\t"
      "mov.b64 {n0, n1}, %4;\n\t"
      "mul.wide.u32 %0, a0, w0;\n\t"
      "mad.wide.u32 %0, q0, n0, %0;\n\t"
      "mov.b64 {r0, r1}, %0;\n\t"
      "mad.lo.u32 r1, a0, w1, r1;\n\t"
      "mad.lo.u32 r1, a1, w0, r1;\n\t"
      "mad.lo.u32 r1, q0, n1, r1;\n\t"
      "mad.lo.u32 r1, q1, n0, r1;\n\t"
      "mov.b64 %0, {r0, r1};\n\t}"
      : "=l"(r)
      : "l"(a), "l"(w), "l"(q), "l"(np));
  const uint64_t out = fold_p(r, p);
#if HG_CHECKED
  if (out != mulmod_exact(a, w, p)) checked_fault(kDevProduct);
#endif
  return out;
}

// x mod p for any 64-bit x (x < 4p because p > 2^62; 2p itself exceeds
// 2^63, so the first correction compares).
__device__ __forceinline__ uint64_t reduce64(uint64_t x, uint64_t p) {
  return fold_p(fold_any(x, p << 1), p);
}

// Carry-lookahead pair for the final carry scan: with carry-in c, a
// position (or a run of positions) emits carry g | (p & c).
struct GP {
  uint32_t g, p;
};
// Compose: first `lo` (less significant run), then `hi`.
__host__ __device__ __forceinline__ GP gp_compose(GP lo, GP hi) {
  return GP{hi.g | (hi.p & lo.g), hi.p & lo.p};
}

}  // namespace hg
