// hg_series.cu -- the base cases of binary splitting on the device.
//
// binary-split-base-case=1 (src/binary-splitting.lisp:102-110) turns each term
// k of a series into the partial P = p(k), Q = q(k), B = b(k), R = p(k) a(k).
// For the reference's series (src/binary-splitting.lisp:147-231,
// src/pi.lisp:24-43) a, b, p and q are integer polynomials in k, with p(0) and
// q(0) replaced by 1.  One thread per term evaluates them by Horner's rule in
// 256-bit two's complement (k < 2^63, coefficients int64; the caller checks
// that every value and R fit in 255 bits) and writes sign, length without
// high zero limbs and four limbs per value.
#include "hg_host.h"
#include "hypergeometrica_gb300.h"

namespace hg {
namespace {

struct U256 {
  uint64_t w[4];
};

__device__ __forceinline__ U256 mul_small(const U256 &a, uint64_t n) {  // a * n mod 2^256
  U256 r;
  uint64_t carry = 0;
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const uint64_t lo = a.w[i] * n, hi = __umul64hi(a.w[i], n);
    r.w[i] = lo + carry;
    carry = hi + (r.w[i] < lo ? 1 : 0);
  }
  return r;
}

__device__ __forceinline__ U256 add_signed(const U256 &a, int64_t c) {  // a + c mod 2^256
  const uint64_t ext = c < 0 ? ~0ull : 0ull;
  U256 r;
  uint64_t carry = 0;
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const uint64_t y = i == 0 ? static_cast<uint64_t>(c) : ext;
    const uint64_t s = a.w[i] + y;
    const uint64_t t = s + carry;
    carry = (s < a.w[i] ? 1 : 0) + (t < s ? 1 : 0);
    r.w[i] = t;
  }
  return r;
}

__device__ __forceinline__ bool negative(const U256 &a) { return static_cast<int64_t>(a.w[3]) < 0; }

__device__ __forceinline__ U256 negate(const U256 &a) {
  U256 r;
  uint64_t carry = 1;
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const uint64_t x = ~a.w[i];
    r.w[i] = x + carry;
    carry = r.w[i] < x ? 1 : 0;
  }
  return r;
}

__device__ U256 eval_poly(const hg_poly &q, uint64_t n) {
  U256 acc{{0, 0, 0, 0}};
  if (n == 0 && q.has_zero_value) return add_signed(acc, q.zero_value);
  for (int i = q.degree; i >= 0; --i) acc = add_signed(mul_small(acc, n), q.coef[i]);
  return acc;
}

// Magnitude product mod 2^256 of two non-negative values.
__device__ U256 mul_mag(const U256 &a, const U256 &b) {
  U256 r{{0, 0, 0, 0}};
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    uint64_t carry = 0;
#pragma unroll
    for (int j = 0; j + i < 4; ++j) {
      const uint64_t lo = a.w[i] * b.w[j], hi = __umul64hi(a.w[i], b.w[j]);
      const uint64_t s = r.w[i + j] + lo;
      const uint64_t t = s + carry;
      carry = hi + (s < lo ? 1 : 0) + (t < s ? 1 : 0);
      r.w[i + j] = t;
    }
  }
  return r;
}

__device__ void emit(const U256 &v, uint64_t *limbs, int64_t *ss) {
  const bool neg = negative(v);
  const U256 m = neg ? negate(v) : v;
  int size = 0;
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    limbs[i] = m.w[i];
    if (m.w[i]) size = i + 1;
  }
  ss[0] = (neg && size) ? -1 : 1;
  ss[1] = size;
}

__global__ void leaves_kernel(hg_poly pa, hg_poly pb, hg_poly pp, hg_poly pq, uint64_t lower, uint64_t count,
                              uint64_t *limbs, int64_t *ss) {
  const uint64_t k = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x;
  if (k >= count) return;
  const uint64_t n = lower + k;
  const U256 p = eval_poly(pp, n), q = eval_poly(pq, n), b = eval_poly(pb, n), a = eval_poly(pa, n);
  const bool pn = negative(p), an = negative(a);
  U256 r = mul_mag(pn ? negate(p) : p, an ? negate(a) : a);
  if (pn != an) r = negate(r);
  const U256 vals[4] = {p, q, b, r};
#pragma unroll
  for (int j = 0; j < 4; ++j) emit(vals[j], limbs + (j * count + k) * 4, ss + (j * count + k) * 2);
}

// ---- whole nodes ----------------------------------------------------------
//
// A node's partial (P, Q, B, R) over terms [lo, hi) is a function of the
// range alone: combine (src/binary-splitting.lisp:112-121) is exact integer
// arithmetic, so any split of the range gives the same four integers.  Here
// one thread folds the terms left to right: with a one-term right part t,
// combine is
//   R <- b_t q_t R + (B P) r_t,  P <- P p_t,  Q <- Q q_t,  B <- B b_t,
// where r_t = p_t a_t, so keeping BP = B P as a fifth value makes every step
// a product by a value below 2^256.  Values are sign and magnitude; the
// magnitudes live in global memory, W limbs each.

// acc (three words) += a * b.
__device__ __forceinline__ void mac3(uint64_t &a0, uint64_t &a1, uint64_t &a2, uint64_t a, uint64_t b) {
  const uint64_t lo = a * b, hi = __umul64hi(a, b);
  a0 += lo;
  const uint64_t c0 = a0 < lo ? 1 : 0;
  const uint64_t t = a1 + hi;
  const uint64_t c1 = t < hi ? 1 : 0;
  a1 = t + c0;
  a2 += c1 + (a1 < c0 ? 1 : 0);
}

__device__ __forceinline__ int limbs_of(const U256 &m) {
  int n = 4;
  while (n > 0 && m.w[n - 1] == 0) --n;
  return n;
}

__device__ __forceinline__ int trimmed_size(const uint64_t *x, int n) {
  while (n > 0 && x[n - 1] == 0) --n;
  return n;
}

// out[0, n + |m|) = x[0, n) * m (magnitudes); out may be x itself: limb i
// of the product needs x[i - 3 .. i] only, and the three below i are kept in
// registers before they are overwritten.  Returns the trimmed size, or -1
// when the product may not fit in cap limbs.
__device__ int mul_by(uint64_t *out, const uint64_t *x, int n, const U256 &m, int cap) {
  const int ms = limbs_of(m);
  if (n == 0 || ms == 0) return 0;
  if (n + ms > cap) return -1;
  uint64_t w1 = 0, w2 = 0, w3 = 0, c0 = 0, c1 = 0;
  for (int i = 0; i < n + ms; ++i) {
    const uint64_t xi = i < n ? x[i] : 0;
    uint64_t a0 = c0, a1 = c1, a2 = 0;
    mac3(a0, a1, a2, xi, m.w[0]);
    if (ms > 1) mac3(a0, a1, a2, w1, m.w[1]);
    if (ms > 2) mac3(a0, a1, a2, w2, m.w[2]);
    if (ms > 3) mac3(a0, a1, a2, w3, m.w[3]);
    out[i] = a0;
    c0 = a1;
    c1 = a2;
    w3 = w2;
    w2 = w1;
    w1 = xi;
  }
  return trimmed_size(out, n + ms);
}

// x (sign sx, size nx) += y (sign sy, size ny), in place in x.  Returns the
// trimmed size (sx updated), or -1 when the sum may not fit in cap limbs.
__device__ int add_signed_big(uint64_t *x, int nx, int &sx, const uint64_t *y, int ny, int sy, int cap) {
  if (ny == 0) return nx;
  if (nx == 0) {
    if (ny > cap) return -1;
    for (int i = 0; i < ny; ++i) x[i] = y[i];
    sx = sy;
    return ny;
  }
  const int n = nx > ny ? nx : ny;
  if (sx == sy) {
    if (n + 1 > cap) return -1;
    uint64_t carry = 0;
    for (int i = 0; i < n; ++i) {
      const uint64_t a = i < nx ? x[i] : 0, b = i < ny ? y[i] : 0;
      const uint64_t s = a + b, t = s + carry;
      carry = (s < a ? 1 : 0) + (t < s ? 1 : 0);
      x[i] = t;
    }
    x[n] = carry;
    return trimmed_size(x, n + 1);
  }
  // Opposite signs: subtract the smaller magnitude from the larger.
  int cmp = nx != ny ? (nx > ny ? 1 : -1) : 0;
  for (int i = n - 1; cmp == 0 && i >= 0; --i)
    if (x[i] != y[i]) cmp = x[i] > y[i] ? 1 : -1;
  if (cmp == 0) return 0;  // zero: sign is irrelevant
  uint64_t borrow = 0;
  for (int i = 0; i < n; ++i) {
    const uint64_t a = i < nx ? x[i] : 0, b = i < ny ? y[i] : 0;
    const uint64_t big = cmp > 0 ? a : b, small = cmp > 0 ? b : a;
    const uint64_t d = big - small, e = d - borrow;
    borrow = (big < small ? 1 : 0) + (d < borrow ? 1 : 0);
    x[i] = e;
  }
  if (cmp < 0) sx = sy;
  return trimmed_size(x, n);
}

struct Term {
  U256 p, q, b, r;  // magnitudes
  int sp, sq, sb, sr;
};

__device__ Term eval_term(const hg_poly &pa, const hg_poly &pb, const hg_poly &pp, const hg_poly &pq, uint64_t k) {
  const U256 p = eval_poly(pp, k), q = eval_poly(pq, k), b = eval_poly(pb, k), a = eval_poly(pa, k);
  Term t;
  const bool pn = negative(p), qn = negative(q), bn = negative(b), an = negative(a);
  t.p = pn ? negate(p) : p;
  t.q = qn ? negate(q) : q;
  t.b = bn ? negate(b) : b;
  t.r = mul_mag(t.p, an ? negate(a) : a);
  t.sp = pn ? -1 : 1;
  t.sq = qn ? -1 : 1;
  t.sb = bn ? -1 : 1;
  t.sr = pn != an ? -1 : 1;
  return t;
}

__device__ int set_u256(uint64_t *x, const U256 &m) {
#pragma unroll
  for (int i = 0; i < 4; ++i) x[i] = m.w[i];
  return limbs_of(m);
}

// One thread per node: ranges[2 i], ranges[2 i + 1] = lo, hi.  Value j of
// node i: limbs[(j n + i) W ..], sign_size[(j n + i) 2 ..]; scratch holds BP
// and a temporary, 2 W limbs per node.  A size that would pass W is written
// as -1 (and the node's values are not used).
__global__ void nodes_kernel(hg_poly pa, hg_poly pb, hg_poly pp, hg_poly pq, const uint64_t *ranges, uint64_t n,
                             uint64_t width, uint64_t *limbs, int64_t *ss, uint64_t *scratch) {
  const uint64_t i = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x;
  if (i >= n) return;
  const uint64_t lo = ranges[2 * i], hi = ranges[2 * i + 1];
  const int cap = static_cast<int>(width);
  uint64_t *P = limbs + (0 * n + i) * width, *Q = limbs + (1 * n + i) * width;
  uint64_t *B = limbs + (2 * n + i) * width, *R = limbs + (3 * n + i) * width;
  uint64_t *BP = scratch + (2 * i) * width, *T = scratch + (2 * i + 1) * width;
  Term t = eval_term(pa, pb, pp, pq, lo);
  int nP = set_u256(P, t.p), nQ = set_u256(Q, t.q), nB = set_u256(B, t.b), nR = set_u256(R, t.r);
  int sP = t.sp, sQ = t.sq, sB = t.sb, sR = t.sr;
  int nBP = mul_by(BP, B, nB, t.p, cap), sBP = sB * sP;
  bool ok = nBP >= 0;
  for (uint64_t k = lo + 1; ok && k < hi; ++k) {
    t = eval_term(pa, pb, pp, pq, k);
    // R <- b q R + BP r
    nR = mul_by(R, R, nR, t.q, cap);
    if (nR >= 0) nR = mul_by(R, R, nR, t.b, cap);
    sR *= t.sq * t.sb;
    const int nT = mul_by(T, BP, nBP, t.r, cap);
    if (nR >= 0 && nT >= 0) nR = add_signed_big(R, nR, sR, T, nT, sBP * t.sr, cap);
    // P, Q, B, BP
    nP = mul_by(P, P, nP, t.p, cap);
    nQ = mul_by(Q, Q, nQ, t.q, cap);
    nB = mul_by(B, B, nB, t.b, cap);
    nBP = mul_by(BP, BP, nBP, t.b, cap);
    if (nBP >= 0) nBP = mul_by(BP, BP, nBP, t.p, cap);
    sP *= t.sp;
    sQ *= t.sq;
    sB *= t.sb;
    sBP *= t.sb * t.sp;
    ok = nR >= 0 && nT >= 0 && nP >= 0 && nQ >= 0 && nB >= 0 && nBP >= 0;
  }
  const int sizes[4] = {nP, nQ, nB, nR}, signs[4] = {sP, sQ, sB, sR};
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    int64_t *o = ss + (j * n + i) * 2;
    o[0] = (signs[j] < 0 && sizes[j] > 0) ? -1 : 1;
    o[1] = ok ? sizes[j] : -1;
  }
}

}  // namespace
#if HG_CHECKED
HG_CHECKED_READER(checked_fault_series)
#endif

}  // namespace hg

using namespace hg;

extern "C" {

int hg_series_leaves_device(const hg_poly *polys, uint64_t lower, uint64_t count, uint64_t *limbs, int64_t *sign_size,
                            void *stream) {
  if (!polys || (count && (!limbs || !sign_size))) return lib_fail(HG_ERR_ARG, "null pointer");
  if (!lib_ready()) return lib_fail(HG_ERR_NOT_INIT, "hg_series_leaves_device: call hg_init first");
  for (int j = 0; j < 4; ++j)
    if (polys[j].degree < 0 || polys[j].degree > 7)
      return lib_fail(HG_ERR_ARG, "polynomial %d: degree %d outside 0..7", j, polys[j].degree);
  if (count == 0) return HG_OK;
  if (lower + count < lower || lower + count > (uint64_t(1) << 63))
    return lib_fail(HG_ERR_ARG, "terms [%llu, %llu) out of range", (unsigned long long)lower,
                    (unsigned long long)(lower + count));
  const uint64_t blocks = (count + 255) / 256;
  if (blocks > 0x7fffffffull) return lib_fail(HG_ERR_ARG, "%llu terms exceed one launch", (unsigned long long)count);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  leaves_kernel<<<static_cast<unsigned>(blocks), 256, 0, st>>>(polys[0], polys[1], polys[2], polys[3], lower, count,
                                                               limbs, sign_size);
  const cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? HG_OK : lib_cuda_fail(e, "series leaves");
}

int hg_series_nodes_device(const hg_poly *polys, const uint64_t *ranges, uint64_t n, uint64_t width, uint64_t *limbs,
                           int64_t *sign_size, uint64_t *scratch, void *stream) {
  if (!polys || (n && (!ranges || !limbs || !sign_size || !scratch))) return lib_fail(HG_ERR_ARG, "null pointer");
  if (!lib_ready()) return lib_fail(HG_ERR_NOT_INIT, "hg_series_nodes_device: call hg_init first");
  for (int j = 0; j < 4; ++j)
    if (polys[j].degree < 0 || polys[j].degree > 7)
      return lib_fail(HG_ERR_ARG, "polynomial %d: degree %d outside 0..7", j, polys[j].degree);
  if (width < 8 || width > (1u << 30)) return lib_fail(HG_ERR_ARG, "width %llu outside 8..2^30", (unsigned long long)width);
  if (n == 0) return HG_OK;
  const uint64_t blocks = (n + 127) / 128;
  if (blocks > 0x7fffffffull) return lib_fail(HG_ERR_ARG, "%llu nodes exceed one launch", (unsigned long long)n);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  nodes_kernel<<<static_cast<unsigned>(blocks), 128, 0, st>>>(polys[0], polys[1], polys[2], polys[3], ranges, n,
                                                              width, limbs, sign_size, scratch);
  const cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? HG_OK : lib_cuda_fail(e, "series nodes");
}

}  // extern "C"
