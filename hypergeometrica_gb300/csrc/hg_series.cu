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

}  // namespace
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

}  // extern "C"
