// hg_sum.cu -- signed sums and trimmed sizes of many device integers at once.
//
// mpz-+ on two mpz/ram (src/mpz-ram.lisp:292-306) adds magnitudes when the
// signs agree (%mpz/ram-+, :217-232, with the carry loop of
// %add-storages/unsafe, :184-215) and otherwise subtracts the smaller
// magnitude from the larger (%mpz/ram--, :276-290; %subtract-storages/unsafe,
// :234-274, adds the complement with an initial carry of 1).  mpz-size is the
// length without high zero limbs (vec-digit-length*, src/vec.lisp:218-229).
// Binary splitting needs both for every node of a tree level at once
// (combine, src/binary-splitting.lisp:112-121), so each kernel takes an array
// of descriptors and runs one CTA per integer.
//
// Within a CTA the sum moves in chunks of 2048 limbs (8 per thread): each
// thread forms its limbs' generate/propagate pair, the CTA scans the pairs
// (warp shuffles, then the eight warp totals), and the chunk's carry-out
// feeds the next chunk.
#include "hg_host.h"
#include "hypergeometrica_gb300.h"

namespace hg {
namespace {

constexpr int kSumThreads = 256;
constexpr int kSumPer = 8;
constexpr uint64_t kSumChunk = kSumThreads * kSumPer;

struct SumDesc {
  const uint64_t *a;
  uint64_t na;
  const uint64_t *b;
  uint64_t nb;
  uint64_t *out;
  uint64_t nout;
  int64_t sa, sb;
  int64_t *res;  // (sign, size)
};

// Sums of at least this many limbs run over the whole GPU (large_sum_device)
// instead of in one CTA.
constexpr uint64_t kLargeSum = uint64_t(1) << 15;

struct VecDesc {
  const uint64_t *p;
  uint64_t n;
};

// Descriptors of a launch: a device array, or up to kInline of them carried
// in the kernel's parameters (no allocation or copy for small batches, whose
// cost is then one launch).
constexpr int kInline = 32;
template <class Desc>
struct Descs {
  const Desc *p;  // device array, or null: use inl
  Desc inl[kInline];
  __device__ __forceinline__ Desc operator[](uint64_t i) const { return p ? p[i] : inl[i]; }
};

// Highest index < n whose limb is nonzero (or differs between a and b when
// b != nullptr), -1 if none; scanned from the top one chunk at a time.
__device__ long long top_index(const uint64_t *a, uint64_t na, const uint64_t *b, uint64_t nb, uint64_t n) {
  __shared__ long long s_top;
  if (threadIdx.x == 0) s_top = -1;
  __syncthreads();
  for (uint64_t hi = n; hi > 0;) {
    const uint64_t lo = hi > kSumChunk ? hi - kSumChunk : 0;
    for (uint64_t i = lo + threadIdx.x; i < hi; i += kSumThreads) {
      const uint64_t x = i < na ? a[i] : 0;
      const uint64_t y = b ? (i < nb ? b[i] : 0) : 0;
      if (x != y) atomicMax(&s_top, static_cast<long long>(i));
    }
    __syncthreads();
    // Every thread reads the flag before any thread can move on and update
    // it for the next chunk: the CTA leaves the loop together.
    const bool found = s_top >= 0;
    __syncthreads();
    if (found) break;
    hi = lo;
  }
  const long long t = s_top;
  __syncthreads();
  return t;
}

__global__ void __launch_bounds__(kSumThreads) sum_kernel(const Descs<SumDesc> descs) {
  const SumDesc d = descs[blockIdx.x];
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  const uint64_t n = d.na > d.nb ? d.na : d.nb;
  const bool sub = d.sa != d.sb;
  const uint64_t *X = d.a, *Y = d.b;
  uint64_t nX = d.na, nY = d.nb;
  int64_t sign = d.sa;
  if (sub) {
    const long long t = top_index(d.a, d.na, d.b, d.nb, n);
    if (t < 0) {  // equal magnitudes: zero
      for (uint64_t i = tid; i < d.nout; i += kSumThreads) d.out[i] = 0;
      if (tid == 0) {
        d.res[0] = 1;
        d.res[1] = 0;
      }
      return;
    }
    const uint64_t at = static_cast<uint64_t>(t) < d.na ? d.a[t] : 0;
    const uint64_t bt = static_cast<uint64_t>(t) < d.nb ? d.b[t] : 0;
    if (bt > at) {
      X = d.b;
      nX = d.nb;
      Y = d.a;
      nY = d.na;
      sign = d.sb;
    }
  }
  __shared__ GP s_warp[kSumThreads / 32];
  __shared__ uint32_t s_cin;
  __shared__ long long s_top;
  if (tid == 0) {
    s_cin = sub ? 1u : 0u;  // the complement's +1
    s_top = -1;
  }
  __syncthreads();
  // Subtraction: X + (2^(64n) - 1 - Y) + 1 over exactly n limbs; the carry
  // out of limb n - 1 is dropped and the limbs above are zero.
  const uint64_t span = sub ? n : d.nout;
  for (uint64_t c0 = 0; c0 < d.nout; c0 += kSumChunk) {
    const uint64_t i0 = c0 + static_cast<uint64_t>(tid) * kSumPer;
    uint64_t s[kSumPer];
    uint32_t gen = 0;  // bit j: limb j generates a carry
    GP run{0, 1};
#pragma unroll
    for (int j = 0; j < kSumPer; ++j) {
      const uint64_t i = i0 + j;
      uint64_t x = 0, y = 0;
      if (i < span) {
        x = i < nX ? X[i] : 0;
        y = i < nY ? Y[i] : 0;
        if (sub) y = ~y;
      }
      s[j] = x + y;
      const GP g{s[j] < x ? 1u : 0u, s[j] == ~0ull ? 1u : 0u};
      gen |= g.g << j;
      run = gp_compose(run, g);
    }
    // Exclusive scan of the thread runs in thread order.
    GP inc = run;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
      const uint32_t g = __shfl_up_sync(0xffffffffu, inc.g, off), p = __shfl_up_sync(0xffffffffu, inc.p, off);
      if (lane >= off) inc = gp_compose(GP{g, p}, inc);
    }
    if (lane == 31) s_warp[wid] = inc;
    __syncthreads();
    GP before{0, 1};
    for (int w = 0; w < wid; ++w) before = gp_compose(before, s_warp[w]);
    const uint32_t gx = __shfl_up_sync(0xffffffffu, inc.g, 1), px = __shfl_up_sync(0xffffffffu, inc.p, 1);
    if (lane > 0) before = gp_compose(before, GP{gx, px});
    const uint32_t chunk_cin = s_cin;
    uint32_t carry = before.g | (before.p & chunk_cin);
    long long top = -1;
#pragma unroll
    for (int j = 0; j < kSumPer; ++j) {
      const uint64_t i = i0 + j;
      // Beyond the span (subtraction only) the limbs are zero: the carry out
      // of limb n - 1 is the complement's and is dropped.
      const uint64_t v = i < span ? s[j] + carry : 0;
      carry = ((gen >> j) & 1u) | (s[j] == ~0ull ? carry : 0u);
      if (i < d.nout) {
        d.out[i] = v;
        if (v) top = static_cast<long long>(i);
      }
    }
    if (top >= 0) atomicMax(&s_top, top);
    __syncthreads();
    if (tid == kSumThreads - 1) {
      GP all{0, 1};
      for (int w = 0; w < kSumThreads / 32; ++w) all = gp_compose(all, s_warp[w]);
      s_cin = all.g | (all.p & chunk_cin);
    }
    __syncthreads();
  }
  if (tid == 0) {
    const int64_t size = s_top + 1;
    d.res[0] = size ? sign : 1;
    d.res[1] = size;
  }
}

__global__ void __launch_bounds__(kSumThreads) trim_kernel(const Descs<VecDesc> descs, uint64_t *sizes) {
  const VecDesc d = descs[blockIdx.x];
  const long long t = top_index(d.p, d.n, nullptr, 0, d.n);
  if (threadIdx.x == 0) sizes[blockIdx.x] = static_cast<uint64_t>(t + 1);
}

// %multiply-storage/schoolboy (src/mpz-ram.lisp:404-431) for many small
// products, one thread each: column k of the product is the 192-bit sum of
// x_i y_(k-i) plus the carry from column k - 1 (< 2^71 for <= 64-limb
// operands).
__global__ void small_mul_kernel(const Descs<ProductDesc> descs, uint64_t n) {
  const uint64_t k = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x;
  if (k >= n) return;
  const ProductDesc d = descs[k];
  const uint64_t *x = d.x, *y = d.y ? d.y : d.x;
  uint64_t nx = d.nx, ny = d.y ? d.ny : d.nx;
  if (nx < ny) {
    const uint64_t *t = x;
    x = y;
    y = t;
    const uint64_t u = nx;
    nx = ny;
    ny = u;
  }
  uint64_t w = 0;
  if (ny > 0) {
    uint64_t c0 = 0, c1 = 0;
    for (uint64_t col = 0; col + 1 < nx + ny; ++col) {
      uint64_t a0 = c0, a1 = c1, a2 = 0;
      const uint64_t ilo = col >= ny ? col - ny + 1 : 0, ihi = col < nx ? col : nx - 1;
      for (uint64_t i = ilo; i <= ihi; ++i) {
        const uint64_t u = x[i], v = y[col - i];
        const uint64_t lo = u * v, hi = __umul64hi(u, v);
        a0 += lo;
        const uint64_t cl = a0 < lo ? 1 : 0;
        const uint64_t t = a1 + hi;
        const uint64_t ch = t < hi ? 1 : 0;
        a1 = t + cl;
        a2 += ch + (a1 < cl ? 1 : 0);
      }
      d.out[col] = a0;
      c0 = a1;
      c1 = a2;
    }
    d.out[nx + ny - 1] = c0;
    w = nx + ny;
  }
  for (uint64_t i = w; i < d.nout; ++i) d.out[i] = 0;
}

template <class Desc, class Launch>
int run_batch(const Desc *host, size_t n, cudaStream_t st, const char *what, Launch launch) {
  if (n == 0) return HG_OK;
  if (n > 0x7fffffffull) return lib_fail(HG_ERR_ARG, "%s: %zu integers exceed one launch", what, n);
  if (n <= static_cast<size_t>(kInline)) {
    Descs<Desc> d{};
    for (size_t k = 0; k < n; ++k) d.inl[k] = host[k];
    launch(d, static_cast<unsigned>(n));
    const cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? HG_OK : lib_cuda_fail(e, what);
  }
  Desc *dev = nullptr;
  cudaError_t e = cudaMallocAsync(&dev, n * sizeof(Desc), st);
  if (e != cudaSuccess) return lib_cuda_fail(e, what);
  e = cudaMemcpyAsync(dev, host, n * sizeof(Desc), cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) {
    Descs<Desc> d{};
    d.p = dev;
    launch(d, static_cast<unsigned>(n));
    e = cudaGetLastError();
  }
  const cudaError_t f = cudaFreeAsync(dev, st);
  if (e != cudaSuccess) return lib_cuda_fail(e, what);
  if (f != cudaSuccess) return lib_cuda_fail(f, what);
  return HG_OK;
}

}  // namespace
#if HG_CHECKED
HG_CHECKED_READER(checked_fault_sum)
#endif

}  // namespace hg

using namespace hg;

extern "C" {

int hg_add_batch_device(const hg_sum *sums, size_t n, int64_t *result, void *stream) {
  if (n && (!sums || !result)) return lib_fail(HG_ERR_ARG, "null pointer");
  if (!lib_ready()) return lib_fail(HG_ERR_NOT_INIT, "hg_add_batch_device: call hg_init first");
  std::vector<SumDesc> d;
  d.reserve(n);
  for (size_t k = 0; k < n; ++k) {
    const hg_sum &s = sums[k];
    if ((s.na && !s.a) || (s.nb && !s.b) || (s.nout && !s.out)) return lib_fail(HG_ERR_ARG, "sum %zu: null pointer", k);
    if ((s.sa != 1 && s.sa != -1) || (s.sb != 1 && s.sb != -1))
      return lib_fail(HG_ERR_ARG, "sum %zu: signs must be +1 or -1", k);
    const size_t need = (s.na > s.nb ? s.na : s.nb) + 1;
    if (s.nout < need) return lib_fail(HG_ERR_ARG, "sum %zu: nout = %zu cannot hold %zu limbs", k, s.nout, need);
  }
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  for (size_t k = 0; k < n; ++k) {
    const hg_sum &s = sums[k];
    if ((s.na > s.nb ? s.na : s.nb) >= kLargeSum) {
      const int rc = large_sum_device(s.a, s.na, s.sa, s.b, s.nb, s.sb, s.out, s.nout, result + 2 * k, st);
      if (rc) return rc;
    } else {
      d.push_back(SumDesc{s.a, s.na, s.b, s.nb, s.out, s.nout, s.sa, s.sb, result + 2 * k});
    }
  }
  return run_batch(d.data(), d.size(), st, "signed sums", [&](const Descs<SumDesc> &dev, unsigned grid) {
    sum_kernel<<<grid, kSumThreads, 0, st>>>(dev);
  });
}

int hg_mul_small_batch_device(const hg_product *prods, size_t n, void *stream) {
  if (n && !prods) return lib_fail(HG_ERR_ARG, "null pointer");
  if (!lib_ready()) return lib_fail(HG_ERR_NOT_INIT, "hg_mul_small_batch_device: call hg_init first");
  std::vector<ProductDesc> d(n);
  for (size_t k = 0; k < n; ++k) {
    const hg_product &p = prods[k];
    const bool square = p.y == nullptr;
    const size_t ny = square ? p.nx : p.ny;
    if (!p.out || (p.nx && !p.x)) return lib_fail(HG_ERR_ARG, "product %zu: null pointer", k);
    if (p.nx > HG_SMALL_MAX_LIMBS || ny > HG_SMALL_MAX_LIMBS)
      return lib_fail(HG_ERR_ARG, "product %zu: %zu x %zu limbs exceeds the %d-limb schoolbook limit", k, p.nx, ny,
                      HG_SMALL_MAX_LIMBS);
    if (p.nout < p.nx + ny)
      return lib_fail(HG_ERR_ARG, "product %zu: nout = %zu cannot hold %zu limbs", k, p.nout, p.nx + ny);
    d[k] = ProductDesc{p.x, p.y, p.nx, ny, p.out, p.nout};
  }
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  return run_batch(d.data(), n, st, "small products", [&](const Descs<ProductDesc> &dev, unsigned count) {
    small_mul_kernel<<<(count + 127) / 128, 128, 0, st>>>(dev, count);
  });
}

int hg_trim_batch_device(const hg_vec *vecs, size_t n, uint64_t *sizes, void *stream) {
  if (n && (!vecs || !sizes)) return lib_fail(HG_ERR_ARG, "null pointer");
  if (!lib_ready()) return lib_fail(HG_ERR_NOT_INIT, "hg_trim_batch_device: call hg_init first");
  std::vector<VecDesc> d(n);
  for (size_t k = 0; k < n; ++k) {
    if (vecs[k].n && !vecs[k].p) return lib_fail(HG_ERR_ARG, "vector %zu: null pointer", k);
    d[k] = VecDesc{vecs[k].p, vecs[k].n};
  }
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  return run_batch(d.data(), n, st, "trimmed sizes", [&](const Descs<VecDesc> &dev, unsigned grid) {
    trim_kernel<<<grid, kSumThreads, 0, st>>>(dev, sizes);
  });
}

}  // extern "C"
