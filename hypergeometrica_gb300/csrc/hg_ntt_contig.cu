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
#include "hg_ntt_bodies.cuh"

namespace hg {
namespace {

using namespace rounds;
using namespace bodies;

template <int T, int MODE>
__global__ void __launch_bounds__(kTileThreads, contig_min_blocks(T)) ntt_contig_kernel(const PassArgs P) {
  extern __shared__ uint64_t smem[];
  const uint64_t bx = blockIdx.x;
  const int by = static_cast<int>(blockIdx.y);
#include "hg_contig_body.inc"
}

__global__ void ntt_tiny_kernel(const PassArgs P, int mode) {
  tiny_body(P, mode, blockIdx.x, static_cast<int>(blockIdx.y));
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

#if HG_CHECKED
HG_CHECKED_READER(checked_fault_contig)
#endif

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
