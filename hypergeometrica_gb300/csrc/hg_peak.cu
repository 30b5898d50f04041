// hg_peak.cu -- the integer-pipe ceiling of the modular butterflies.
//
// The NTT passes are bound by the integer pipes, not by HBM: each radix-2
// butterfly is a 64-bit modular add, a subtract and a Shoup product built
// from 32-bit IMAD and ALU instructions.  This kernel runs the same
// butterflies (hg_ntt_rounds.cuh's stages: canonical forward, inverse on
// [0, 2p)) on 16 registers per thread with twiddles from shared memory and
// no global traffic, half forward (DIF) then half inverse (DIT), over every
// SM: its rate is the practical peak a memory-free butterfly network
// reaches on this GPU, the denominator of the product's integer-pipe
// roofline.
#include <cstdio>

#include "hg_host.h"
#include "hypergeometrica_gb300.h"

namespace hg {
namespace {

constexpr int kPeakIters = 64;

__global__ void __launch_bounds__(256) peak_kernel(uint64_t *sink, PrimeConst pc, const ulonglong2 *table) {
  __shared__ ulonglong2 tw[16];
  if (threadIdx.x < 16) tw[threadIdx.x] = table[threadIdx.x * 64];
  __syncthreads();
  const uint64_t p = pc.p;
  const uint32_t c = pc.c;
  const uint64_t gid = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x;
  uint64_t v[16];
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = (gid * 16 + i) % p;
  const int off = threadIdx.x & 7;
  for (int it = 0; it < kPeakIters; ++it) {
    const bool dit = it >= kPeakIters / 2;
#pragma unroll
    for (int j = 3; j >= 0; --j) {
#pragma unroll
      for (int i = 0; i < 16; ++i) {
        if (i & (1 << j)) continue;
        const ulonglong2 t = tw[((i & ((1 << j) - 1)) + off) & 15];
        const uint64_t u = v[i], x = v[i | (1 << j)];
        if (!dit) {
          v[i] = add_mod(u, x, p);
          v[i | (1 << j)] = shoup_mul(u - x + p, t.x, t.y, p, c);
        } else {
          const uint64_t uu = fold_p(u, p);
          const uint64_t y = shoup_mul(x, t.x, t.y, p, c);
          v[i] = uu + y;
          v[i | (1 << j)] = uu - y + p;
        }
      }
    }
  }
  uint64_t s = 0;
#pragma unroll
  for (int i = 0; i < 16; ++i) s ^= v[i];
  sink[gid] = s;  // keeps the network live
}

}  // namespace

int butterfly_peak(double *per_s, const PrimeConst &pc, const ulonglong2 *table) {
  int dev = 0, sms = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e != cudaSuccess) return lib_cuda_fail(e, "device query");
  const unsigned blocks = static_cast<unsigned>(sms) * 8;
  const uint64_t threads = static_cast<uint64_t>(blocks) * 256;
  uint64_t *sink = nullptr;
  cudaStream_t st = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  float best = 0;
  if ((e = cudaMalloc(&sink, threads * sizeof(uint64_t))) == cudaSuccess &&
      (e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking)) == cudaSuccess &&
      (e = cudaEventCreate(&e0)) == cudaSuccess && (e = cudaEventCreate(&e1)) == cudaSuccess) {
    for (int rep = 0; rep < 4 && e == cudaSuccess; ++rep) {
      cudaEventRecord(e0, st);
      peak_kernel<<<blocks, 256, 0, st>>>(sink, pc, table);
      cudaEventRecord(e1, st);
      e = cudaEventSynchronize(e1);
      float ms = 0;
      if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
      if (e == cudaSuccess && rep > 0 && (best == 0 || ms < best)) best = ms;  // rep 0 warms up
    }
  }
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  if (st) cudaStreamDestroy(st);
  if (sink) cudaFree(sink);
  if (e != cudaSuccess) return lib_cuda_fail(e, "butterfly peak");
  const double butterflies = static_cast<double>(threads) * kPeakIters * 4 * 8;
  *per_s = butterflies / (best / 1000.0);
  return HG_OK;
}

#if HG_CHECKED
HG_CHECKED_READER(checked_fault_peak)
#endif

}  // namespace hg
