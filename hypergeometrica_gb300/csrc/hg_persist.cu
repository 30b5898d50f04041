// hg_persist.cu -- a batch of products in one persistent launch.
//
// Binary splitting multiplies thousands of independent pairs of uneven
// sizes per tree level (combine, src/binary-splitting.lisp:112-121).  The
// per-pass schedule runs each group of one transform length as one launch
// per pass; this kernel runs the whole batch as one launch instead.  The
// host lays the batch out as a work list of phases -- for each group its
// forward passes, the middle (or the whole single-pass product), its
// inverse passes, the reconstruction and the carry fix, and the zeroing of
// result tails -- each phase a range of items, an item being one CTA's
// share of the per-pass launch it replaces (one tile, one block, one carry
// tile).  Phases are listed level by level across groups (every group's
// first phase, then every group's second, ...), so groups of different
// lengths overlap on the GPU.
//
// A fixed grid of CTAs claims items in list order from one atomic counter;
// an item is one or more consecutive CTAs' shares, so that the claim, the
// phase lookup and the completion count are paid once per several tiles.
// An item whose phase depends on an earlier phase of its group waits until
// that phase has counted all its items done.  The wait cannot deadlock: a
// phase's items all come earlier in the list than those of the phases that
// wait for it, and only running CTAs claim items, so every item a CTA waits
// for has been claimed by a running CTA that does not wait for it in turn.
// Every wait is bounded: one that runs out sets the batch's abort word and
// latches an error, and every CTA stops claiming.
//
// Items run the same bodies as the per-pass kernels (hg_ntt_bodies.cuh,
// hg_carry.cuh): the product is the same integer, limb for limb.  Residues
// written by one phase are read by another CTA in a later phase; the
// acquire load of the dependency counter and the CTA barrier after it order
// those reads after the writes.
#include "hg_carry.cuh"
#include "hg_host.h"
#include "hg_ntt_bodies.cuh"

namespace hg {
namespace {

using namespace rounds;
using namespace bodies;

constexpr int kPersistThreads = 256;
constexpr int kPersistCarryTile = kPersistThreads * carry::kCarryPer;

__device__ __forceinline__ unsigned ld_acquire(const unsigned *p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

// Each kind of item is a separate (not inlined) function, so that ptxas
// allocates registers per body rather than across all of them at once.
template <int LOGR, bool INV>
__device__ __noinline__ void run_strided_dir(const PassArgs &P, uint64_t item, ulonglong2 *tw, uint64_t *sm) {
  strided_ldg_body<LOGR, INV>(P, item, tw, sm);
}

template <int LOGR>
__device__ __forceinline__ void run_strided(const PassArgs &P, bool inv, uint64_t item, ulonglong2 *tw,
                                            uint64_t *sm) {
  if (inv)
    run_strided_dir<LOGR, true>(P, item, tw, sm);
  else
    run_strided_dir<LOGR, false>(P, item, tw, sm);
}

template <int T, int MODE>
__device__ __noinline__ void run_contig_mode(const PassArgs &P, uint64_t bx, int by, uint64_t *sm) {
  contig_body<T, MODE>(P, bx, by, sm);
}

template <int T>
__device__ __forceinline__ void run_contig(const PassArgs &P, int mode, uint64_t bx, int by, uint64_t *sm) {
  if (mode == kMul)
    run_contig_mode<T, kMul>(P, bx, by, sm);
  else
    run_contig_mode<T, kSqr>(P, bx, by, sm);
}

__device__ __noinline__ void run_tiny(const PersistPhase &ph, uint64_t item) {
  const uint64_t pair = item * kPersistThreads + threadIdx.x;
  if (pair < ph.a.nprod * static_cast<uint64_t>(ph.a.nprimes))
    tiny_body(ph.a, ph.sel, pair / ph.a.nprimes, static_cast<int>(pair % ph.a.nprimes));
}

// Residues prescaled (the group's last inverse pass read its scaled table)
// or not: each reconstruction has its own body.
template <bool PRESCALED>
__device__ __noinline__ void run_carry_t(const PersistPhase &ph, uint64_t item, uint64_t *dyn, GP *s_warp) {
  using Producer = carry::CrtProducerT<true, PRESCALED>;
  carry::carry_body<Producer, kPersistThreads>(Producer{ph.res, ph.n, ph.cc}, nullptr, 0, ph.ss, ph.batch, ph.tpp,
                                               ph.ws_stride, ph.n, item, reinterpret_cast<uint64_t(*)[9]>(dyn),
                                               s_warp);
}

__device__ __forceinline__ void run_carry(const PersistPhase &ph, uint64_t item, uint64_t *dyn, GP *s_warp) {
  if (ph.cc.prescaled)
    run_carry_t<true>(ph, item, dyn, s_warp);
  else
    run_carry_t<false>(ph, item, dyn, s_warp);
}

__device__ __noinline__ void run_fix(const PersistPhase &ph, uint64_t item) {
  carry::fix_body<kPersistCarryTile>(nullptr, 0, ph.tiles, ph.ss, false, ph.batch, ph.tpp, ph.n,
                                     item * (kPersistThreads / 32) + (threadIdx.x >> 5));
}

// out[n, nout) of product `item` (out[0, nout) when n == 0).
__device__ __noinline__ void run_zero(const PersistPhase &ph, uint64_t item) {
  const ProductDesc d = ph.batch[item];
  for (uint64_t i = ph.n + threadIdx.x; i < d.nout; i += kPersistThreads) d.out[i] = 0;
}

__device__ __forceinline__ void run_item(const PersistPhase &ph, uint64_t item, uint64_t *dyn, ulonglong2 *tw,
                                         GP *s_warp) {
  switch (ph.kind) {
    case kPhaseStrided: {
      const bool inv = (ph.sel >> 4) & 1;
      switch (ph.sel & 15) {
        case 4: run_strided<4>(ph.a, inv, item, tw, dyn); break;
        case 5: run_strided<5>(ph.a, inv, item, tw, dyn); break;
        case 6: run_strided<6>(ph.a, inv, item, tw, dyn); break;
        case 7: run_strided<7>(ph.a, inv, item, tw, dyn); break;
        case 8: run_strided<8>(ph.a, inv, item, tw, dyn); break;
        default: break;
      }
      break;
    }
    case kPhaseContig: {
      const int mode = ph.sel >> 4;
      const uint64_t bx = item % ph.gx;
      const int by = static_cast<int>(item / ph.gx);
      switch (ph.sel & 15) {
        case 4: run_contig<4>(ph.a, mode, bx, by, dyn); break;
        case 5: run_contig<5>(ph.a, mode, bx, by, dyn); break;
        case 6: run_contig<6>(ph.a, mode, bx, by, dyn); break;
        case 7: run_contig<7>(ph.a, mode, bx, by, dyn); break;
        case 8: run_contig<8>(ph.a, mode, bx, by, dyn); break;
        case 9: run_contig<9>(ph.a, mode, bx, by, dyn); break;
        case 10: run_contig<10>(ph.a, mode, bx, by, dyn); break;
        case 11: run_contig<11>(ph.a, mode, bx, by, dyn); break;
        case 12: run_contig<12>(ph.a, mode, bx, by, dyn); break;
        default: break;
      }
      break;
    }
    case kPhaseTiny: run_tiny(ph, item); break;
    case kPhaseCarry: run_carry(ph, item, dyn, s_warp); break;
    case kPhaseFix: run_fix(ph, item); break;
    case kPhaseZero: run_zero(ph, item); break;
    default: break;
  }
}

// Two CTAs of 256 threads per SM: 128 registers, so that the 9..11-bit
// middle blocks do not spill, and 64 KB of shared memory for a middle block
// of two operands.
__global__ void __launch_bounds__(kPersistThreads, 2)
    persist_kernel(const PersistPhase *__restrict__ phases, int nphases, uint64_t total, PersistState *state,
                   int *err) {
  extern __shared__ __align__(16) uint64_t dyn[];
  __shared__ ulonglong2 s_tw[128];
  __shared__ GP s_warp[kPersistThreads / 32];
  __shared__ uint64_t s_first[kPersistMaxPhases + 1];
  __shared__ PersistPhase s_ph;
  __shared__ uint64_t s_item;
  __shared__ int s_idx, s_stop, s_new;
  const int tid = threadIdx.x;
  for (int i = tid; i < nphases; i += kPersistThreads) s_first[i] = phases[i].first;
  if (tid == 0) {
    s_first[nphases] = total;
    s_idx = -1;
  }
  for (;;) {
    __syncthreads();  // every thread is done with the previous item and its shared memory
    if (tid == 0) {
      const volatile unsigned *abort = &state->abort;
      uint64_t it = total;
      if (!*abort) it = atomicAdd(&state->next, 1ull);
      s_item = it;
      int ph = -1;
      if (it < total) {
        int lo = 0, hi = nphases - 1;  // the last phase whose first item is <= it
        while (lo < hi) {
          const int mid = (lo + hi + 1) >> 1;
          if (s_first[mid] <= it) lo = mid;
          else hi = mid - 1;
        }
        ph = lo;
      }
      s_stop = ph < 0;
      s_new = ph != s_idx;
      if (ph >= 0 && ph != s_idx) {
        // A new phase for this CTA: wait, once, until the phase it depends on is complete.
        const int dep = phases[ph].dep;
        if (dep >= 0) {
          const uint64_t need = phases[dep].count;
          const long long t0 = clock64();
          while (ld_acquire(&state->done[dep]) < need) {
            if (*abort || clock64() - t0 > (1ll << 32)) {
              if (!*abort) {
                atomicExch(&state->abort, 1u);
                latch_error(err, kDevQueueTimeout);
              }
              s_stop = 1;
              break;
            }
            __nanosleep(256);
          }
          __threadfence();
        }
      }
      s_idx = ph;
    }
    __syncthreads();
    if (s_stop) break;
    const uint64_t item = s_item;
    const int ph = s_idx;
    if (s_new) {  // the phase's descriptor, into shared memory when the CTA enters the phase
      const uint64_t *src = reinterpret_cast<const uint64_t *>(phases + ph);
      uint64_t *dst = reinterpret_cast<uint64_t *>(&s_ph);
      for (int w = tid; w < static_cast<int>(sizeof(PersistPhase) / 8); w += kPersistThreads) dst[w] = src[w];
      __syncthreads();
    }
    {
      const uint64_t u0 = (item - s_ph.first) * s_ph.per;
      const uint64_t u1 = u0 + s_ph.per < s_ph.units ? u0 + s_ph.per : s_ph.units;
      for (uint64_t u = u0; u < u1; ++u) {
        if (u != u0) __syncthreads();  // the unit before is done with shared memory
        run_item(s_ph, u, dyn, s_tw, s_warp);
      }
    }
    __syncthreads();
    if (tid == 0) {
      __threadfence();
      atomicAdd(&state->done[ph], 1u);
    }
  }
}

}  // namespace

static_assert(sizeof(PersistPhase) % 8 == 0, "phase descriptors are copied as 8-byte words");

int persist_grid() {
  static int grid = 0;
  if (!grid) {
    int dev = 0, sms = 0, per = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
        cudaFuncSetAttribute(persist_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             static_cast<int>(kPersistSmemBytes)) != cudaSuccess ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, persist_kernel, kPersistThreads, kPersistSmemBytes) !=
            cudaSuccess ||
        per < 1) {
      cudaGetLastError();
      return 0;
    }
    grid = sms * per;
  }
  return grid;
}

uint64_t persist_carry_tiles(uint64_t n) { return (n + kPersistCarryTile - 1) / kPersistCarryTile; }

cudaError_t launch_persist(const PersistPhase *phases, int nphases, uint64_t total, PersistState *state, int *err,
                           cudaStream_t st) {
  if (nphases < 1 || nphases > kPersistMaxPhases || total == 0) return cudaErrorInvalidValue;
  const int grid = persist_grid();
  if (!grid) return cudaErrorInvalidConfiguration;
  cudaError_t e = cudaMemsetAsync(state, 0, persist_state_bytes(nphases), st);
  if (e != cudaSuccess) return e;
  const unsigned g = static_cast<unsigned>(total < static_cast<uint64_t>(grid) ? total : grid);
  persist_kernel<<<g, kPersistThreads, kPersistSmemBytes, st>>>(phases, nphases, total, state, err);
  return cudaGetLastError();
}

#if HG_CHECKED
HG_CHECKED_READER(checked_fault_persist)
#endif

}  // namespace hg
