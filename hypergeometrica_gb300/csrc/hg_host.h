// hg_host.h -- host-side pieces of the library shared between hg_api.cu
// (the C ABI, the context, single and batched products) and hg_service.cu
// (the device-resident multiply service).
#pragma once

#include <cstdint>
#include <mutex>
#include <vector>

#include "hg_internal.h"

namespace hg {

// One pass of a transform plan: logR row bits, stride 2^logS, 2^logT-word tiles.
struct PassPlan {
  int logR, logS, logT;
};

// Products of one transform length and kind, run as one launch per pass.
struct BatchGroup {
  int L = 0;
  bool square = false;
  bool tails = false;              // some product has nout > N
  std::vector<PassPlan> plan;
  uint64_t first = 0, nprod = 0;   // descriptors [first, first + nprod)
  uint64_t flags_off = 0;          // first carry-scan flag word
};

// A planned batch: groups contiguous in desc, then the products with an empty
// operand (zeroed, no transform).  Groups run one after another and share
// one workspace of ws_words words.
struct BatchPlan {
  std::vector<BatchGroup> groups;
  std::vector<ProductDesc> desc;
  uint64_t zero_first = 0, nzero = 0;
  uint64_t ws_words = 0, flag_words = 0;
};

// Device buffers a planned batch runs in.
struct BatchBufs {
  const ProductDesc *desc;    // device copy of BatchPlan::desc
  uint64_t *ws;               // ws_words words
  unsigned long long *flags;  // flag_words words
  unsigned long long *tickets;  // one per group
  int *err;                   // device error word
};

// Workspace bytes one product occupies while its group runs.
uint64_t product_workspace_bytes(uint64_t nx, uint64_t ny, bool square);

// Group validated descriptors by (transform length, square) and split groups
// so that none needs more than ws_cap_bytes of workspace.
int plan_batch(const ProductDesc *items, size_t n, uint64_t ws_cap_bytes, BatchPlan &bp);

// sa |a| + sb |b| into out[0, nout) over the whole GPU (nout >= max(na,
// nb) + 1; limbs past the sum are zeroed); (sign, size) into result[0, 2)
// on the device.  Uses the library's carry-scan state, ordered like the
// products' workspace.
int large_sum_device(const uint64_t *a, uint64_t na, int64_t sa, const uint64_t *b, uint64_t nb, int64_t sb,
                     uint64_t *out, uint64_t nout, int64_t *result, cudaStream_t st);

// Enqueue a planned batch on st: clear its scan state, zero the empty
// products, run every group.  Takes no lock and allocates nothing.
int enqueue_batch(const BatchPlan &bp, const BatchBufs &bb, cudaStream_t st);

// The library's state, for code outside hg_api.cu.
std::recursive_mutex &lib_mutex();
bool lib_ready();
int lib_device();
// Record an error message (hg_last_error) and return code.
int lib_fail(int code, const char *fmt, ...);
int lib_cuda_fail(cudaError_t e, const char *what);
// Count of open services; hg_shutdown refuses while it is nonzero.
void lib_service_count(int delta);

// Butterflies per second of a memory-free network of the library's modular
// butterflies (hg_peak.cu), with prime pc and a device table of at least
// 1024 (twiddle, companion) pairs.
int butterfly_peak(double *per_s, const PrimeConst &pc, const ulonglong2 *table);

}  // namespace hg
