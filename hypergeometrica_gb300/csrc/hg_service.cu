// hg_service.cu -- the device-resident multiply service (hg_svc_*).
//
// Callers (binary splitting, Newton steps) submit products whose operands and
// results already live in device memory; the service runs them on the GPU
// with continuous batching:
//   - a worker thread owns S slots, each a CUDA stream with its own workspace,
//     descriptor buffers, carry-scan state and device error word, all
//     allocated once when the service opens;
//   - pending products are admitted first in, first out into a free slot
//     while their transform workspace fits in the slot's free memory (and up
//     to max_batch products); one admitted set runs as one batch: one launch
//     per pass per transform length;
//   - products submitted while every slot is busy wait and join the next
//     batch as soon as a slot retires, so their work overlaps on the device
//     with the batches still running on the other streams;
//   - each product's latency runs from its submission to the moment the
//     worker sees its batch's completion event; p50 and p99 are reported.
// The reference multiplies one product at a time inside binary-split /
// combine (src/binary-splitting.lisp:100-133); the service changes only where
// the products run, not what they compute.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <memory>
#include <thread>

#include "hg_host.h"
#include "hypergeometrica_gb300.h"

namespace hg {
namespace {

using Clock = std::chrono::steady_clock;

constexpr int kMaxSlots = 8;
constexpr size_t kSlotTickets = 128;  // carry-scan tickets per slot (one per group)

struct SvcRequest {
  ProductDesc d;
  uint64_t ticket;
  uint64_t ws_bytes;
  Clock::time_point t_submit;
};

struct SvcSlot {
  cudaStream_t st = nullptr;
  cudaEvent_t done = nullptr;
  uint64_t *ws = nullptr;
  ProductDesc *d_desc = nullptr;
  ProductDesc *h_desc = nullptr;  // pinned staging of the descriptors
  unsigned long long *flags = nullptr;
  unsigned long long *tickets = nullptr;
  int *d_err = nullptr;
  int *h_err = nullptr;  // pinned copy of the error word after the batch
  uint64_t flag_cap = 0;
  bool busy = false;
  std::vector<SvcRequest> batch;
  BatchPlan plan;
};

}  // namespace
}  // namespace hg

struct hg_svc {
  int device = 0;
  uint64_t slot_ws_bytes = 0;
  size_t max_batch = 0;
  std::vector<hg::SvcSlot> slots;
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<hg::SvcRequest> pending;
  std::vector<int8_t> status;  // per ticket: 0 pending, 1 done, < 0 an HG_ERR_* code
  uint64_t next_ticket = 0;
  uint64_t submitted = 0, completed = 0, failed = 0, batches = 0;
  uint64_t peak_batch_bytes = 0, peak_batch_products = 0;
  std::vector<float> lat_us;  // since the last stats reset
  bool have_first = false;
  hg::Clock::time_point t_first, t_last;
  bool closing = false;
  std::thread worker;
};

namespace hg {
namespace {

void slot_free(SvcSlot &s) {
  if (s.done) cudaEventDestroy(s.done);
  if (s.st) cudaStreamDestroy(s.st);
  if (s.ws) cudaFree(s.ws);
  if (s.d_desc) cudaFree(s.d_desc);
  if (s.h_desc) cudaFreeHost(s.h_desc);
  if (s.flags) cudaFree(s.flags);
  if (s.tickets) cudaFree(s.tickets);
  if (s.d_err) cudaFree(s.d_err);
  if (s.h_err) cudaFreeHost(s.h_err);
  s = SvcSlot();
}

int slot_alloc(SvcSlot &s, uint64_t ws_bytes, size_t max_batch) {
#define SVC_CUDA(call, what)                                 \
  do {                                                       \
    cudaError_t e_ = (call);                                 \
    if (e_ != cudaSuccess) return lib_cuda_fail(e_, what);   \
  } while (0)
  SVC_CUDA(cudaStreamCreateWithFlags(&s.st, cudaStreamNonBlocking), "service stream");
  SVC_CUDA(cudaEventCreateWithFlags(&s.done, cudaEventDisableTiming), "service event");
  SVC_CUDA(cudaMalloc(&s.ws, ws_bytes), "service workspace");
  SVC_CUDA(cudaMalloc(&s.d_desc, max_batch * sizeof(ProductDesc)), "service descriptors");
  SVC_CUDA(cudaMallocHost(&s.h_desc, max_batch * sizeof(ProductDesc)), "service descriptor staging");
  // Every admitted product holds at least 3N workspace words and needs at
  // most N / 2048 + 1 flag words.
  s.flag_cap = ws_bytes / 8 / 3 / 2048 + max_batch + 64;
  SVC_CUDA(cudaMalloc(&s.flags, s.flag_cap * 8), "service scan flags");
  SVC_CUDA(cudaMalloc(&s.tickets, kSlotTickets * 8), "service scan tickets");
  SVC_CUDA(cudaMalloc(&s.d_err, sizeof(int)), "service error word");
  SVC_CUDA(cudaMemset(s.d_err, 0, sizeof(int)), "service error word");
  SVC_CUDA(cudaMallocHost(&s.h_err, sizeof(int)), "service error staging");
  *s.h_err = 0;
  return HG_OK;
#undef SVC_CUDA
}

int err_code(int dev_err) {
  if (dev_err == kDevCarryOverflow || dev_err == kDevTicket) return HG_ERR_INCONSISTENT;
  return HG_ERR_CUDA;
}

// Enqueue slot.batch on the slot's stream.  Called without the service lock.
int slot_launch(hg_svc *svc, SvcSlot &s) {
  std::vector<ProductDesc> items(s.batch.size());
  for (size_t i = 0; i < s.batch.size(); ++i) items[i] = s.batch[i].d;
  int rc = plan_batch(items.data(), items.size(), svc->slot_ws_bytes, s.plan);
  if (rc) return rc;
  if (s.plan.groups.size() > kSlotTickets || s.plan.flag_words > s.flag_cap || s.plan.desc.size() > svc->max_batch)
    return lib_fail(HG_ERR_ARG, "service batch exceeds its slot (%zu groups, %llu flag words)", s.plan.groups.size(),
                    (unsigned long long)s.plan.flag_words);
  // The pinned staging buffer is free: the slot's previous batch has retired.
  std::memcpy(s.h_desc, s.plan.desc.data(), s.plan.desc.size() * sizeof(ProductDesc));
  cudaError_t e = cudaMemcpyAsync(s.d_desc, s.h_desc, s.plan.desc.size() * sizeof(ProductDesc),
                                  cudaMemcpyHostToDevice, s.st);
  if (e != cudaSuccess) return lib_cuda_fail(e, "service descriptor upload");
  const BatchBufs bb{s.d_desc, s.ws, s.flags, s.tickets, s.d_err};
  if ((rc = enqueue_batch(s.plan, bb, s.st))) return rc;
  if ((e = cudaMemcpyAsync(s.h_err, s.d_err, sizeof(int), cudaMemcpyDeviceToHost, s.st)) != cudaSuccess ||
      (e = cudaMemsetAsync(s.d_err, 0, sizeof(int), s.st)) != cudaSuccess ||
      (e = cudaEventRecord(s.done, s.st)) != cudaSuccess)
    return lib_cuda_fail(e, "service batch completion");
  return HG_OK;
}

// Mark every request of a batch with its outcome.  Called with the lock held.
void settle(hg_svc *svc, std::vector<SvcRequest> &batch, int code, Clock::time_point now) {
  for (const SvcRequest &r : batch) {
    svc->status[r.ticket] = static_cast<int8_t>(code == HG_OK ? 1 : code);
    if (code == HG_OK) {
      ++svc->completed;
      svc->lat_us.push_back(std::chrono::duration<float, std::micro>(now - r.t_submit).count());
    } else {
      ++svc->failed;
    }
  }
  svc->t_last = now;
  batch.clear();
}

void worker_loop(hg_svc *svc) {
  cudaSetDevice(svc->device);
  std::unique_lock<std::mutex> lk(svc->mu);
  for (;;) {
    bool busy = false;
    for (SvcSlot &s : svc->slots) {
      if (!s.busy) continue;
      const cudaError_t q = cudaEventQuery(s.done);
      if (q == cudaErrorNotReady) {
        busy = true;
        continue;
      }
      int code = HG_OK;
      if (q != cudaSuccess) code = HG_ERR_CUDA;
      else if (*s.h_err) code = err_code(*s.h_err);
      *s.h_err = 0;
      s.busy = false;
      settle(svc, s.batch, code, Clock::now());
      svc->cv_done.notify_all();
    }
    SvcSlot *slot = nullptr;
    for (SvcSlot &s : svc->slots)
      if (!s.busy) {
        slot = &s;
        break;
      }
    if (slot && !svc->pending.empty()) {
      uint64_t used = 0;
      while (!svc->pending.empty() && slot->batch.size() < svc->max_batch) {
        const SvcRequest &r = svc->pending.front();
        if (!slot->batch.empty() && used + r.ws_bytes > svc->slot_ws_bytes) break;
        used += r.ws_bytes;
        slot->batch.push_back(r);
        svc->pending.pop_front();
      }
      svc->peak_batch_bytes = std::max(svc->peak_batch_bytes, used);
      svc->peak_batch_products = std::max<uint64_t>(svc->peak_batch_products, slot->batch.size());
      lk.unlock();
      const int rc = slot_launch(svc, *slot);
      lk.lock();
      if (rc) {
        cudaStreamSynchronize(slot->st);
        settle(svc, slot->batch, rc, Clock::now());
        svc->cv_done.notify_all();
      } else {
        slot->busy = true;
        ++svc->batches;
      }
      continue;
    }
    if (svc->closing && svc->pending.empty() && !busy) break;
    if (busy)
      svc->cv_work.wait_for(lk, std::chrono::microseconds(20));
    else
      svc->cv_work.wait(lk, [&] { return svc->closing || !svc->pending.empty(); });
  }
}

}  // namespace
}  // namespace hg

using namespace hg;

extern "C" {

int hg_svc_open(size_t workspace_bytes, int slots, size_t max_batch, hg_svc **out) {
  if (!out) return lib_fail(HG_ERR_ARG, "null pointer");
  *out = nullptr;
  std::lock_guard<std::recursive_mutex> lock(lib_mutex());
  if (!lib_ready()) return lib_fail(HG_ERR_NOT_INIT, "hg_svc_open: call hg_init first");
  if (slots < 1 || slots > kMaxSlots) return lib_fail(HG_ERR_ARG, "slots = %d, expected 1..%d", slots, kMaxSlots);
  if (max_batch == 0) max_batch = size_t(1) << 20;
  if (workspace_bytes == 0) {
    size_t free_b = 0, total_b = 0;
    cudaError_t e = cudaMemGetInfo(&free_b, &total_b);
    if (e != cudaSuccess) return lib_cuda_fail(e, "free memory query");
    workspace_bytes = std::min<size_t>(free_b / 2, size_t(8) << 30);
  }
  const uint64_t per_slot = (workspace_bytes / static_cast<size_t>(slots)) & ~uint64_t(255);
  if (per_slot < 4096)
    return lib_fail(HG_ERR_ARG, "workspace of %zu bytes is too small for %d slots", workspace_bytes, slots);
  std::unique_ptr<hg_svc> svc(new hg_svc());
  svc->device = lib_device();
  svc->slot_ws_bytes = per_slot;
  svc->max_batch = max_batch;
  svc->slots.resize(static_cast<size_t>(slots));
  for (SvcSlot &s : svc->slots) {
    int rc = slot_alloc(s, per_slot, max_batch);
    if (rc) {
      for (SvcSlot &t : svc->slots) slot_free(t);
      return rc;
    }
  }
  lib_service_count(1);
  hg_svc *p = svc.release();
  p->worker = std::thread(worker_loop, p);
  *out = p;
  return HG_OK;
}

int hg_svc_submit(hg_svc *svc, const hg_product *prods, size_t n, uint64_t *first_ticket) {
  if (!svc || (n && !prods)) return lib_fail(HG_ERR_ARG, "null pointer");
  std::vector<SvcRequest> reqs(n);
  for (size_t i = 0; i < n; ++i) {
    const hg_product &p = prods[i];
    const bool square = p.y == nullptr;
    const uint64_t size = square ? 2 * p.nx : p.nx + p.ny;
    if (!p.out || (p.nx && !p.x)) return lib_fail(HG_ERR_ARG, "product %zu: null pointer", i);
    if (p.nout < size)
      return lib_fail(HG_ERR_ARG, "product %zu: nout = %zu cannot hold %llu limbs", i, p.nout,
                      (unsigned long long)size);
    if (size > (uint64_t(1) << kLogNmax))
      return lib_fail(HG_ERR_ARG, "product %zu: %llu limbs exceed the 2^%d transform limit", i,
                      (unsigned long long)size, kLogNmax);
    const uint64_t ws = product_workspace_bytes(p.nx, square ? p.nx : p.ny, square);
    if (ws > svc->slot_ws_bytes)
      return lib_fail(HG_ERR_ARG, "product %zu needs %llu workspace bytes; a slot of this service holds %llu", i,
                      (unsigned long long)ws, (unsigned long long)svc->slot_ws_bytes);
    reqs[i].d = ProductDesc{p.x, p.y, p.nx, square ? p.nx : p.ny, p.out, p.nout};
    reqs[i].ws_bytes = ws;
  }
  const Clock::time_point now = Clock::now();
  {
    std::lock_guard<std::mutex> lk(svc->mu);
    if (svc->closing) return lib_fail(HG_ERR_ARG, "service is closing");
    if (first_ticket) *first_ticket = svc->next_ticket;
    if (!svc->have_first) {
      svc->have_first = true;
      svc->t_first = now;
    }
    svc->status.resize(svc->next_ticket + n, 0);
    for (SvcRequest &r : reqs) {
      r.ticket = svc->next_ticket++;
      r.t_submit = now;
      svc->pending.push_back(r);
    }
    svc->submitted += n;
  }
  svc->cv_work.notify_one();
  return HG_OK;
}

int hg_svc_status(hg_svc *svc, uint64_t ticket) {
  if (!svc) return lib_fail(HG_ERR_ARG, "null pointer");
  std::lock_guard<std::mutex> lk(svc->mu);
  if (ticket >= svc->next_ticket) return lib_fail(HG_ERR_ARG, "unknown ticket %llu", (unsigned long long)ticket);
  return svc->status[ticket];
}

int hg_svc_wait(hg_svc *svc, uint64_t ticket, double timeout_s) {
  if (!svc) return lib_fail(HG_ERR_ARG, "null pointer");
  std::unique_lock<std::mutex> lk(svc->mu);
  if (ticket >= svc->next_ticket) return lib_fail(HG_ERR_ARG, "unknown ticket %llu", (unsigned long long)ticket);
  const auto pred = [&] { return svc->status[ticket] != 0; };
  if (timeout_s < 0)
    svc->cv_done.wait(lk, pred);
  else if (!svc->cv_done.wait_for(lk, std::chrono::duration<double>(timeout_s), pred))
    return lib_fail(HG_ERR_TIMEOUT, "product %llu not finished within %.3f s", (unsigned long long)ticket, timeout_s);
  const int st = svc->status[ticket];
  return st == 1 ? HG_OK : lib_fail(st, "product %llu failed on the device", (unsigned long long)ticket);
}

int hg_svc_wait_all(hg_svc *svc, double timeout_s) {
  if (!svc) return lib_fail(HG_ERR_ARG, "null pointer");
  std::unique_lock<std::mutex> lk(svc->mu);
  const auto pred = [&] { return svc->completed + svc->failed == svc->submitted; };
  if (timeout_s < 0)
    svc->cv_done.wait(lk, pred);
  else if (!svc->cv_done.wait_for(lk, std::chrono::duration<double>(timeout_s), pred))
    return lib_fail(HG_ERR_TIMEOUT, "%llu products not finished within %.3f s",
                    (unsigned long long)(svc->submitted - svc->completed - svc->failed), timeout_s);
  return svc->failed ? lib_fail(HG_ERR_CUDA, "%llu products failed", (unsigned long long)svc->failed) : HG_OK;
}

int hg_svc_stats(hg_svc *svc, hg_svc_report *out, int reset) {
  if (!svc || !out) return lib_fail(HG_ERR_ARG, "null pointer");
  std::lock_guard<std::mutex> lk(svc->mu);
  std::memset(out, 0, sizeof *out);
  out->submitted = svc->submitted;
  out->completed = svc->completed;
  out->failed = svc->failed;
  out->batches = svc->batches;
  out->pending = svc->pending.size();
  uint64_t in_flight = 0;
  for (const SvcSlot &s : svc->slots) in_flight += s.batch.size();
  out->in_flight = in_flight;
  out->peak_batch_products = svc->peak_batch_products;
  out->peak_batch_workspace_bytes = svc->peak_batch_bytes;
  out->slot_workspace_bytes = svc->slot_ws_bytes;
  out->slots = static_cast<int>(svc->slots.size());
  std::vector<float> &l = svc->lat_us;
  out->latency_samples = l.size();
  if (!l.empty()) {
    std::vector<float> v(l);
    auto q = [&](double f) {
      const size_t k = std::min(v.size() - 1, static_cast<size_t>(f * static_cast<double>(v.size())));
      std::nth_element(v.begin(), v.begin() + static_cast<std::ptrdiff_t>(k), v.end());
      return static_cast<double>(v[k]);
    };
    out->p50_us = q(0.50);
    out->p99_us = q(0.99);
    double sum = 0, mx = 0;
    for (float x : l) {
      sum += x;
      mx = std::max<double>(mx, x);
    }
    out->mean_us = sum / static_cast<double>(l.size());
    out->max_us = mx;
    const double span = std::chrono::duration<double>(svc->t_last - svc->t_first).count();
    out->products_per_s = span > 0 ? static_cast<double>(l.size()) / span : 0.0;
  }
  if (reset) {
    l.clear();
    svc->have_first = false;
    svc->peak_batch_bytes = svc->peak_batch_products = 0;
  }
  return HG_OK;
}

int hg_svc_close(hg_svc *svc) {
  if (!svc) return HG_OK;
  {
    std::lock_guard<std::mutex> lk(svc->mu);
    svc->closing = true;
  }
  svc->cv_work.notify_all();
  if (svc->worker.joinable()) svc->worker.join();
  int rc = HG_OK;
  for (SvcSlot &s : svc->slots) {
    if (s.st && cudaStreamSynchronize(s.st) != cudaSuccess) rc = lib_fail(HG_ERR_CUDA, "service stream failed");
    slot_free(s);
  }
  delete svc;
  lib_service_count(-1);
  return rc;
}

}  // extern "C"
