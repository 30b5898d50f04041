// hg_api.cu -- host driver behind the C ABI (include/hypergeometrica_gb300.h).
//
// Owns the library context: the scheme (moduli and generators, rebuilt here
// exactly as make-modular-scheme / default-moduli build them,
// src/moduli.lisp:173-191, 257-353), the device twiddle tables, a grow-only
// device workspace, the carry-scan state and the device error word.  Plans
// the NTT passes for a transform length and enqueues the kernels of one
// product: forward passes (the first reads the limbs and reduces them),
// pointwise product, inverse passes, reconstruction + carry.
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <algorithm>
#include <atomic>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <tuple>
#include <vector>

#include "hg_host.h"
#include "hypergeometrica_gb300.h"

namespace hg {
namespace {

using u128 = unsigned __int128;

// ---- host modular arithmetic -------------------------------------------
uint64_t mulmod_h(uint64_t a, uint64_t b, uint64_t m) { return static_cast<uint64_t>((u128)a * b % m); }
uint64_t powmod_h(uint64_t a, uint64_t e, uint64_t m) {
  uint64_t r = 1 % m;
  a %= m;
  while (e) {
    if (e & 1) r = mulmod_h(r, a, m);
    a = mulmod_h(a, a, m);
    e >>= 1;
  }
  return r;
}
uint64_t invmod_h(uint64_t x, uint64_t m) { return powmod_h(x % m, m - 2, m); }  // m prime
uint64_t mont_h(uint64_t x, uint64_t m) { return static_cast<uint64_t>(((u128)(x % m) << 64) % m); }

bool isprime_h(uint64_t n) {
  if (n < 2) return false;
  static const uint64_t bases[] = {2, 3, 5, 7, 11, 13, 17, 19, 23, 29, 31, 37};
  for (uint64_t b : bases)
    if (n % b == 0) return n == b;
  uint64_t d = n - 1;
  int s = 0;
  while (!(d & 1)) {
    d >>= 1;
    ++s;
  }
  for (uint64_t b : bases) {
    uint64_t x = powmod_h(b, d, n);
    if (x == 1 || x == n - 1) continue;
    bool comp = true;
    for (int r = 1; r < s && comp; ++r) {
      x = mulmod_h(x, x, n);
      if (x == n - 1) comp = false;
    }
    if (comp) return false;
  }
  return true;
}

// find-finite-field-generator (src/moduli.lisp:173-179): smallest prime g
// with g^((m-1)/f) != 1 for each prime factor f of m - 1.
uint64_t generator_h(uint64_t m) {
  std::vector<uint64_t> f;
  uint64_t n = m - 1;
  for (uint64_t q = 2; q * q <= n; ++q)
    if (n % q == 0) {
      f.push_back(q);
      while (n % q == 0) n /= q;
    }
  if (n > 1) f.push_back(n);
  for (uint64_t g = 2;; ++g) {
    if (!isprime_h(g)) continue;
    bool ok = true;
    for (uint64_t q : f)
      if (powmod_h(g, (m - 1) / q, m) == 1) ok = false;
    if (ok) return g;
  }
}

// default-moduli (src/moduli.lisp:257-264): primes c*2^55 + 1 of integer
// length 63, largest first.
std::vector<uint64_t> default_moduli_h() {
  std::vector<uint64_t> v;
  for (uint64_t c = 255; c >= 128; --c) {
    const uint64_t p = (c << kShift) + 1;
    if (isprime_h(p)) v.push_back(p);
  }
  return v;
}

// ---- context -----------------------------------------------------------
struct DevBuf {
  void *p = nullptr;
  size_t bytes = 0;
  cudaError_t ensure(size_t b) {
    if (b <= bytes) return cudaSuccess;
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
    cudaError_t e = cudaMalloc(&p, b);
    if (e == cudaSuccess) bytes = b;
    return e;
  }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
  }
  uint64_t *u64() const { return static_cast<uint64_t *>(p); }
};

// Column slices of an operand upload from host memory (ntt_product_device).
constexpr int kUploadSlices = 4;

// The streams, workspace and carry-scan state one product at a time runs
// in.  Every entry point uses lane 0; hg_mul_host_pipeline alternates
// between the lanes so that one product's download and the next one's
// upload and transforms overlap.
struct Lane {
  cudaStream_t stream = nullptr;
  DevBuf A, B, X, Y, OUT, flags;
  DevBuf misc;  // bytes [0, 8) carry-scan ticket, [8, 12) error word (lane 0's is the library's), [16, 24) large-sum top index
  unsigned long long ticket_count = 0;
  uint32_t epoch = 0;
  cudaEvent_t ws_done = nullptr;
  cudaStream_t copy_stream = nullptr;  // host entry points: operand uploads
  cudaEvent_t copy_done = nullptr;
  cudaEvent_t slice_done[2][kUploadSlices] = {};  // per operand, per column slice of the upload
  bool ws_pending = false;
  cudaStream_t d2h_stream = nullptr;  // hg_mul_host_pipeline: product downloads
  cudaEvent_t carry_done = nullptr, d2h_done = nullptr;
  bool d2h_pending = false;
};
constexpr int kLanes = 2;

struct Context {
  bool ready = false;
  int device = 0;
  uint64_t moduli[kPrimes] = {};
  uint64_t gens[kPrimes] = {};
  PrimeConst pc[kPrimes] = {};
  NttTables tb[kPrimes] = {};
  DevBuf tables;
  Lane lanes[kLanes];
  Lane *lane = &lanes[0];  // the lane products are enqueued in
  std::recursive_mutex mu;
};

Context g_ctx;

// The library's device error word (lane 0's); every lane's kernels latch here.
int *err_word() { return reinterpret_cast<int *>(static_cast<char *>(g_ctx.lanes[0].misc.p) + 8); }
thread_local std::string t_err;

// ---- instrumentation: launch counters and optional event timing ---------
struct ProfRecord {
  int cls;
  cudaEvent_t b, e;
};
struct Profile {
  std::mutex mu;
  bool on = false;
  uint64_t launches[HG_KC_COUNT] = {};
  double bytes[HG_KC_COUNT] = {};
  std::vector<ProfRecord> recs;
};
Profile g_prof;

// Counts `launches` kernel launches of class `cls` moving `bytes` algorithmic
// bytes, bracketed by a CUDA event pair on `st` while recording is on.
class ProfScope {
 public:
  ProfScope(int cls, cudaStream_t st, double bytes, int launches = 1) : cls_(cls), st_(st) {
    std::lock_guard<std::mutex> lk(g_prof.mu);
    g_prof.launches[cls] += launches;
    g_prof.bytes[cls] += bytes;
    if (g_prof.on && cudaEventCreate(&b_) == cudaSuccess) cudaEventRecord(b_, st_);
  }
  ~ProfScope() {
    if (!b_) return;
    cudaEvent_t e = nullptr;
    if (cudaEventCreate(&e) == cudaSuccess) {
      cudaEventRecord(e, st_);
      std::lock_guard<std::mutex> lk(g_prof.mu);
      g_prof.recs.push_back({cls_, b_, e});
    } else {
      cudaEventDestroy(b_);
    }
  }

 private:
  int cls_;
  cudaStream_t st_;
  cudaEvent_t b_ = nullptr;
};

int fail(int code, const char *fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  t_err = buf;
  return code;
}

int cuda_fail(cudaError_t e, const char *what) {
  if (e == cudaErrorMemoryAllocation) return fail(HG_ERR_OOM, "%s: %s", what, cudaGetErrorString(e));
  return fail(HG_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

#define HG_CUDA(call, what)                   \
  do {                                        \
    cudaError_t e_ = (call);                  \
    if (e_ != cudaSuccess) return cuda_fail(e_, what); \
  } while (0)

constexpr size_t kSubEntries = 2048;           // (w, companion) pairs per direction
constexpr size_t kSubWords = 2 * kSubEntries;  // words per direction
constexpr size_t kLevelWords = size_t(1) << kTwLevelBits;
constexpr size_t kSwzWords = 2 * 2 * kTwInverse;  // both directions, (w, companion) pairs
constexpr size_t kPrimeTableWords = 2 * kSubWords + 4 * kLevelWords + kSwzWords;

// Shoup companion floor(w * 2^64 / p) (calc-b-inv, src/modular-arithmetic.lisp:207-208).
uint64_t shoup_h(uint64_t w, uint64_t p) { return static_cast<uint64_t>(((u128)w << 64) / p); }

// Largest transform the reference's scheme supports for these moduli
// (max-transform-length-bits, src/moduli.lisp:266-267): every p - 1 is
// divisible by 2^55.
constexpr int kSchemeMaxLg = 55;

// A caller's table of primitive roots against the library's: roots[i *
// (maxlg + 1) + q] must be w_{2^q} for moduli[i], the root the scheme's
// table holds at [q][i][0][0] (find-primitive-root of 2^q, the generator
// raised to (m - 1) / 2^q, src/moduli.lisp:181-191, 318-332).  For q <= 30
// the library's device tables are built from w_{2^30}, so the expected root
// is w_{2^30}^(2^(30 - q)), the very value they use; above 30 it is the
// generator's power.
int check_roots(const uint64_t *moduli, int k, const uint64_t *roots, int maxlg) {
  if (!roots) return HG_OK;
  if (!moduli || k <= 0) return fail(HG_ERR_NOT_INIT, "a roots table needs the moduli it belongs to");
  if (maxlg < 0 || maxlg > kSchemeMaxLg)
    return fail(HG_ERR_NOT_INIT, "roots table of 2^0 .. 2^%d: the scheme's transforms stop at 2^%d", maxlg,
                kSchemeMaxLg);
  for (int i = 0; i < k; ++i) {
    const uint64_t m = moduli[i];
    const uint64_t g = generator_h(m);
    const uint64_t w30 = powmod_h(g, (m - 1) >> kLogNmax, m);
    for (int q = 0; q <= maxlg; ++q) {
      const uint64_t want = q <= kLogNmax ? powmod_h(w30, uint64_t(1) << (kLogNmax - q), m)
                                          : powmod_h(g, (m - 1) >> q, m);
      const uint64_t got = roots[static_cast<size_t>(i) * (maxlg + 1) + q];
      if (got != want)
        return fail(HG_ERR_NOT_INIT,
                    "primitive 2^%d-th root of unity for modulus %d (0x%llx) is 0x%llx in the caller's scheme, 0x%llx "
                    "in the library's tables",
                    q, i, (unsigned long long)m, (unsigned long long)got, (unsigned long long)want);
    }
  }
  return HG_OK;
}

int init_locked(const uint64_t *moduli, int k, const uint64_t *roots, int maxlg, int device) {
  Context &c = g_ctx;
  std::vector<uint64_t> dm = default_moduli_h();
  if (dm.size() != kPrimes) return fail(HG_ERR_NOT_INIT, "expected %d default moduli, found %zu", kPrimes, dm.size());
  if (moduli && k > 0) {
    std::vector<uint64_t> given(moduli, moduli + k);
    std::sort(given.begin(), given.end(), [](uint64_t a, uint64_t b) { return a > b; });
    if (given != dm)
      return fail(HG_ERR_NOT_INIT, "moduli differ from the scheme this library implements (default-moduli)");
  }
  int rc = check_roots(moduli, k, roots, maxlg);
  if (rc) return rc;
  if (c.ready) {
    if (device >= 0 && device != c.device)
      return fail(HG_ERR_ARG, "library already initialised on device %d", c.device);
    return HG_OK;
  }
  if (device >= 0) HG_CUDA(cudaSetDevice(device), "cudaSetDevice");
  HG_CUDA(cudaGetDevice(&c.device), "cudaGetDevice");
  std::vector<uint64_t> host(kPrimeTableWords * kPrimes);
  for (int i = 0; i < kPrimes; ++i) {
    const uint64_t p = dm[i];
    c.moduli[i] = p;
    c.pc[i] = PrimeConst{p, static_cast<uint32_t>(p >> kShift), 0};
    c.gens[i] = generator_h(p);
    const uint64_t w30 = powmod_h(c.gens[i], (p - 1) >> kLogNmax, p);
    const uint64_t w30i = invmod_h(w30, p);
    const uint64_t w4096 = powmod_h(w30, uint64_t(1) << (kLogNmax - kTileBits), p);
    const uint64_t w4096i = invmod_h(w4096, p);
    uint64_t *t = host.data() + i * kPrimeTableWords;
    uint64_t *sub_f = t, *sub_i = t + kSubWords, *hi_f = t + 2 * kSubWords, *lo_f = hi_f + kLevelWords,
             *hi_i = lo_f + kLevelWords, *lo_i = hi_i + kLevelWords;
    uint64_t a = 1, b = 1;
    for (size_t e = 0; e < kSubEntries; ++e) {
      sub_f[2 * e] = a;
      sub_f[2 * e + 1] = shoup_h(a, p);
      sub_i[2 * e] = b;
      sub_i[2 * e + 1] = shoup_h(b, p);
      a = mulmod_h(a, w4096, p);
      b = mulmod_h(b, w4096i, p);
    }
    const uint64_t step_f = powmod_h(w30, kLevelWords, p), step_i = powmod_h(w30i, kLevelWords, p);
    uint64_t lf = 1, li = 1, hf = 1, hi = 1;
    for (size_t e = 0; e < kLevelWords; ++e) {
      lo_f[e] = mont_h(lf, p);
      lo_i[e] = mont_h(li, p);
      hi_f[e] = mont_h(hf, p);
      hi_i[e] = mont_h(hi, p);
      lf = mulmod_h(lf, w30, p);
      li = mulmod_h(li, w30i, p);
      hf = mulmod_h(hf, step_f, p);
      hi = mulmod_h(hi, step_i, p);
    }
  }
  // Per block size 2^T, the sub-transform tables in padded (tw_pos) order,
  // copied from the 4096-point tables above (entry e of the table of T is
  // entry e * 2^(12 - T) of the 4096-point one); gap entries stay zero.
  for (int i = 0; i < kPrimes; ++i) {
    uint64_t *t = host.data() + i * kPrimeTableWords;
    const uint64_t *sub_f = t, *sub_i = t + kSubWords;
    uint64_t *swz = t + 2 * kSubWords + 4 * kLevelWords;
    for (int T = 1; T <= kTileBits; ++T) {
      const uint32_t base = tw_base(T);
      for (uint32_t e = 0; e < (1u << (T - 1)); ++e) {
        const uint32_t src = e << (kTileBits - T), dst = base + tw_pos(e);
        swz[2 * dst] = sub_f[2 * src];
        swz[2 * dst + 1] = sub_f[2 * src + 1];
        swz[2 * (kTwInverse + dst)] = sub_i[2 * src];
        swz[2 * (kTwInverse + dst) + 1] = sub_i[2 * src + 1];
      }
    }
  }
  HG_CUDA(c.tables.ensure(host.size() * sizeof(uint64_t)), "table allocation");
  HG_CUDA(cudaMemcpy(c.tables.p, host.data(), host.size() * sizeof(uint64_t), cudaMemcpyHostToDevice), "table upload");
  for (int i = 0; i < kPrimes; ++i) {
    const uint64_t *t = c.tables.u64() + i * kPrimeTableWords;
    c.tb[i].sub_fwd = reinterpret_cast<const ulonglong2 *>(t);
    c.tb[i].sub_inv = reinterpret_cast<const ulonglong2 *>(t + kSubWords);
    c.tb[i].hi_fwd = t + 2 * kSubWords;
    c.tb[i].lo_fwd = c.tb[i].hi_fwd + kLevelWords;
    c.tb[i].hi_inv = c.tb[i].lo_fwd + kLevelWords;
    c.tb[i].lo_inv = c.tb[i].hi_inv + kLevelWords;
    c.tb[i].swz = reinterpret_cast<const ulonglong2 *>(t + 2 * kSubWords + 4 * kLevelWords);
  }
  for (Lane &L : c.lanes) {
    HG_CUDA(cudaStreamCreateWithFlags(&L.stream, cudaStreamNonBlocking), "stream creation");
    HG_CUDA(cudaEventCreateWithFlags(&L.ws_done, cudaEventDisableTiming), "event creation");
    HG_CUDA(cudaStreamCreateWithFlags(&L.copy_stream, cudaStreamNonBlocking), "stream creation");
    HG_CUDA(cudaEventCreateWithFlags(&L.copy_done, cudaEventDisableTiming), "event creation");
    for (auto &op : L.slice_done)
      for (cudaEvent_t &e : op) HG_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming), "event creation");
    HG_CUDA(cudaStreamCreateWithFlags(&L.d2h_stream, cudaStreamNonBlocking), "stream creation");
    HG_CUDA(cudaEventCreateWithFlags(&L.carry_done, cudaEventDisableTiming), "event creation");
    HG_CUDA(cudaEventCreateWithFlags(&L.d2h_done, cudaEventDisableTiming), "event creation");
    HG_CUDA(L.misc.ensure(64), "scan state allocation");
    HG_CUDA(cudaMemset(L.misc.p, 0, 64), "scan state init");
  }
  c.lane = &c.lanes[0];
  c.ready = true;
  return HG_OK;
}

int ensure_init() {
  if (g_ctx.ready) return HG_OK;
  return init_locked(nullptr, 0, nullptr, 0, -1);
}

int ilog2_ceil(uint64_t n) {
  int l = 0;
  while ((uint64_t(1) << l) < n) ++l;
  return l;
}

uint64_t trimmed(const uint64_t *x, uint64_t n) {
  while (n > 0 && x[n - 1] == 0) --n;
  return n;
}

// Passes for N = 2^L: strided passes of 4..8 row bits over 4096-residue tiles
// (>= 16 columns, i.e. >= 128-byte row segments), then one contiguous pass
// over blocks of 2^T <= 4096 residues.  The last entry is the contiguous one.
std::vector<PassPlan> plan_passes(int L) {
  std::vector<PassPlan> v;
  if (L <= kTileBits) {
    v.push_back({L, 0, L});
    return v;
  }
  std::vector<int> parts;
  if (L < kTileBits + 4) {
    parts.push_back(4);  // 13..15: one 4-bit strided pass, a 9..11-bit block
  } else {
    const int rem = L - kTileBits;
    const int k = (rem + 7) / 8;
    for (int i = 0; i < k; ++i) parts.push_back(rem / k + (i < rem % k ? 1 : 0));
  }
  int logS = L;
  for (int part : parts) {
    logS -= part;
    v.push_back({part, logS, kTileBits});
  }
  v.push_back({logS, 0, logS});
  return v;
}

PassArgs base_args(int L, int nops) {
  PassArgs a{};
  a.nops = nops;
  a.logN = L;
  a.prime_lo = 0;
  a.nprimes = kPrimes;
  a.prime_stride = uint64_t(1) << L;
  a.nprod = 1;
  a.ws_stride = static_cast<uint64_t>(kPrimes) << L;
  for (int i = 0; i < kPrimes; ++i) {
    a.pc[i] = g_ctx.pc[i];
    a.tb[i] = g_ctx.tb[i];
  }
  a.err = err_word();
  return a;
}

// Algorithmic bytes of a launch over nops operands: every residue written
// once, every input read once (limbs when a pass reduces them itself).
double pass_bytes(const PassArgs &a, int readers, int writers) {
  const double words =
      static_cast<double>(a.nprimes) * static_cast<double>(uint64_t(1) << a.logN) * static_cast<double>(a.nprod);
  double bytes = 8.0 * words * writers;
  for (int op = 0; op < readers; ++op)
    bytes += a.limbs[op] ? 8.0 * static_cast<double>(a.nlimbs[op]) : 8.0 * words;
  return bytes;
}

// ---- inter-pass twiddle tables --------------------------------------------
//
// A strided pass over blocks of M = R * S residues multiplies row r of column
// s by w_M^(+-s * bitrev r).  For M up to 2^27 those M twiddles per prime are
// built once per (M, R, direction) and read by the pass (8 bytes per residue,
// shared by both operands), which saves the kernel the recurrence that forms
// them (one Montgomery product per residue): 2^26 x 2^26-limb products
// 25.0 -> 23.3 ms with the 2^27-point tables (3.2 GB per table, against 6.4 GB
// of workspace for the product itself).  Larger passes form them.
constexpr int kPassTwiddleMaxLogM = 27;
std::mutex g_ptw_mu;
std::map<std::tuple<int, int, bool, bool>, DevBuf> g_ptw;

// A table not built yet is not built while `st` is being captured into a
// CUDA graph (that would allocate and synchronise inside the capture): the
// pass then forms its twiddles.
const uint64_t *pass_twiddles(int logM, int logR, bool inverse, cudaStream_t st, const uint64_t *scale = nullptr) {
  if (logM > kPassTwiddleMaxLogM) return nullptr;
  std::lock_guard<std::mutex> lk(g_ptw_mu);
  const auto key = std::make_tuple(logM, logR, inverse, scale != nullptr);
  auto it = g_ptw.find(key);
  if (it != g_ptw.end()) return it->second.u64();
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(st, &cs) != cudaSuccess || cs != cudaStreamCaptureStatusNone) {
    cudaGetLastError();
    return nullptr;
  }
  DevBuf b;
  const size_t bytes = (static_cast<size_t>(kPrimes) << logM) * sizeof(uint64_t);
  if (b.ensure(bytes) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;  // no room: the pass forms its twiddles
  }
  cudaStream_t bs = nullptr;
  if (cudaStreamCreateWithFlags(&bs, cudaStreamNonBlocking) != cudaSuccess ||
      launch_pass_twiddles(b.u64(), logM, logR, inverse, g_ctx.tb, g_ctx.pc, kPrimes, bs, scale) != cudaSuccess ||
      cudaStreamSynchronize(bs) != cudaSuccess) {
    if (bs) cudaStreamDestroy(bs);
    cudaGetLastError();
    b.release();
    return nullptr;
  }
  cudaStreamDestroy(bs);
  const uint64_t *p = b.u64();
  g_ptw.emplace(key, b);
  return p;
}

void release_pass_twiddles() {
  std::lock_guard<std::mutex> lk(g_ptw_mu);
  for (auto &kv : g_ptw) kv.second.release();
  g_ptw.clear();
}

// Strided passes [s0, s1) of `plan` (whose last entry is the contiguous
// pass), forward in order or inverse in reverse order.  scale_last (inverse
// only): the last inverse pass reads its table multiplied by these
// Montgomery-form factors, and *scaled says whether it did (it forms its
// twiddles unscaled when no table can be had).
cudaError_t run_strided_range(PassArgs a, const std::vector<PassPlan> &plan, bool inverse, int s0, int s1,
                              cudaStream_t st, const uint64_t *scale_last = nullptr, bool *scaled = nullptr) {
  const int np = static_cast<int>(plan.size()) - 1;
  for (int s = s0; s < s1 && s < np; ++s) {
    const PassPlan &pp = plan[inverse ? np - 1 - s : s];
    a.logR = pp.logR;
    a.logS = pp.logS;
    a.logT = pp.logT;
    a.tiles = (uint64_t(1) << a.logN) >> pp.logT;
    const bool last_inverse = inverse && s == np - 1;
    a.ptw = pass_twiddles(pp.logR + pp.logS, pp.logR, inverse, st, last_inverse ? scale_last : nullptr);
    if (last_inverse && scaled) *scaled = scale_last && a.ptw;
    cudaError_t e;
    {
      ProfScope ps(inverse ? HG_KC_NTT_INVERSE : HG_KC_NTT_FORWARD, st, pass_bytes(a, a.nops, a.nops));
      e = launch_ntt_strided(a, inverse, st);
    }
    if (e != cudaSuccess) return e;
    a.limbs[0] = a.limbs[1] = nullptr;  // only the first forward pass reads limbs
    a.read_limbs = 0;
  }
  return cudaSuccess;
}

// All strided passes of `plan`.
cudaError_t run_strided(const PassArgs &a, const std::vector<PassPlan> &plan, bool inverse, cudaStream_t st,
                        const uint64_t *scale_last = nullptr, bool *scaled = nullptr) {
  return run_strided_range(a, plan, inverse, 0, static_cast<int>(plan.size()) - 1, st, scale_last, scaled);
}

// The contiguous pass (the plan's last entry) in the given mode.
cudaError_t run_contig(PassArgs a, const PassPlan &pp, int mode, cudaStream_t st) {
  a.logR = pp.logR;
  a.logS = 0;
  a.logT = pp.logT;
  a.tiles = (uint64_t(1) << a.logN) >> pp.logT;
  const int readers = mode == kContigMul ? 2 : 1;
  const int cls = mode == kContigFwd ? HG_KC_NTT_FORWARD : (mode == kContigInv ? HG_KC_NTT_INVERSE : HG_KC_MIDDLE);
  ProfScope ps(cls, st, pass_bytes(a, readers, 1));
  return launch_ntt_contig(a, mode, st);
}

// Montgomery-form factors N^-1 2^64 mod p_j for a 2^L-point product, which a
// product's last inverse pass folds into its table so that the
// reconstruction receives the coefficients mod p_j; false where the moduli
// do not meet the prescaled reconstruction's bounds (p0 < 2 p1, p0 < 2 p2,
// 3 p2 < 2^64).
bool prescale_factors(int L, uint64_t (&s)[kPrimes]) {
  const uint64_t p0 = g_ctx.moduli[0], p1 = g_ctx.moduli[1], p2 = g_ctx.moduli[2];
  if (!(p0 < 2 * p1 && p0 < 2 * p2 && p2 < ~uint64_t(0) / 3)) return false;
  const uint64_t N = uint64_t(1) << L;
  for (int j = 0; j < kPrimes; ++j) {
    const uint64_t p = g_ctx.moduli[j];
    s[j] = mont_h(mulmod_h(invmod_h(N % p, p), mont_h(1, p), p), p);
  }
  return true;
}

CrtConst crt_const(int L, bool prescaled = false) {
  CrtConst k{};
  k.prescaled = prescaled ? 1u : 0u;
  const uint64_t p0 = g_ctx.moduli[0], p1 = g_ctx.moduli[1], p2 = g_ctx.moduli[2];
  for (int i = 0; i < kPrimes; ++i) k.pc[i] = g_ctx.pc[i];
  const uint64_t N = uint64_t(1) << L;
  const uint64_t n0 = invmod_h(N % p0, p0), n1 = invmod_h(N % p1, p1), n2 = invmod_h(N % p2, p2);
  const uint64_t R0 = mont_h(1, p0), R1 = mont_h(1, p1), R2 = mont_h(1, p2);  // 2^64 mod p
  const uint64_t inv01 = invmod_h(p0 % p1, p1);
  const uint64_t inv012 = invmod_h(mulmod_h(p0 % p2, p1 % p2, p2), p2);
  auto pair = [](uint64_t w, uint64_t p) { return make_ulonglong2(w, shoup_h(w, p)); };
  k.k0 = pair(mulmod_h(n0, R0, p0), p0);
  k.k1a = pair(mulmod_h(mulmod_h(n1, R1, p1), inv01, p1), p1);
  k.k1b = pair(inv01, p1);
  k.k2a = pair(mulmod_h(mulmod_h(n2, R2, p2), inv012, p2), p2);
  k.k2b = pair(inv012, p2);
  k.k2c = pair(mulmod_h(p0 % p2, inv012, p2), p2);
  const u128 p01 = (u128)p0 * p1;
  k.p01_lo = static_cast<uint64_t>(p01);
  k.p01_hi = static_cast<uint64_t>(p01 >> 64);
  return k;
}

// Serialise use of the shared workspace across streams.
cudaError_t ws_acquire(cudaStream_t st) {
  if (g_ctx.lane->ws_pending) return cudaStreamWaitEvent(st, g_ctx.lane->ws_done, 0);
  return cudaSuccess;
}
cudaError_t ws_release(cudaStream_t st) {
  g_ctx.lane->ws_pending = true;
  return cudaEventRecord(g_ctx.lane->ws_done, st);
}

int scan_state(uint64_t tiles, ScanState *ss) {
  Context &c = g_ctx;
  const size_t need = (tiles + 1) * sizeof(unsigned long long);
  if (need > c.lane->flags.bytes) {
    HG_CUDA(cudaDeviceSynchronize(), "sync before flag growth");
    HG_CUDA(c.lane->flags.ensure(need * 2), "flag allocation");
    HG_CUDA(cudaMemset(c.lane->flags.p, 0, c.lane->flags.bytes), "flag init");
  }
  if (++c.lane->epoch == 0) c.lane->epoch = 1;
  ss->ticket = static_cast<unsigned long long *>(c.lane->misc.p);
  ss->ticket_base = c.lane->ticket_count;
  ss->flags = static_cast<unsigned long long *>(c.lane->flags.p);
  ss->epoch = c.lane->epoch;
  ss->err = err_word();
  c.lane->ticket_count += tiles;
  return HG_OK;
}

int check_len(int L) {
  if (L > kLogNmax) return fail(HG_ERR_ARG, "transform length 2^%d exceeds the supported 2^%d", L, kLogNmax);
  return HG_OK;
}

// ---- unbalanced products in chunks ----------------------------------------
//
// When one operand is much longer than the other, one transform of the whole
// product (N = pow2 >= nx + ny, src/ntt-multiply.lisp:174-254) spends most of
// its work on zero padding.  The long operand is cut into K chunks of C limbs
// instead; the short one (ns limbs) is transformed once to a 2^L-point
// spectrum, 2^L >= C + ns; each chunk's 2^L-point transform is multiplied by
// that spectrum and transformed back, all chunks in one launch per pass; the
// reconstruction adds the two chunk products that meet at each position (the
// product is the same integer: sum_k chunk_k * short * 2^(64 C k)).
struct ChunkPlan {
  int L = 0;
  uint64_t chunk = 0, nchunks = 0;
};

// Cost of a transform of 2^L points in units of one radix-2 stage over one
// point: L stages plus about kPassCost stages' worth of memory passes.  On
// GB300 the measured time of chunked products is 0.93-0.97 of this model's
// ratio to one transform (2^16..2^25 long operands, ratios 0.17-0.80).
constexpr double kPassCost = 4.0;
// Chunk only when the estimate is below this fraction of one transform.
constexpr double kChunkGain = 0.95;

// The cheapest chunking of a long operand of nl limbs and a short one of ns
// <= nl limbs, or false when one transform of the whole product is cheaper.
// C = (2^L - ns) rounded down to a multiple of 8 (>= 2^(L-1) because
// 2^L >= 2 pow2(ns) >= 16), so that at most two chunk products meet at any
// position of the result.
std::atomic<int> g_chunking{1};  // hg_set_chunking

bool plan_chunks(uint64_t nl, uint64_t ns, ChunkPlan &cp) {
  if (ns == 0 || nl < ns || !g_chunking.load()) return false;
  const int Lf = ilog2_ceil(nl + ns);
  const auto cost = [](double transforms, int L) { return transforms * std::ldexp(L + kPassCost, L); };
  double best = kChunkGain * cost(3.0, Lf);
  bool found = false;
  const int Lmin = std::max(4, ilog2_ceil(ns) + 1);
  for (int L = Lmin; L < Lf && L <= Lmin + 4; ++L) {
    const uint64_t T = uint64_t(1) << L;
    const uint64_t c = (T - ns) & ~uint64_t(7);
    const uint64_t k = (nl + c - 1) / c;
    if (k < 2) continue;
    const double e = cost(2.0 * static_cast<double>(k) + 1.0, L);
    if (e < best) {
      best = e;
      cp = ChunkPlan{L, c, k};
      found = true;
    }
  }
  return found;
}

// The chunked schedule of ntt_product_device.  Chunk k's residues occupy
// workspace A at k * 3 * 2^L words, the short operand's spectrum workspace
// B.  Caller's operand 0 (x) is resident; when y_ready is given, y may still
// be in flight, so the work on x's role comes first.
int chunk_product_device(const uint64_t *x, uint64_t nx, const uint64_t *y, uint64_t ny, uint64_t *out,
                         uint64_t nout, const ChunkPlan &cp, cudaStream_t st, cudaEvent_t y_ready) {
  Context &c = g_ctx;
  const bool x_long = nx >= ny;
  const uint64_t *lng = x_long ? x : y, *sht = x_long ? y : x;
  const uint64_t nl = x_long ? nx : ny, ns = x_long ? ny : nx;
  const int L = cp.L;
  const uint64_t T = uint64_t(1) << L;
  const uint64_t slab = static_cast<uint64_t>(kPrimes) * T;
  HG_CUDA(ws_acquire(st), "workspace ordering");
  if (c.lane->A.bytes < cp.nchunks * slab * 8 || c.lane->B.bytes < slab * 8) {
    HG_CUDA(cudaDeviceSynchronize(), "sync before workspace growth");
    HG_CUDA(c.lane->A.ensure(cp.nchunks * slab * 8), "workspace allocation");
    HG_CUDA(c.lane->B.ensure(slab * 8), "workspace allocation");
  }
  const std::vector<PassPlan> plan = plan_passes(L);
  const bool one_pass = plan.size() == 1;
  PassArgs a = base_args(L, 1);  // the chunks
  a.data[0] = c.lane->A.u64();
  a.data[1] = c.lane->B.u64();
  a.limbs[0] = lng;
  a.nlimbs[0] = nl;
  a.chunk = cp.chunk;
  a.nprod = cp.nchunks;
  a.ws_stride = slab;
  PassArgs sp = base_args(L, 1);  // the short operand's spectrum
  sp.data[0] = c.lane->B.u64();
  sp.limbs[0] = sht;
  sp.nlimbs[0] = ns;
  auto chunks_forward = [&]() -> int {
    HG_CUDA(run_strided(a, plan, false, st), "forward transform");
    return HG_OK;
  };
  auto spectrum_forward = [&]() -> int {
    HG_CUDA(run_strided(sp, plan, false, st), "forward transform");
    PassArgs f = sp;
    if (!one_pass) f.limbs[0] = nullptr;
    HG_CUDA(run_contig(f, plan.back(), kContigFwd, st), "forward transform");
    return HG_OK;
  };
  int rc = x_long ? chunks_forward() : spectrum_forward();
  if (rc) return rc;
  if (y_ready) HG_CUDA(cudaStreamWaitEvent(st, y_ready, 0), "operand upload ordering");
  rc = x_long ? spectrum_forward() : chunks_forward();
  if (rc) return rc;
  {
    PassArgs m = a;
    if (!one_pass) m.limbs[0] = nullptr;
    HG_CUDA(run_contig(m, plan.back(), kContigMulSpec, st), "middle pass");
  }
  PassArgs inv = base_args(L, 1);
  inv.data[0] = c.lane->A.u64();
  inv.nprod = cp.nchunks;
  inv.ws_stride = slab;
  uint64_t sc[kPrimes];
  bool scaled = false;
  HG_CUDA(run_strided(inv, plan, true, st, prescale_factors(L, sc) ? sc : nullptr, &scaled), "inverse transform");
  const uint64_t size = nx + ny;
  if (nout > size) HG_CUDA(cudaMemsetAsync(out + size, 0, (nout - size) * sizeof(uint64_t), st), "zero tail");
  ScanState ss;
  rc = scan_state(carry_tiles(size), &ss);
  if (rc) return rc;
  uint64_t tiles = 0;
  {
    ProfScope ps(HG_KC_CARRY, st, 32.0 * static_cast<double>(size), 2);  // local scan + fix
    HG_CUDA(launch_crt_carry_chunks(c.lane->A.u64(), slab, L, cp.chunk, cp.nchunks, crt_const(L, scaled), out, size,
                                    ss, st, &tiles),
            "reconstruction");
  }
  HG_CUDA(ws_release(st), "workspace ordering");
  return HG_OK;
}

// Operands the host entry points still hold in host memory.  Given these,
// ntt_product_device copies them into its device operands x, y itself, so
// that the copies overlap the first forward pass.
struct HostOperands {
  const uint64_t *hx, *hy;  // hy null for a square
};


// Copy columns [c0, c1) of every row of the first strided pass (row r holds
// limbs [r S, (r + 1) S)) of n host limbs into dst: one 2-D copy for the
// full rows, one copy for the part of the last row below n.
cudaError_t copy_columns(uint64_t *dst, const uint64_t *src, uint64_t n, uint64_t S, uint64_t c0, uint64_t c1,
                         cudaStream_t st) {
  const uint64_t full = n / S;
  cudaError_t e = cudaSuccess;
  if (full && c1 > c0)
    e = cudaMemcpy2DAsync(dst + c0, S * sizeof(uint64_t), src + c0, S * sizeof(uint64_t), (c1 - c0) * sizeof(uint64_t),
                          full, cudaMemcpyHostToDevice, st);
  const uint64_t base = full * S;
  if (e == cudaSuccess && base + c0 < n) {
    const uint64_t end = std::min(base + c1, n);
    e = cudaMemcpyAsync(dst + base + c0, src + base + c0, (end - base - c0) * sizeof(uint64_t), cudaMemcpyHostToDevice,
                        st);
  }
  return e;
}

// |x| * |y| (or |x|^2 when y == nullptr) into out[0, nout) on device memory.
// An unbalanced pair runs in chunks (chunk_product_device).
// With host operands (x, y are then the device buffers to fill), each
// operand is copied on the copy stream in column slices of the first strided
// pass, and that pass runs slice by slice as the copies land: only one slice
// of the upload is left exposed.  A chunked product copies x ahead of its
// work and y on the copy stream (chunk_product_device waits for y).
int ntt_product_device(const uint64_t *x, uint64_t nx, const uint64_t *y, uint64_t ny, uint64_t *out, uint64_t nout,
                       cudaStream_t st, const HostOperands *host = nullptr) {
  Context &c = g_ctx;
  const bool square = (y == nullptr);
  if (square) ny = nx;
  const uint64_t size = nx + ny;
  if (!out || (nx && !x) || (!square && ny && !y)) return fail(HG_ERR_ARG, "null pointer");
  if (nout < size) return fail(HG_ERR_ARG, "nout = %llu cannot hold the %llu-limb product", (unsigned long long)nout,
                               (unsigned long long)size);
  if (nx == 0 || ny == 0) {
    HG_CUDA(cudaMemsetAsync(out, 0, nout * sizeof(uint64_t), st), "zero product");
    return HG_OK;
  }
  ChunkPlan cp;
  if (!square && plan_chunks(std::max(nx, ny), std::min(nx, ny), cp)) {
    cudaEvent_t y_ready = nullptr;
    if (host) {
      HG_CUDA(cudaMemcpyAsync(const_cast<uint64_t *>(x), host->hx, nx * 8, cudaMemcpyHostToDevice, st),
              "operand upload");
      HG_CUDA(cudaMemcpyAsync(const_cast<uint64_t *>(y), host->hy, ny * 8, cudaMemcpyHostToDevice, c.lane->copy_stream),
              "operand upload");
      HG_CUDA(cudaEventRecord(c.lane->copy_done, c.lane->copy_stream), "operand upload");
      y_ready = c.lane->copy_done;
    }
    return chunk_product_device(x, nx, y, ny, out, nout, cp, st, y_ready);
  }
  const int L = ilog2_ceil(size);
  int rc = check_len(L);
  if (rc) return rc;
  const uint64_t N = uint64_t(1) << L;
  const size_t words = static_cast<size_t>(kPrimes) * N;
  HG_CUDA(ws_acquire(st), "workspace ordering");
  if (c.lane->A.bytes < words * 8 || (!square && c.lane->B.bytes < words * 8)) {
    HG_CUDA(cudaDeviceSynchronize(), "sync before workspace growth");
    HG_CUDA(c.lane->A.ensure(words * 8), "workspace allocation");
    if (!square) HG_CUDA(c.lane->B.ensure(words * 8), "workspace allocation");
  }
  // Strided forward passes, the fused middle (last forward pass of both
  // operands + pointwise product + first inverse pass), strided inverse passes.
  const std::vector<PassPlan> plan = plan_passes(L);
  PassArgs a = base_args(L, square ? 1 : 2);
  a.data[0] = c.lane->A.u64();
  a.data[1] = c.lane->B.u64();
  a.limbs[0] = x;
  a.limbs[1] = square ? nullptr : y;
  a.nlimbs[0] = nx;
  a.nlimbs[1] = square ? 0 : ny;
  if (host && plan.size() == 1) {  // one contiguous pass reads the limbs: copy them first
    HG_CUDA(cudaMemcpyAsync(const_cast<uint64_t *>(x), host->hx, nx * 8, cudaMemcpyHostToDevice, st),
            "operand upload");
    if (!square)
      HG_CUDA(cudaMemcpyAsync(const_cast<uint64_t *>(y), host->hy, ny * 8, cudaMemcpyHostToDevice, st),
              "operand upload");
  }
  if (host && plan.size() > 1) {
    // The first strided pass covers one block of N = R S residues; its tile t
    // reads columns [t C, (t + 1) C) (C = 4096 / R) of every row.
    const PassPlan &p0 = plan[0];
    const uint64_t S = uint64_t(1) << p0.logS;
    const uint64_t C = uint64_t(1) << (kTileBits - p0.logR);
    const uint64_t ntiles = N >> kTileBits;
    const int K = static_cast<int>(std::min<uint64_t>(kUploadSlices, ntiles));
    const int nops = square ? 1 : 2;
    const uint64_t *ptw = pass_twiddles(p0.logR + p0.logS, p0.logR, false, st);
    // Each slice's copy is issued just before the pass slice that reads it.
    // From page-locked memory the copies are asynchronous and run back to
    // back on the copy stream.  From pageable memory the driver returns only
    // once a copy is staged, so the host stages slice k + 1 while the device
    // runs the pass on slice k (2^24 x 2^24 limbs: 9.30 -> 8.15 ms end to end).
    for (int op = 0; op < nops; ++op) {
      for (int k = 0; k < K; ++k) {
        const uint64_t t0 = ntiles * k / K, t1 = ntiles * (k + 1) / K;
        HG_CUDA(copy_columns(const_cast<uint64_t *>(op ? y : x), op ? host->hy : host->hx, op ? ny : nx, S, t0 * C,
                             t1 * C, c.lane->copy_stream),
                "operand upload");
        HG_CUDA(cudaEventRecord(c.lane->slice_done[op][k], c.lane->copy_stream), "operand upload");
        HG_CUDA(cudaStreamWaitEvent(st, c.lane->slice_done[op][k], 0), "operand upload ordering");
        PassArgs f = a;
        f.nops = 1;
        f.data[0] = op ? c.lane->B.u64() : c.lane->A.u64();
        f.limbs[0] = op ? y : x;
        f.nlimbs[0] = op ? ny : nx;
        f.logR = p0.logR;
        f.logS = p0.logS;
        f.logT = p0.logT;
        f.tile_lo = t0;
        f.tiles = t1 - t0;
        f.ptw = ptw;
        ProfScope ps(HG_KC_NTT_FORWARD, st, pass_bytes(f, 1, 1) * static_cast<double>(t1 - t0) / ntiles);
        HG_CUDA(launch_ntt_strided(f, false, st), "forward transform");
      }
      // This operand's remaining strided passes run while the next one's
      // upload lands (2^24 x 2^24 end to end: 7.29 -> 7.25 ms).
      PassArgs rest = a;
      rest.nops = 1;
      rest.data[0] = op ? c.lane->B.u64() : c.lane->A.u64();
      rest.limbs[0] = rest.limbs[1] = nullptr;
      rest.nlimbs[0] = rest.nlimbs[1] = 0;
      HG_CUDA(run_strided_range(rest, plan, false, 1, static_cast<int>(plan.size()) - 1, st), "forward transform");
    }
  } else {
    HG_CUDA(run_strided(a, plan, false, st), "forward transform");
  }
  {
    PassArgs m = a;
    if (plan.size() > 1) m.limbs[0] = m.limbs[1] = nullptr;
    HG_CUDA(run_contig(m, plan.back(), square ? kContigSqr : kContigMul, st), "middle pass");
  }
  PassArgs inv = base_args(L, 1);
  inv.data[0] = c.lane->A.u64();
  uint64_t sc[kPrimes];
  bool scaled = false;
  HG_CUDA(run_strided(inv, plan, true, st, prescale_factors(L, sc) ? sc : nullptr, &scaled), "inverse transform");
  if (nout > N) HG_CUDA(cudaMemsetAsync(out + N, 0, (nout - N) * sizeof(uint64_t), st), "zero tail");
  ScanState ss;
  const uint64_t nproc = nout < N ? nout : N;
  rc = scan_state(carry_tiles(nproc), &ss);
  if (rc) return rc;
  uint64_t tiles = 0;
  {
    ProfScope ps(HG_KC_CARRY, st, 32.0 * static_cast<double>(nproc), 2);  // local scan + fix
    HG_CUDA(launch_crt_carry(c.lane->A.u64(), L, crt_const(L, scaled), out, nout, ss, st, &tiles),
            "reconstruction");
  }
  HG_CUDA(ws_release(st), "workspace ordering");
  return HG_OK;
}

// ---- products on a fixed scratch array (hg_mul_device_noalloc) ----------
//
// Scratch layout, in words: operand 0's residues [3][2^16], operand 1's
// residues [3][2^16], the carry scan's ticket word, then one flag word per
// carry tile (16 at 2^16).  Static device memory is zero when the module
// loads; the residue area needs no initial value (the first pass writes
// every word it later reads), and the call clears the ticket and flag words
// on its stream before each reconstruction.
constexpr int kNoAllocLogN = 16;
constexpr uint64_t kNoAllocN = uint64_t(1) << kNoAllocLogN;
constexpr uint64_t kNoAllocResWords = 2ull * kPrimes * kNoAllocN;
constexpr uint64_t kNoAllocScanWords = 64;
constexpr int kNoAllocDevices = 64;
static_assert(kNoAllocN == HG_NOALLOC_MAX_LIMBS, "public limit and scratch size disagree");

static __device__ __align__(256) uint64_t g_noalloc_scratch[kNoAllocResWords + kNoAllocScanWords];

// Device address of g_noalloc_scratch per device ordinal, looked up once.
uint64_t *g_noalloc_ptr[kNoAllocDevices] = {};

// ntt_product_device's schedule on the static scratch: at 2^L <= 2^16 the
// plan is one contiguous pass (L <= 12) or one 4-bit strided pass around an
// (L - 4)-bit contiguous block, launched here without the growing workspace,
// the shared scan state or the profiling events of the general path.
int noalloc_product_device(const uint64_t *x, uint64_t nx, const uint64_t *y, uint64_t ny, uint64_t *out,
                           uint64_t nout, cudaStream_t st) {
  Context &c = g_ctx;
  const bool square = (y == nullptr);
  if (square) ny = nx;
  const uint64_t size = nx + ny;
  if (!out || (nx && !x) || (!square && ny && !y)) return fail(HG_ERR_ARG, "null pointer");
  if (nout < size) return fail(HG_ERR_ARG, "nout = %llu cannot hold the %llu-limb product", (unsigned long long)nout,
                               (unsigned long long)size);
  if (size > kNoAllocN)
    return fail(HG_ERR_ARG, "hg_mul_device_noalloc: a %llu-limb product exceeds its fixed scratch limit of %llu limbs",
                (unsigned long long)size, (unsigned long long)kNoAllocN);
  int dev = -1;
  HG_CUDA(cudaGetDevice(&dev), "cudaGetDevice");
  if (dev != c.device)
    return fail(HG_ERR_ARG, "hg_mul_device_noalloc: current device %d is not the library's device %d", dev, c.device);
  if (dev < 0 || dev >= kNoAllocDevices) return fail(HG_ERR_ARG, "device ordinal %d out of range", dev);
  if (!g_noalloc_ptr[dev]) {
    void *p = nullptr;
    HG_CUDA(cudaGetSymbolAddress(&p, g_noalloc_scratch), "scratch address lookup");
    g_noalloc_ptr[dev] = static_cast<uint64_t *>(p);
  }
  uint64_t *scratch = g_noalloc_ptr[dev];
  if (nx == 0 || ny == 0) {
    HG_CUDA(cudaMemsetAsync(out, 0, nout * sizeof(uint64_t), st), "zero product");
    return HG_OK;
  }
  const int L = ilog2_ceil(size);
  const uint64_t N = uint64_t(1) << L;
  const int logC = L <= kTileBits ? L : L - 4;  // contiguous block bits
  PassArgs a = base_args(L, square ? 1 : 2);
  a.data[0] = scratch;
  a.data[1] = scratch + kPrimes * kNoAllocN;
  a.limbs[0] = x;
  a.limbs[1] = square ? nullptr : y;
  a.nlimbs[0] = nx;
  a.nlimbs[1] = square ? 0 : ny;
  if (L > kTileBits) {
    PassArgs f = a;
    f.logR = 4;
    f.logS = logC;
    f.logT = kTileBits;
    f.tiles = N >> kTileBits;
    HG_CUDA(launch_ntt_strided(f, false, st), "forward transform");
    a.limbs[0] = a.limbs[1] = nullptr;
  }
  a.logR = logC;
  a.logS = 0;
  a.logT = logC;
  a.tiles = N >> logC;
  HG_CUDA(launch_ntt_contig(a, square ? kContigSqr : kContigMul, st), "middle pass");
  if (L > kTileBits) {
    PassArgs inv = base_args(L, 1);
    inv.data[0] = scratch;
    inv.logR = 4;
    inv.logS = logC;
    inv.logT = kTileBits;
    inv.tiles = N >> kTileBits;
    HG_CUDA(launch_ntt_strided(inv, true, st), "inverse transform");
  }
  if (nout > N) HG_CUDA(cudaMemsetAsync(out + N, 0, (nout - N) * sizeof(uint64_t), st), "zero tail");
  const uint64_t nproc = nout < N ? nout : N;
  const uint64_t tiles = carry_tiles(nproc);
  if (tiles + 1 > kNoAllocScanWords) return fail(HG_ERR_ARG, "carry scan of %llu tiles exceeds the scratch",
                                                 (unsigned long long)tiles);
  uint64_t *scan = scratch + kNoAllocResWords;
  HG_CUDA(cudaMemsetAsync(scan, 0, (tiles + 1) * sizeof(uint64_t), st), "scan state reset");
  ScanState ss;
  ss.ticket = reinterpret_cast<unsigned long long *>(scan);
  ss.ticket_base = 0;
  ss.flags = reinterpret_cast<unsigned long long *>(scan + 1);
  ss.epoch = 1;
  ss.err = err_word();
  uint64_t used = 0;
  HG_CUDA(launch_crt_carry(scratch, L, crt_const(L), out, nout, ss, st, &used), "reconstruction");
  return HG_OK;
}

int small_product_device(const uint64_t *x, uint64_t nx, const uint64_t *y, uint64_t ny, uint64_t d, uint64_t *out,
                         uint64_t nout, cudaStream_t st) {
  const uint64_t size = y ? nx + ny : nx + 1;
  if (!out || (nx && !x)) return fail(HG_ERR_ARG, "null pointer");
  if (y && nx < ny) return fail(HG_ERR_ARG, "schoolboy needs nx >= ny");
  if (nout < size) return fail(HG_ERR_ARG, "nout = %llu cannot hold the %llu-limb product", (unsigned long long)nout,
                               (unsigned long long)size);
  if (nx == 0 || (y && ny == 0) || (!y && d == 0)) {
    HG_CUDA(cudaMemsetAsync(out, 0, nout * sizeof(uint64_t), st), "zero product");
    return HG_OK;
  }
  if (nout > size) HG_CUDA(cudaMemsetAsync(out + size, 0, (nout - size) * sizeof(uint64_t), st), "zero tail");
  HG_CUDA(ws_acquire(st), "workspace ordering");
  ScanState ss;
  int rc = scan_state(carry_tiles(size), &ss);
  if (rc) return rc;
  uint64_t tiles = 0;
  {
    ProfScope ps(HG_KC_SMALL, st, 8.0 * static_cast<double>(nx + (y ? ny : 0) + size), 2);
    if (y)
      HG_CUDA(launch_schoolboy_carry(x, nx, y, ny, out, size, ss, st, &tiles), "schoolboy product");
    else
      HG_CUDA(launch_digit_carry(x, nx, d, out, size, ss, st, &tiles), "digit product");
  }
  HG_CUDA(ws_release(st), "workspace ordering");
  return HG_OK;
}

#if HG_CHECKED
// The first fault a check latched in any translation unit since the last read.
int read_checked_faults() {
  static int (*const readers[])() = {checked_fault_strided, checked_fault_contig, checked_fault_crt,
                                     checked_fault_persist, checked_fault_peak,   checked_fault_sum,
                                     checked_fault_series};
  int first = 0;
  for (auto r : readers) {
    const int v = r();
    if (v && !first) first = v;
  }
  if (first == kDevRange) return fail(HG_ERR_INCONSISTENT, "checked build: a residue left its range");
  if (first == kDevBounds) return fail(HG_ERR_INCONSISTENT, "checked build: a residue index left its array");
  if (first == kDevProduct)
    return fail(HG_ERR_INCONSISTENT, "checked build: a modular product differs from the exact reduction");
  if (first) return fail(HG_ERR_CUDA, "checked build: fault word unreadable or code %d", first);
  return HG_OK;
}
#endif

int read_device_error(cudaStream_t st) {
  int err = 0;
  int *d_err = err_word();
  HG_CUDA(cudaMemcpyAsync(&err, d_err, sizeof(int), cudaMemcpyDeviceToHost, st), "error word read");
  HG_CUDA(cudaStreamSynchronize(st), "stream synchronise");
#if HG_CHECKED
  {
    const int rc = read_checked_faults();
    if (rc) return rc;
  }
#endif
  if (err) {
    HG_CUDA(cudaMemsetAsync(d_err, 0, sizeof(int), st), "error word reset");
    HG_CUDA(cudaStreamSynchronize(st), "stream synchronise");
    if (err == kDevCarryOverflow) return fail(HG_ERR_INCONSISTENT, "a carry left the top of the result storage");
    if (err == kDevCopyTimeout) return fail(HG_ERR_CUDA, "a tile copy did not complete within its wait limit");
    return fail(HG_ERR_CUDA, "device error %d", err);
  }
  return HG_OK;
}

// Device address of a page-locked host buffer (cudaHostAlloc, pinned torch
// tensors, cudaHostRegister), or nullptr for pageable or unknown memory.
const void *pinned_view(const void *h) {
  if (!h) return nullptr;
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, h) != cudaSuccess) {
    cudaGetLastError();  // clear the sticky-free error of an unregistered pointer
    return nullptr;
  }
  if (a.type == cudaMemoryTypeHost && a.devicePointer) return a.devicePointer;
  return nullptr;
}

// Host-memory wrapper: stage operands, run, copy back, check.
enum class Kind { Ntt, Square, Schoolboy, Digit };

int host_product(Kind kind, const uint64_t *x, size_t nx, const uint64_t *y, size_t ny, uint64_t d, uint64_t *out,
                 size_t nout) {
  std::lock_guard<std::recursive_mutex> lock(g_ctx.mu);
  int rc = ensure_init();
  if (rc) return rc;
  Context &c = g_ctx;
  if (!out || (nx && !x) || (ny && !y && (kind == Kind::Ntt || kind == Kind::Schoolboy)))
    return fail(HG_ERR_ARG, "null pointer");
  nx = trimmed(x, nx);
  if (kind == Kind::Ntt || kind == Kind::Schoolboy) ny = trimmed(y, ny);
  if (kind == Kind::Square) ny = nx;
  if (kind == Kind::Digit) ny = 1;
  const size_t size = nx + ny;
  if (nout < size) return fail(HG_ERR_ARG, "nout = %zu cannot hold the %zu-limb product", nout, size);
  if (kind == Kind::Schoolboy && nx < ny) return fail(HG_ERR_ARG, "schoolboy needs nx >= ny");
  const bool zero = nx == 0 || ((kind == Kind::Ntt || kind == Kind::Schoolboy) && ny == 0) ||
                    (kind == Kind::Digit && d == 0);
  if (zero) {
    memset(out, 0, nout * sizeof(uint64_t));
    return HG_OK;
  }
  const size_t nd = size;  // limbs computed on the device; the rest are zero
  cudaStream_t st = c.lane->stream;
  // Pinned (page-locked) host buffers are addressable from the device over
  // the host link, so the kernels read the operands and write the product
  // in place; pageable buffers go through device staging buffers.
  const bool two = (kind == Kind::Ntt || kind == Kind::Schoolboy);
  const uint64_t *dx = static_cast<const uint64_t *>(pinned_view(x));
  const uint64_t *dy = two ? static_cast<const uint64_t *>(pinned_view(y)) : nullptr;
  uint64_t *dout = static_cast<uint64_t *>(const_cast<void *>(pinned_view(out)));
  // An NTT product or square with strided passes copies its operands over
  // the host link instead of reading them in place; ntt_product_device
  // overlaps the copies with the first forward pass.
  const bool host_ops = (kind == Kind::Ntt || kind == Kind::Square) && ilog2_ceil(size) > kTileBits;
  const HostOperands ho{x, kind == Kind::Ntt ? y : nullptr};
  if (host_ops) {
    HG_CUDA(c.lane->X.ensure(nx * 8), "operand allocation");
    dx = c.lane->X.u64();
    if (kind == Kind::Ntt) {
      HG_CUDA(c.lane->Y.ensure(ny * 8), "operand allocation");
      dy = c.lane->Y.u64();
    }
  }
  if (!dx) {
    HG_CUDA(c.lane->X.ensure(nx * 8), "operand allocation");
    HG_CUDA(cudaMemcpyAsync(c.lane->X.p, x, nx * 8, cudaMemcpyHostToDevice, st), "operand upload");
    dx = c.lane->X.u64();
  }
  if (two && !dy) {
    HG_CUDA(c.lane->Y.ensure(ny * 8), "operand allocation");
    HG_CUDA(cudaMemcpyAsync(c.lane->Y.p, y, ny * 8, cudaMemcpyHostToDevice, st), "operand upload");
    dy = c.lane->Y.u64();
  }
  const bool staged_out = (dout == nullptr);
  if (staged_out) {
    HG_CUDA(c.lane->OUT.ensure(nd * 8), "result allocation");
    dout = c.lane->OUT.u64();
  }
  switch (kind) {
    case Kind::Ntt: rc = ntt_product_device(dx, nx, dy, ny, dout, nd, st, host_ops ? &ho : nullptr); break;
    case Kind::Square: rc = ntt_product_device(dx, nx, nullptr, 0, dout, nd, st, host_ops ? &ho : nullptr); break;
    case Kind::Schoolboy: rc = small_product_device(dx, nx, dy, ny, 0, dout, nd, st); break;
    case Kind::Digit: rc = small_product_device(dx, nx, nullptr, 0, d, dout, nd, st); break;
  }
  if (rc) return rc;
  if (staged_out) HG_CUDA(cudaMemcpyAsync(out, dout, nd * 8, cudaMemcpyDeviceToHost, st), "result download");
  rc = read_device_error(st);
  if (rc) return rc;
  if (nout > nd) memset(out + nd, 0, (nout - nd) * sizeof(uint64_t));
  return HG_OK;
}

// ---- many host-memory products, pipelined (hg_mul_host_pipeline) ----------
//
// Product i runs in lane i mod 2: its operands go up on the lane's copy
// stream in column slices of the first pass (as in hg_mul), its transforms
// and carry run on the lane's stream into the lane's device result buffer,
// and a copy on the lane's download stream brings the result down.  While
// product i's result goes down, product i + 1's operands go up and its
// transforms run in the other lane; product i + 2 reuses lane i's buffers
// once product i's download is done (its upload waits for product i's carry,
// its carry for product i's download).

struct TailZero {
  uint64_t *p;
  size_t n;
};

void CUDART_CB zero_tail(void *arg) {
  TailZero *t = static_cast<TailZero *>(arg);
  memset(t->p, 0, t->n * sizeof(uint64_t));
  delete t;
}

int pipeline_one(Lane &L, const hg_host_product &q) {
  const bool square = q.y == nullptr;
  if (!q.out || (q.nx && !q.x) || (!square && q.ny && !q.y)) return fail(HG_ERR_ARG, "null pointer");
  const size_t nx = trimmed(q.x, q.nx);
  const size_t ny = square ? nx : trimmed(q.y, q.ny);
  const size_t size = nx + ny;
  if (q.nout < size) return fail(HG_ERR_ARG, "nout = %zu cannot hold the %zu-limb product", q.nout, size);
  if (L.d2h_pending) {
    HG_CUDA(cudaStreamWaitEvent(L.copy_stream, L.carry_done, 0), "lane ordering");
    HG_CUDA(cudaStreamWaitEvent(L.stream, L.d2h_done, 0), "lane ordering");
  }
  size_t nd = 0;  // limbs computed on the device
  if (nx && ny) {
    if (ilog2_ceil(size) <= kTileBits) {  // one contiguous pass reads the operands: they go up on the stream
      HG_CUDA(L.X.ensure(nx * 8), "operand allocation");
      HG_CUDA(cudaMemcpyAsync(L.X.p, q.x, nx * 8, cudaMemcpyHostToDevice, L.stream), "operand upload");
      if (!square) {
        HG_CUDA(L.Y.ensure(ny * 8), "operand allocation");
        HG_CUDA(cudaMemcpyAsync(L.Y.p, q.y, ny * 8, cudaMemcpyHostToDevice, L.stream), "operand upload");
      }
      HG_CUDA(L.OUT.ensure(size * 8), "result allocation");
      const int rc = ntt_product_device(L.X.u64(), nx, square ? nullptr : L.Y.u64(), ny, L.OUT.u64(), size, L.stream);
      if (rc) return rc;
    } else {
      HG_CUDA(L.X.ensure(nx * 8), "operand allocation");
      if (!square) HG_CUDA(L.Y.ensure(ny * 8), "operand allocation");
      HG_CUDA(L.OUT.ensure(size * 8), "result allocation");
      const HostOperands ho{q.x, square ? nullptr : q.y};
      const int rc = ntt_product_device(L.X.u64(), nx, square ? nullptr : L.Y.u64(), ny, L.OUT.u64(), size,
                                        L.stream, &ho);
      if (rc) return rc;
    }
    nd = size;
  }
  HG_CUDA(cudaEventRecord(L.carry_done, L.stream), "lane ordering");
  HG_CUDA(cudaStreamWaitEvent(L.d2h_stream, L.carry_done, 0), "lane ordering");
  if (nd) HG_CUDA(cudaMemcpyAsync(q.out, L.OUT.p, nd * 8, cudaMemcpyDeviceToHost, L.d2h_stream), "result download");
  if (q.nout > nd) {
    TailZero *t = new TailZero{q.out + nd, q.nout - nd};
    const cudaError_t e = cudaLaunchHostFunc(L.d2h_stream, zero_tail, t);
    if (e != cudaSuccess) {
      delete t;
      return cuda_fail(e, "result tail");
    }
  }
  HG_CUDA(cudaEventRecord(L.d2h_done, L.d2h_stream), "lane ordering");
  L.d2h_pending = true;
  return HG_OK;
}

int host_pipeline(const hg_host_product *prods, size_t n) {
  std::lock_guard<std::recursive_mutex> lock(g_ctx.mu);
  int rc = ensure_init();
  if (rc) return rc;
  if (n && !prods) return fail(HG_ERR_ARG, "null pointer");
  Context &c = g_ctx;
  for (size_t i = 0; i < n && rc == HG_OK; ++i) {
    c.lane = &c.lanes[i % kLanes];
    rc = pipeline_one(*c.lane, prods[i]);
  }
  c.lane = &c.lanes[0];
  // Nothing of this call may still write into the caller's buffers after it returns.
  for (Lane &L : c.lanes) {
    if (!L.d2h_pending) continue;
    const cudaError_t e = cudaStreamSynchronize(L.d2h_stream);
    if (e != cudaSuccess && rc == HG_OK) rc = cuda_fail(e, "result download");
    L.d2h_pending = false;
  }
  if (rc) {
    cudaDeviceSynchronize();
    return rc;
  }
  return read_device_error(c.lanes[0].stream);
}

int spectrum(uint64_t *a, size_t n, int mod_num, bool inverse, cudaStream_t st) {
  std::lock_guard<std::recursive_mutex> lock(g_ctx.mu);
  int rc = ensure_init();
  if (rc) return rc;
  if (!a) return fail(HG_ERR_ARG, "null pointer");
  if (mod_num < 0 || mod_num >= kPrimes) return fail(HG_ERR_ARG, "modulus index %d out of range", mod_num);
  if (n == 0 || (n & (n - 1))) return fail(HG_ERR_ARG, "length %zu is not a power of two", n);
  if (n == 1) return HG_OK;
  const int L = ilog2_ceil(n);
  rc = check_len(L);
  if (rc) return rc;
  PassArgs pa = base_args(L, 1);
  pa.data[0] = a;
  pa.prime_lo = mod_num;
  pa.nprimes = 1;
  pa.prime_stride = 0;
  const std::vector<PassPlan> plan = plan_passes(L);
  if (!inverse) {
    HG_CUDA(run_strided(pa, plan, false, st), "forward transform");
    HG_CUDA(run_contig(pa, plan.back(), kContigFwd, st), "forward transform");
  } else {
    HG_CUDA(run_contig(pa, plan.back(), kContigInv, st), "inverse transform");
    HG_CUDA(run_strided(pa, plan, true, st), "inverse transform");
  }
  if (inverse) {
    const uint64_t p = g_ctx.moduli[mod_num];
    ProfScope ps(HG_KC_OTHER, st, 16.0 * static_cast<double>(n));
    HG_CUDA(launch_scale(a, n, mont_h(invmod_h(n % p, p), p), g_ctx.pc[mod_num], st), "1/N scaling");
  }
  return HG_OK;
}

// ---- batches -------------------------------------------------------------

// Products of one transform length (and kind) run by one launch per pass.
// Candidate pass splits of a 2^L transform: the default plan and, for
// L >= 12, every contiguous block size T with the remaining L - T bits in
// as few strided passes of 4..8 bits as possible.
std::vector<std::vector<PassPlan>> plan_candidates(int L) {
  std::vector<std::vector<PassPlan>> out{plan_passes(L)};
  if (L < kTileBits) return out;
  for (int T = 4; T <= kTileBits; ++T) {
    const int rem = L - T;
    if (rem < 4) continue;
    const int k = (rem + 7) / 8;
    if (rem < 4 * k) continue;
    std::vector<PassPlan> v;
    int logS = L;
    for (int i = 0; i < k; ++i) {
      const int part = rem / k + (i < rem % k ? 1 : 0);
      logS -= part;
      v.push_back({part, logS, kTileBits});
    }
    // A strided pass over R rows needs columns of at least 2^(12 - logR)
    // words so that its 4096-word tile spans whole rows.
    if (logS + v.back().logR < kTileBits) continue;
    v.push_back({logS, 0, logS});
    bool same = v.size() == out[0].size();
    for (size_t i = 0; same && i < v.size(); ++i)
      same = v[i].logR == out[0][i].logR && v[i].logS == out[0][i].logS && v[i].logT == out[0][i].logT;
    if (!same) out.push_back(v);
  }
  return out;
}

// Schedules chosen by timing, keyed by (L, square, products in the group).
std::mutex g_tune_mu;
std::map<std::tuple<int, bool, uint64_t>, std::vector<PassPlan>> g_tuned;

}  // namespace
}  // namespace hg

struct hg_batch {
  hg::BatchPlan bp;
  hg::DevBuf d_desc, ws, flags, tickets;
  // The persistent schedule: its work list and its counters.
  std::vector<hg::PersistPhase> phases;
  uint64_t items = 0;
  uint64_t persist_flag_words = 0;
  hg::DevBuf d_phases, d_state;
  bool persistent = false;
};

namespace hg {
namespace {

// Enqueue group gi with the given schedule.  The group's ticket and flags
// must be zero.
int run_group(const BatchGroup &g, size_t gi, const BatchBufs &bb, const std::vector<PassPlan> &plan,
              cudaStream_t st) {
  const int nops = g.square ? 1 : 2;
  const uint64_t N = uint64_t(1) << g.L;
  const uint64_t slab = static_cast<uint64_t>(kPrimes) * N;
  const ProductDesc *d = bb.desc + g.first;
  uint64_t *ws = bb.ws;
  if (g.tails) HG_CUDA(launch_zero_tails(d, g.nprod, N, st), "zero tails");
  PassArgs a = base_args(g.L, nops);
  a.err = bb.err;
  a.batch = d;
  a.read_limbs = 1;
  a.nprod = g.nprod;
  a.ws_stride = slab;
  a.data[0] = ws;
  a.data[1] = ws + g.nprod * slab;
  HG_CUDA(run_strided(a, plan, false, st), "forward transform");
  PassArgs m = a;
  if (plan.size() > 1) m.read_limbs = 0;
  HG_CUDA(run_contig(m, plan.back(), g.square ? kContigSqr : kContigMul, st), "middle pass");
  PassArgs inv = base_args(g.L, 1);
  inv.err = bb.err;
  inv.batch = d;
  inv.nprod = g.nprod;
  inv.ws_stride = slab;
  inv.data[0] = ws;
  uint64_t sc[kPrimes];
  bool scaled = false;
  HG_CUDA(run_strided(inv, plan, true, st, prescale_factors(g.L, sc) ? sc : nullptr, &scaled), "inverse transform");
  ScanState ss;
  ss.ticket = bb.tickets + gi;
  ss.ticket_base = 0;
  ss.flags = bb.flags + g.flags_off;
  ss.epoch = 1;
  ss.err = bb.err;
  {
    ProfScope ps(HG_KC_CARRY, st, 32.0 * static_cast<double>(N) * static_cast<double>(g.nprod), 2);  // tiles + fix
    HG_CUDA(launch_crt_carry_batch(ws, slab, g.L, crt_const(g.L, scaled), d, g.nprod, ss, st), "reconstruction");
  }
  return HG_OK;
}

BatchBufs batch_bufs(hg_batch *b) {
  return BatchBufs{static_cast<const ProductDesc *>(b->d_desc.p), b->ws.u64(),
                   static_cast<unsigned long long *>(b->flags.p), static_cast<unsigned long long *>(b->tickets.p),
                   err_word()};
}

// ---- the persistent schedule (hg_persist.cu) -------------------------------
//
// Group workspaces and carry flags lie back to back (the groups run at the
// same time); the phases of each group follow run_group's launches one for
// one, with the same arguments.
constexpr uint64_t kPersistWorkspaceCap = uint64_t(16) << 30;  // bytes

struct PersistLayout {
  std::vector<uint64_t> ws_off, flag_off;  // per group, words
  uint64_t ws_words = 0, flag_words = 0;
};

PersistLayout persist_layout(const BatchPlan &bp) {
  PersistLayout l;
  for (const BatchGroup &g : bp.groups) {
    const uint64_t N = uint64_t(1) << g.L;
    l.ws_off.push_back(l.ws_words);
    l.flag_off.push_back(l.flag_words);
    l.ws_words += static_cast<uint64_t>(g.square ? 1 : 2) * kPrimes * N * g.nprod;
    l.flag_words += persist_carry_tiles(N) * g.nprod;
  }
  return l;
}

// The phases of one group, in dependency order.
std::vector<PersistPhase> group_phases(const BatchGroup &g, const BatchBufs &bb, uint64_t *ws,
                                       unsigned long long *flags, cudaStream_t st) {
  std::vector<PersistPhase> v;
  const int nops = g.square ? 1 : 2;
  const uint64_t N = uint64_t(1) << g.L;
  const uint64_t slab = static_cast<uint64_t>(kPrimes) * N;
  const ProductDesc *d = bb.desc + g.first;
  const std::vector<PassPlan> &plan = g.plan;
  const int np = static_cast<int>(plan.size()) - 1;
  auto phase = [](int kind, int sel, uint64_t count) {
    PersistPhase p{};
    p.kind = kind;
    p.sel = sel;
    p.count = count;
    p.dep = -1;
    return p;
  };
  PassArgs a = base_args(g.L, nops);
  a.err = bb.err;
  a.batch = d;
  a.read_limbs = 1;
  a.nprod = g.nprod;
  a.ws_stride = slab;
  a.data[0] = ws;
  a.data[1] = ws + g.nprod * slab;
  for (int s = 0; s < np; ++s) {
    PassArgs f = a;
    f.logR = plan[s].logR;
    f.logS = plan[s].logS;
    f.logT = plan[s].logT;
    f.tiles = N >> plan[s].logT;
    f.ptw = pass_twiddles(f.logR + f.logS, f.logR, false, st);
    PersistPhase p = phase(kPhaseStrided, f.logR, f.tiles * g.nprod * static_cast<uint64_t>(nops) * kPrimes);
    p.a = f;
    v.push_back(p);
    a.read_limbs = 0;
  }
  {
    PassArgs m = a;
    const int T = plan.back().logT;
    m.logR = T;
    m.logS = 0;
    m.logT = T;
    m.tiles = N >> T;
    const int mode = g.square ? kContigSqr : kContigMul;
    if (T < 4) {
      PersistPhase p = phase(kPhaseTiny, mode, (g.nprod * kPrimes + 255) / 256);
      p.a = m;
      v.push_back(p);
    } else {
      const uint64_t bpc = uint64_t(1) << (kTileBits - T);
      const uint64_t gx = (m.tiles * g.nprod + bpc - 1) / bpc;
      PersistPhase p = phase(kPhaseContig, T | (mode << 4), gx * kPrimes);
      p.gx = gx;
      p.a = m;
      v.push_back(p);
    }
  }
  PassArgs inv = base_args(g.L, 1);
  inv.err = bb.err;
  inv.batch = d;
  inv.nprod = g.nprod;
  inv.ws_stride = slab;
  inv.data[0] = ws;
  uint64_t sc[kPrimes];
  const bool can_scale = prescale_factors(g.L, sc);
  bool scaled = false;
  for (int s = 0; s < np; ++s) {
    const PassPlan &pp = plan[np - 1 - s];
    PassArgs f = inv;
    f.logR = pp.logR;
    f.logS = pp.logS;
    f.logT = pp.logT;
    f.tiles = N >> pp.logT;
    const bool last = s == np - 1;  // the last inverse pass: its table prescaled
    f.ptw = pass_twiddles(f.logR + f.logS, f.logR, true, st, last && can_scale ? sc : nullptr);
    if (last) scaled = can_scale && f.ptw;
    PersistPhase p = phase(kPhaseStrided, f.logR | 16, f.tiles * g.nprod * kPrimes);
    p.a = f;
    v.push_back(p);
  }
  PersistPhase c = phase(kPhaseCarry, 0, persist_carry_tiles(N) * g.nprod);
  c.res = ws;
  c.n = N;
  c.ws_stride = slab;
  c.cc = crt_const(g.L, scaled);
  c.batch = d;
  c.tpp = persist_carry_tiles(N);
  c.tiles = c.tpp * g.nprod;
  c.ss.ticket = nullptr;
  c.ss.ticket_base = 0;
  c.ss.flags = flags;
  c.ss.epoch = 1;
  c.ss.err = bb.err;
  v.push_back(c);
  PersistPhase f = c;
  f.kind = kPhaseFix;
  f.count = (c.tiles + 7) / 8;
  v.push_back(f);
  return v;
}

// Build the work list for the groups' current plans, or leave the batch on
// the per-pass schedule when it cannot run persistently (too many phases,
// or group workspaces that together exceed the cap).
int persist_build(hg_batch *b) {
  b->phases.clear();
  b->items = 0;
  const BatchPlan &bp = b->bp;
  if (bp.groups.empty() || !persist_grid()) return HG_OK;
  const PersistLayout l = persist_layout(bp);
  if (l.ws_words * 8 > kPersistWorkspaceCap) return HG_OK;
  if (b->ws.bytes < l.ws_words * 8) HG_CUDA(b->ws.ensure(l.ws_words * 8), "batch workspace");
  if (b->flags.bytes < l.flag_words * 8) HG_CUDA(b->flags.ensure(l.flag_words * 8), "batch scan flags");
  b->persist_flag_words = l.flag_words;
  const BatchBufs bb = batch_bufs(b);
  std::vector<std::vector<PersistPhase>> per;
  std::vector<PersistPhase> indep;  // zeroing: waits for nothing
  for (size_t gi = 0; gi < bp.groups.size(); ++gi) {
    const BatchGroup &g = bp.groups[gi];
    per.push_back(group_phases(g, bb, bb.ws + l.ws_off[gi], bb.flags + l.flag_off[gi], g_ctx.lane->stream));
    if (g.tails) {
      PersistPhase z{};
      z.kind = kPhaseZero;
      z.dep = -1;
      z.n = uint64_t(1) << g.L;
      z.batch = bb.desc + g.first;
      z.count = g.nprod;
      indep.push_back(z);
    }
  }
  if (bp.nzero) {
    PersistPhase z{};
    z.kind = kPhaseZero;
    z.dep = -1;
    z.n = 0;
    z.batch = bb.desc + bp.zero_first;
    z.count = bp.nzero;
    indep.push_back(z);
  }
  // Level by level across groups; each phase waits for its group's previous one.
  std::vector<PersistPhase> out = indep;
  std::vector<int> last(per.size(), -1);
  size_t levels = 0;
  for (const auto &v : per) levels = std::max(levels, v.size());
  for (size_t lv = 0; lv < levels; ++lv)
    for (size_t gi = 0; gi < per.size(); ++gi) {
      if (lv >= per[gi].size()) continue;
      PersistPhase p = per[gi][lv];
      p.dep = lv == 0 ? -1 : last[gi];
      last[gi] = static_cast<int>(out.size());
      out.push_back(p);
    }
  if (out.size() > static_cast<size_t>(kPersistMaxPhases)) return HG_OK;
  // Items of up to 8 units, but at least four items per CTA of the grid
  // where the phase has that many units.
  const uint64_t grid = static_cast<uint64_t>(persist_grid());
  uint64_t first = 0;
  for (PersistPhase &p : out) {
    p.units = p.count;
    p.per = std::max<uint64_t>(1, std::min<uint64_t>(8, p.units / (4 * grid)));
    p.count = (p.units + p.per - 1) / p.per;
    p.first = first;
    first += p.count;
  }
  HG_CUDA(b->d_phases.ensure(out.size() * sizeof(PersistPhase)), "batch work list");
  HG_CUDA(cudaMemcpy(b->d_phases.p, out.data(), out.size() * sizeof(PersistPhase), cudaMemcpyHostToDevice),
          "batch work list upload");
  HG_CUDA(b->d_state.ensure(persist_state_bytes(static_cast<int>(out.size()))), "batch work counters");
  b->phases.swap(out);
  b->items = first;
  return HG_OK;
}

int persist_run(hg_batch *b, cudaStream_t st) {
  const BatchBufs bb = batch_bufs(b);
  if (b->persist_flag_words)
    HG_CUDA(cudaMemsetAsync(bb.flags, 0, b->persist_flag_words * 8, st), "scan flags reset");
  ProfScope ps(HG_KC_BATCH, st, 0.0);
  HG_CUDA(launch_persist(static_cast<const PersistPhase *>(b->d_phases.p), static_cast<int>(b->phases.size()),
                         b->items, static_cast<PersistState *>(b->d_state.p), bb.err, st),
          "persistent batch");
  return HG_OK;
}

int batch_clear_scan(const BatchPlan &bp, const BatchBufs &bb, cudaStream_t st) {
  if (bp.flag_words) HG_CUDA(cudaMemsetAsync(bb.flags, 0, bp.flag_words * 8, st), "scan flags reset");
  if (!bp.groups.empty()) HG_CUDA(cudaMemsetAsync(bb.tickets, 0, bp.groups.size() * 8, st), "scan tickets reset");
  return HG_OK;
}

// Time each candidate schedule of each group (twice; the second run counts)
// and keep the fastest.
int batch_autotune(hg_batch *b) {
  cudaStream_t st = g_ctx.lane->stream;
  cudaEvent_t e0, e1;
  HG_CUDA(cudaEventCreate(&e0), "event creation");
  HG_CUDA(cudaEventCreate(&e1), "event creation");
  int rc = HG_OK;
  const BatchBufs bb = batch_bufs(b);
  for (size_t gi = 0; gi < b->bp.groups.size() && rc == HG_OK; ++gi) {
    BatchGroup &g = b->bp.groups[gi];
    const auto key = std::make_tuple(g.L, g.square, g.nprod);
    {
      std::lock_guard<std::mutex> lk(g_tune_mu);
      auto it = g_tuned.find(key);
      if (it != g_tuned.end()) {
        g.plan = it->second;
        continue;
      }
    }
    const auto cands = plan_candidates(g.L);
    float best = 1e30f;
    for (const auto &plan : cands) {
      float ms = 0;
      for (int rep = 0; rep < 2 && rc == HG_OK; ++rep) {
        if ((rc = batch_clear_scan(b->bp, bb, st))) break;
        cudaEventRecord(e0, st);
        if ((rc = run_group(g, gi, bb, plan, st))) break;
        cudaEventRecord(e1, st);
        if (cudaEventSynchronize(e1) != cudaSuccess) rc = fail(HG_ERR_CUDA, "autotune timing failed");
        else cudaEventElapsedTime(&ms, e0, e1);
      }
      if (rc) break;
      if (ms < best) {
        best = ms;
        g.plan = plan;
      }
    }
    if (rc == HG_OK) {
      std::lock_guard<std::mutex> lk(g_tune_mu);
      g_tuned[key] = g.plan;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (rc == HG_OK) rc = read_device_error(st);
  return rc;
}

// Time the whole batch on both schedules (twice each; the second run
// counts) and keep the faster.
int schedule_autotune(hg_batch *b) {
  cudaStream_t st = g_ctx.lane->stream;
  cudaEvent_t e0, e1;
  HG_CUDA(cudaEventCreate(&e0), "event creation");
  HG_CUDA(cudaEventCreate(&e1), "event creation");
  int rc = HG_OK;
  float ms[2] = {0, 0};
  for (int sched = 0; sched < 2 && rc == HG_OK; ++sched) {
    b->persistent = sched == 1;
    for (int rep = 0; rep < 2 && rc == HG_OK; ++rep) {
      cudaEventRecord(e0, st);
      rc = b->persistent ? persist_run(b, st) : enqueue_batch(b->bp, batch_bufs(b), st);
      if (rc) break;
      cudaEventRecord(e1, st);
      if (cudaEventSynchronize(e1) != cudaSuccess) rc = fail(HG_ERR_CUDA, "schedule timing failed");
      else cudaEventElapsedTime(&ms[sched], e0, e1);
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (rc == HG_OK) rc = read_device_error(st);
  b->persistent = ms[1] <= ms[0];
  return rc;
}

constexpr uint64_t kBatchWorkspaceCap = uint64_t(4) << 30;  // bytes per group chunk

// Validate the C-ABI product list into descriptors.
int product_descs(const hg_product *prods, size_t n, std::vector<ProductDesc> &out) {
  if (n && !prods) return fail(HG_ERR_ARG, "null pointer");
  out.clear();
  out.reserve(n);
  for (size_t i = 0; i < n; ++i) {
    const hg_product &p = prods[i];
    const bool square = p.y == nullptr;
    const uint64_t size = square ? 2 * p.nx : p.nx + p.ny;
    if (!p.out || (p.nx && !p.x)) return fail(HG_ERR_ARG, "product %zu: null pointer", i);
    if (p.nout < size) return fail(HG_ERR_ARG, "product %zu: nout = %zu cannot hold %llu limbs", i, p.nout,
                                   (unsigned long long)size);
    if (p.nx && (square || p.ny)) {
      int rc = check_len(ilog2_ceil(size));
      if (rc) return rc;
    }
    out.push_back(ProductDesc{p.x, p.y, p.nx, square ? p.nx : p.ny, p.out, p.nout});
  }
  return HG_OK;
}

int batch_create(const hg_product *prods, size_t n, int flags, hg_batch **out) {
  if (!out) return fail(HG_ERR_ARG, "null pointer");
  *out = nullptr;
  std::vector<ProductDesc> items;
  int rc = product_descs(prods, n, items);
  if (rc) return rc;
  std::unique_ptr<hg_batch> b(new hg_batch());
  if ((rc = plan_batch(items.data(), items.size(), kBatchWorkspaceCap, b->bp))) return rc;
  const BatchPlan &bp = b->bp;
  if (!bp.desc.empty()) {
    HG_CUDA(b->d_desc.ensure(bp.desc.size() * sizeof(ProductDesc)), "batch descriptors");
    HG_CUDA(cudaMemcpy(b->d_desc.p, bp.desc.data(), bp.desc.size() * sizeof(ProductDesc), cudaMemcpyHostToDevice),
            "batch descriptors upload");
  }
  if (bp.ws_words) HG_CUDA(b->ws.ensure(bp.ws_words * 8), "batch workspace");
  if (bp.flag_words) HG_CUDA(b->flags.ensure(bp.flag_words * 8), "batch scan flags");
  HG_CUDA(b->tickets.ensure(std::max<size_t>(1, bp.groups.size()) * 8), "batch tickets");
  if ((flags & HG_BATCH_PER_PASS) && (flags & HG_BATCH_PERSISTENT))
    return fail(HG_ERR_ARG, "a batch runs either per pass or persistently, not both");
  if (flags & HG_BATCH_AUTOTUNE) {
    if ((rc = batch_autotune(b.get()))) return rc;
  } else {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    for (BatchGroup &g : b->bp.groups) {
      auto it = g_tuned.find(std::make_tuple(g.L, g.square, g.nprod));
      if (it != g_tuned.end()) g.plan = it->second;
    }
  }
  if (!(flags & HG_BATCH_PER_PASS)) {
    if ((rc = persist_build(b.get()))) return rc;
    b->persistent = b->items > 0;
    if ((flags & HG_BATCH_PERSISTENT) && !b->persistent && !b->bp.groups.empty())
      return fail(HG_ERR_ARG, "this batch cannot run as one persistent launch (more than %d phases, or group "
                              "workspaces above %llu bytes)", kPersistMaxPhases, (unsigned long long)kPersistWorkspaceCap);
    if ((flags & HG_BATCH_AUTOTUNE) && !(flags & HG_BATCH_PERSISTENT) && b->persistent &&
        (rc = schedule_autotune(b.get())))
      return rc;
  }
  *out = b.release();
  return HG_OK;
}

int batch_run(hg_batch *b, cudaStream_t st) {
  if (!b) return fail(HG_ERR_ARG, "null batch");
  if (b->persistent) return persist_run(b, st);
  return enqueue_batch(b->bp, batch_bufs(b), st);
}

}  // namespace

uint64_t product_workspace_bytes(uint64_t nx, uint64_t ny, bool square) {
  if (nx == 0 || (!square && ny == 0)) return 0;
  const uint64_t N = uint64_t(1) << ilog2_ceil(square ? 2 * nx : nx + ny);
  return static_cast<uint64_t>(square ? 1 : 2) * kPrimes * N * 8;
}

int plan_batch(const ProductDesc *items, size_t n, uint64_t ws_cap_bytes, BatchPlan &bp) {
  bp = BatchPlan();
  struct Item {
    int L;
    bool square;
    size_t i;
  };
  std::vector<Item> live;
  std::vector<size_t> zeros;
  live.reserve(n);
  for (size_t i = 0; i < n; ++i) {
    const ProductDesc &p = items[i];
    const bool square = p.y == nullptr;
    if (p.nx == 0 || p.ny == 0) {
      zeros.push_back(i);
      continue;
    }
    live.push_back({ilog2_ceil(p.nx + p.ny), square, i});
  }
  std::stable_sort(live.begin(), live.end(), [](const Item &a, const Item &c) {
    return a.L != c.L ? a.L < c.L : a.square < c.square;
  });
  bp.desc.reserve(n);
  for (size_t s = 0; s < live.size();) {
    size_t e = s;
    while (e < live.size() && live[e].L == live[s].L && live[e].square == live[s].square) ++e;
    const int L = live[s].L;
    const bool square = live[s].square;
    const uint64_t N = uint64_t(1) << L;
    const uint64_t per = static_cast<uint64_t>(square ? 1 : 2) * kPrimes * N * 8;
    if (per > ws_cap_bytes)
      return fail(HG_ERR_ARG, "a 2^%d-point product needs %llu workspace bytes, more than the %llu available", L,
                  (unsigned long long)per, (unsigned long long)ws_cap_bytes);
    const uint64_t chunk = std::max<uint64_t>(1, ws_cap_bytes / per);
    for (size_t c = s; c < e; c += chunk) {
      BatchGroup g;
      g.L = L;
      g.square = square;
      g.plan = plan_passes(L);
      g.first = bp.desc.size();
      g.nprod = std::min<uint64_t>(chunk, e - c);
      g.flags_off = bp.flag_words;
      for (size_t k = c; k < c + g.nprod; ++k) {
        bp.desc.push_back(items[live[k].i]);
        if (bp.desc.back().nout > N) g.tails = true;
      }
      bp.flag_words += carry_tiles(N) * g.nprod;
      bp.ws_words = std::max<uint64_t>(bp.ws_words, per / 8 * g.nprod);
      bp.groups.push_back(std::move(g));
    }
    s = e;
  }
  bp.zero_first = bp.desc.size();
  bp.nzero = zeros.size();
  for (size_t z : zeros) bp.desc.push_back(items[z]);
  return HG_OK;
}

int enqueue_batch(const BatchPlan &bp, const BatchBufs &bb, cudaStream_t st) {
  int rc = batch_clear_scan(bp, bb, st);
  if (rc) return rc;
  if (bp.nzero) HG_CUDA(launch_zero_tails(bb.desc + bp.zero_first, bp.nzero, 0, st), "zero products");
  for (size_t gi = 0; gi < bp.groups.size(); ++gi)
    if ((rc = run_group(bp.groups[gi], gi, bb, bp.groups[gi].plan, st))) return rc;
  return HG_OK;
}

std::recursive_mutex &lib_mutex() { return g_ctx.mu; }
bool lib_ready() { return g_ctx.ready; }
int large_sum_device(const uint64_t *a, uint64_t na, int64_t sa, const uint64_t *b, uint64_t nb, int64_t sb,
                     uint64_t *out, uint64_t nout, int64_t *result, cudaStream_t st) {
  std::lock_guard<std::recursive_mutex> lock(g_ctx.mu);
  int rc = ensure_init();
  if (rc) return rc;
  const uint64_t n = na > nb ? na : nb;
  const uint64_t nproc = sa != sb ? n : n + 1;
  HG_CUDA(ws_acquire(st), "workspace ordering");
  if (nout > nproc) HG_CUDA(cudaMemsetAsync(out + nproc, 0, (nout - nproc) * sizeof(uint64_t), st), "zero tail");
  ScanState ss;
  rc = scan_state(carry_tiles(nproc), &ss);
  if (rc) return rc;
  long long *top = reinterpret_cast<long long *>(static_cast<char *>(g_ctx.lane->misc.p) + 16);
  {
    // (top search,) local scan, fix, sign and size
    ProfScope ps(HG_KC_OTHER, st, 24.0 * static_cast<double>(nproc), sa != sb ? 4 : 3);
    HG_CUDA(launch_large_sum(a, na, sa, b, nb, sb, out, top, result, ss, st), "large sum");
  }
  HG_CUDA(ws_release(st), "workspace ordering");
  return HG_OK;
}

int lib_device() { return g_ctx.device; }

int lib_fail(int code, const char *fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  t_err = buf;
  return code;
}

int lib_cuda_fail(cudaError_t e, const char *what) { return cuda_fail(e, what); }

namespace {
std::atomic<int> g_services{0};
}  // namespace

void lib_service_count(int delta) { g_services += delta; }

}  // namespace hg

using namespace hg;

extern "C" {

int hg_batch_create(const hg_product *prods, size_t n, int flags, hg_batch **batch) {
  std::lock_guard<std::recursive_mutex> lock(g_ctx.mu);
  int rc = ensure_init();
  if (rc) return rc;
  return batch_create(prods, n, flags, batch);
}

int hg_batch_run(hg_batch *batch, void *stream) {
  std::lock_guard<std::recursive_mutex> lock(g_ctx.mu);
  int rc = ensure_init();
  if (rc) return rc;
  return batch_run(batch, static_cast<cudaStream_t>(stream));
}

int hg_batch_schedule(const hg_batch *batch, int *persistent, size_t *launches) {
  if (!batch || !persistent || !launches) return fail(HG_ERR_ARG, "null pointer");
  *persistent = batch->persistent ? 1 : 0;
  if (batch->persistent) {
    *launches = 1;
    return HG_OK;
  }
  size_t n = batch->bp.nzero ? 1 : 0;
  for (const hg::BatchGroup &g : batch->bp.groups)
    n += (g.tails ? 1 : 0) + 2 * (g.plan.size() - 1) + 1 + 2;  // zero tails, passes, middle, carry + fix
  *launches = n;
  return HG_OK;
}

int hg_batch_destroy(hg_batch *batch) {
  std::lock_guard<std::recursive_mutex> lock(g_ctx.mu);
  if (!batch) return HG_OK;
  batch->d_phases.release();
  batch->d_state.release();
  batch->d_desc.release();
  batch->ws.release();
  batch->flags.release();
  batch->tickets.release();
  delete batch;
  return HG_OK;
}

int hg_mul_batch_device(const hg_product *prods, size_t n, void *stream) {
  std::lock_guard<std::recursive_mutex> lock(g_ctx.mu);
  int rc = ensure_init();
  if (rc) return rc;
  hg_batch *b = nullptr;
  if ((rc = batch_create(prods, n, 0, &b))) return rc;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  rc = batch_run(b, st);
  if (rc == HG_OK && cudaStreamSynchronize(st) != cudaSuccess) rc = fail(HG_ERR_CUDA, "stream synchronise failed");
  hg_batch_destroy(b);
  return rc;
}

int hg_init(const uint64_t *moduli, int k, int device) {
  std::lock_guard<std::recursive_mutex> lock(g_ctx.mu);
  return init_locked(moduli, k, nullptr, 0, device);
}

int hg_init_scheme(const uint64_t *moduli, int k, const uint64_t *roots, int maxlg, int device) {
  std::lock_guard<std::recursive_mutex> lock(g_ctx.mu);
  return init_locked(moduli, k, roots, maxlg, device);
}

int hg_shutdown(void) {
  std::lock_guard<std::recursive_mutex> lock(g_ctx.mu);
  Context &c = g_ctx;
  if (!c.ready) return HG_OK;
  if (g_services.load() > 0) return fail(HG_ERR_ARG, "close every multiply service before hg_shutdown");
  cudaDeviceSynchronize();
  for (Lane &L : c.lanes) {
    L.A.release();
    L.B.release();
    L.X.release();
    L.Y.release();
    L.OUT.release();
    L.flags.release();
    L.misc.release();
    for (cudaStream_t *st : {&L.stream, &L.copy_stream, &L.d2h_stream}) {
      if (*st) cudaStreamDestroy(*st);
      *st = nullptr;
    }
    for (cudaEvent_t *e : {&L.ws_done, &L.copy_done, &L.carry_done, &L.d2h_done}) {
      if (*e) cudaEventDestroy(*e);
      *e = nullptr;
    }
    for (auto &op : L.slice_done)
      for (cudaEvent_t &e : op) {
        if (e) cudaEventDestroy(e);
        e = nullptr;
      }
    L.ws_pending = L.d2h_pending = false;
    L.ticket_count = 0;
    L.epoch = 0;
  }
  c.lane = &c.lanes[0];
  c.tables.release();
  release_pass_twiddles();
  c.ready = false;
  // The scratch array's device address belongs to the module as loaded in
  // the current context: after a context reset the module loads again, so
  // the next hg_mul_device_noalloc looks the address up afresh.
  for (uint64_t *&p : g_noalloc_ptr) p = nullptr;
  return HG_OK;
}

int hg_build_checked(void) { return HG_CHECKED ? 1 : 0; }

int hg_last_error(char *buf, size_t len) {
  if (!buf || len == 0) return HG_ERR_ARG;
  snprintf(buf, len, "%s", t_err.c_str());
  return HG_OK;
}

int hg_scheme_moduli(uint64_t *out, int cap) {
  std::vector<uint64_t> dm = default_moduli_h();
  for (int i = 0; i < cap && i < static_cast<int>(dm.size()); ++i) out[i] = dm[i];
  return static_cast<int>(dm.size());
}

size_t hg_ntt_length(size_t nx, size_t ny) {
  const size_t s = nx + ny;
  size_t r = 1;
  while (r < s) r <<= 1;
  return r;
}

int hg_chunk_plan(size_t nx, size_t ny, int *log_len, size_t *chunk, size_t *nchunks) {
  if (!log_len || !chunk || !nchunks) return 0;
  hg::ChunkPlan cp;
  if (!hg::plan_chunks(std::max(nx, ny), std::min(nx, ny), cp)) return 0;
  *log_len = cp.L;
  *chunk = cp.chunk;
  *nchunks = cp.nchunks;
  return 1;
}

int hg_set_chunking(int enable) { return hg::g_chunking.exchange(enable ? 1 : 0); }

int hg_mul_host_pipeline(const hg_host_product *prods, size_t n) { return host_pipeline(prods, n); }

int hg_mul(const uint64_t *x, size_t nx, const uint64_t *y, size_t ny, uint64_t *out, size_t nout) {
  return host_product(Kind::Ntt, x, nx, y, ny, 0, out, nout);
}

int hg_sqr(const uint64_t *x, size_t nx, uint64_t *out, size_t nout) {
  return host_product(Kind::Square, x, nx, nullptr, 0, 0, out, nout);
}

int hg_mul_schoolboy(const uint64_t *x, size_t nx, const uint64_t *y, size_t ny, uint64_t *out, size_t nout) {
  return host_product(Kind::Schoolboy, x, nx, y, ny, 0, out, nout);
}

int hg_mul_digit(const uint64_t *x, size_t nx, uint64_t d, uint64_t *out, size_t nout) {
  return host_product(Kind::Digit, x, nx, nullptr, 0, d, out, nout);
}

int hg_mpz_mul(const uint64_t *x, size_t nx, int sx, const uint64_t *y, size_t ny, int sy, int same_object,
               size_t threshold, uint64_t *out, size_t nout, size_t *nres, int *sres) {
  if (!nres || !sres || !out || (nx && !x) || (ny && !y)) return fail(HG_ERR_ARG, "null pointer");
  nx = trimmed(x, nx);
  ny = trimmed(y, ny);
  if (nx < ny) {  // rotatef so that |x| >= |y| (src/multiply.lisp:15-16)
    std::swap(x, y);
    std::swap(nx, ny);
    std::swap(sx, sy);
  }
  int rc = HG_OK;
  int sign = sx * sy;
  if (ny == 0) {  // (src/multiply.lisp:21-22)
    *nres = 0;
    *sres = 1;
    return HG_OK;
  }
  if (ny == 1) {  // (src/multiply.lisp:23-36)
    const uint64_t d = y[0];
    if (d == 1) {
      if (nout < nx) return fail(HG_ERR_ARG, "nout too small");
      memmove(out, x, nx * sizeof(uint64_t));
      sign = (sy == -1) ? -sx : sx;
    } else {
      rc = hg_mul_digit(x, nx, d, out, nout);
    }
  } else if (ny <= threshold) {  // (src/multiply.lisp:37-42)
    rc = hg_mul_schoolboy(x, nx, y, ny, out, nout);
  } else if (same_object) {  // (src/multiply.lisp:43-44)
    rc = hg_sqr(x, nx, out, nout);
    sign = 1;
  } else {  // (src/multiply.lisp:48-49)
    rc = hg_mul(x, nx, y, ny, out, nout);
  }
  if (rc) return rc;
  *nres = trimmed(out, nout);
  *sres = *nres ? sign : 1;
  return HG_OK;
}

int hg_mul_device(const uint64_t *x, size_t nx, const uint64_t *y, size_t ny, uint64_t *out, size_t nout,
                  void *stream) {
  std::lock_guard<std::recursive_mutex> lock(g_ctx.mu);
  int rc = ensure_init();
  if (rc) return rc;
  return ntt_product_device(x, nx, y, ny, out, nout, static_cast<cudaStream_t>(stream));
}

int hg_sqr_device(const uint64_t *x, size_t nx, uint64_t *out, size_t nout, void *stream) {
  std::lock_guard<std::recursive_mutex> lock(g_ctx.mu);
  int rc = ensure_init();
  if (rc) return rc;
  return ntt_product_device(x, nx, nullptr, 0, out, nout, static_cast<cudaStream_t>(stream));
}

int hg_mul_device_noalloc(const uint64_t *x, size_t nx, const uint64_t *y, size_t ny, uint64_t *out, size_t nout,
                          void *stream) {
  std::lock_guard<std::recursive_mutex> lock(g_ctx.mu);
  if (!g_ctx.ready) return fail(HG_ERR_NOT_INIT, "hg_mul_device_noalloc: call hg_init first");
  return noalloc_product_device(x, nx, y, ny, out, nout, static_cast<cudaStream_t>(stream));
}

int hg_mul_schoolboy_device(const uint64_t *x, size_t nx, const uint64_t *y, size_t ny, uint64_t *out, size_t nout,
                            void *stream) {
  std::lock_guard<std::recursive_mutex> lock(g_ctx.mu);
  int rc = ensure_init();
  if (rc) return rc;
  if (!y) return fail(HG_ERR_ARG, "null pointer");
  return small_product_device(x, nx, y, ny, 0, out, nout, static_cast<cudaStream_t>(stream));
}

int hg_butterfly_peak(double *butterflies_per_s) {
  std::lock_guard<std::recursive_mutex> lock(g_ctx.mu);
  int rc = ensure_init();
  if (rc) return rc;
  if (!butterflies_per_s) return fail(HG_ERR_ARG, "null pointer");
  return butterfly_peak(butterflies_per_s, g_ctx.pc[0], g_ctx.tb[0].sub_fwd);
}

int hg_sync(void *stream) {
  std::lock_guard<std::recursive_mutex> lock(g_ctx.mu);
  int rc = ensure_init();
  if (rc) return rc;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (!st) {
    HG_CUDA(cudaDeviceSynchronize(), "device synchronise");
    st = g_ctx.lane->stream;
  }
  return read_device_error(st);
}

int hg_ntt_forward_device(uint64_t *a, size_t n, int mod_num, void *stream) {
  return spectrum(a, n, mod_num, false, static_cast<cudaStream_t>(stream));
}

int hg_ntt_reverse_device(uint64_t *a, size_t n, int mod_num, void *stream) {
  return spectrum(a, n, mod_num, true, static_cast<cudaStream_t>(stream));
}

int hg_profile_enable(int on) {
  std::lock_guard<std::mutex> lk(g_prof.mu);
  g_prof.on = on != 0;
  return HG_OK;
}

int hg_profile_read(uint64_t *launches, double *ms, double *bytes, int cap) {
  std::vector<ProfRecord> recs;
  uint64_t l[HG_KC_COUNT];
  double b[HG_KC_COUNT];
  {
    std::lock_guard<std::mutex> lk(g_prof.mu);
    recs.swap(g_prof.recs);
    for (int i = 0; i < HG_KC_COUNT; ++i) {
      l[i] = g_prof.launches[i];
      b[i] = g_prof.bytes[i];
      g_prof.launches[i] = 0;
      g_prof.bytes[i] = 0;
    }
  }
  double t[HG_KC_COUNT] = {};
  int rc = HG_OK;
  for (const ProfRecord &r : recs) {
    float dt = 0;
    if (cudaEventSynchronize(r.e) == cudaSuccess && cudaEventElapsedTime(&dt, r.b, r.e) == cudaSuccess)
      t[r.cls] += dt;
    else
      rc = fail(HG_ERR_CUDA, "profiling event failed");
    cudaEventDestroy(r.b);
    cudaEventDestroy(r.e);
  }
  for (int i = 0; i < cap && i < HG_KC_COUNT; ++i) {
    if (launches) launches[i] = l[i];
    if (ms) ms[i] = t[i];
    if (bytes) bytes[i] = b[i];
  }
  return rc;
}

}  // extern "C"
