/*
 * hypergeometrica_gb300.h -- C ABI of the GB300 exact multiplication library.
 *
 * This is the drop-in boundary for hypergeometrica's in-core multiplication
 * path.  In the Common Lisp reference, MPZ multiplication goes through the
 * generic mpz-* (src/mpz-protocol.lisp:74), whose method on two mpz/ram
 * (src/multiply.lisp:12-49) picks by-digit, schoolboy, squaring
 * (mpz-square, src/ntt-multiply.lisp:101-172) or the three-prime NTT product
 * (src/ntt-multiply.lisp:174-254).  A CFFI binding replaces those functions
 * with the entry points below; operands arrive as the raw uint64_t digit
 * pointers that vec-digit-pointer hands out (src/vec.lisp:17-19), little-
 * endian 64-bit limbs, magnitude only (the sign stays on the Lisp side).
 *
 * Conventions
 *  - Every entry point returns HG_OK (0) or a negative HG_ERR_* code; the
 *    message of the last failure on the calling thread is available from
 *    hg_last_error().  There is no CPU fallback: a failure is an error.
 *  - Sizes are limb counts.  High zero limbs of an operand are ignored
 *    (mpz-size, src/vec.lisp:218-229).
 *  - Products are exact.  out receives the magnitude in its low limbs and
 *    zeros up to nout; nout must hold the product (at least nx + ny limbs).
 *  - Host entry points take host pointers (pinned memory is fastest) and
 *    return when out is written.  *_device entry points take device
 *    pointers and a cudaStream_t (NULL = the legacy default stream), enqueue
 *    work and return; errors detected on the device surface at the next
 *    hg_sync().
 *  - The library is thread-safe: host entry points serialise on an internal
 *    lock; device entry points must not be called concurrently on the same
 *    stream from two threads.
 */
#ifndef HYPERGEOMETRICA_GB300_H
#define HYPERGEOMETRICA_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define HG_OK 0
#define HG_ERR_ARG (-1)          /* bad argument (null pointer, nout too small, ...)        */
#define HG_ERR_MODULI (-2)       /* the scheme cannot hold the convolution                  */
                                 /* (num-moduli-needed-for-bits, src/moduli.lisp:362-364)   */
#define HG_ERR_OOM (-3)          /* device or pinned memory exhausted                        */
#define HG_ERR_CUDA (-4)         /* a CUDA runtime call failed                               */
#define HG_ERR_INCONSISTENT (-5) /* a carry ran past the result storage                      */
                                 /* (add-big-digit, src/ntt-multiply.lisp:19-22)            */
#define HG_ERR_TIMEOUT (-6)      /* a bounded wait for the multiply service gave up          */
#define HG_ERR_NOT_INIT (-7)     /* hg_init failed or was given foreign moduli               */

/* Library initialisation.  Replaces the load-time construction of the
 * global **scheme** (src/ntt-multiply.lisp:8, make-modular-scheme of
 * default-moduli, src/moduli.lisp:257-353).  moduli/k may be NULL/0 to
 * accept the built-in scheme; otherwise they must be the reference's scheme
 * moduli (any order), which the library checks against its own tables.
 * device selects the CUDA device (-1 = current).  Called implicitly by the
 * first entry point when not called explicitly. */
int hg_init(const uint64_t *moduli, int k, int device);

/* hg_init that also checks the caller's table of primitive roots against the
 * library's (make-modular-scheme's primitive-roots, src/moduli.lisp:302-353):
 * roots[i * (maxlg + 1) + q] is w_{2^q}, the primitive 2^q-th root of unity
 * modulo moduli[i] (the Lisp table's entry [q][i][0][0]), for q = 0 .. maxlg,
 * maxlg <= 55.  A scheme built with another generator would give other
 * spectra; any root that differs from the one the library's device tables
 * are built from fails with HG_ERR_NOT_INIT before anything is allocated.
 * roots may be NULL (then this is hg_init). */
int hg_init_scheme(const uint64_t *moduli, int k, const uint64_t *roots, int maxlg, int device);

/* Release every device buffer, stream and table held by the library. */
int hg_shutdown(void);

/* Copy the message of the last error on this thread into buf. */
int hg_last_error(char *buf, size_t len);

/* 1 when this library is the checked build (libhg_gb300_checked.so), which
 * does what the reference does under :hypergeometrica-safe and -paranoid
 * (src/config.lisp:31-37): every residue a pass reads or writes is checked
 * against its range (ntt-forward's input assertion,
 * src/number-theoretic-transform.lisp:63-64), every residue index against
 * its array, and every modular product against an exact reduction of the
 * 128-bit product (the paranoid re-check of the reference's Shoup product,
 * src/modular-arithmetic.lisp:228-229).
 * A failed check is reported by the next hg_sync (or host-memory call) as
 * HG_ERR_INCONSISTENT.  0 for the regular build. */
int hg_build_checked(void);

/* Number of moduli and their values, largest first (scheme-moduli). */
int hg_scheme_moduli(uint64_t *out, int cap);

// Transform length mpz-*/ntt uses for trimmed sizes nx, ny: the least power
// of two >= nx + ny (src/ntt-multiply.lisp:175-176).  mpz-square uses
// hg_ntt_length(nx, nx) (:103).
size_t hg_ntt_length(size_t nx, size_t ny);

// How hg_mul, hg_mul_device and hg_mpz_mul run an unbalanced product (no
// counterpart in the reference, whose mpz-*/ntt always runs one transform of
// hg_ntt_length(nx, ny) points).  Returns 1 when the longer operand is cut
// into *nchunks chunks of *chunk limbs, each multiplied by the shorter one
// with transforms of 2^*log_len points (the result is the same integer);
// 0 when the product runs as one transform, or on a null pointer.  Host
// arithmetic only: needs no device and no hg_init.
int hg_chunk_plan(size_t nx, size_t ny, int *log_len, size_t *chunk, size_t *nchunks);

// Whether unbalanced products may run in chunks (hg_chunk_plan); on by
// default.  With 0 every product runs as the reference's one transform of
// hg_ntt_length(nx, ny) points.  Returns the previous setting.  Process-wide;
// takes effect for products enqueued after it returns.  No counterpart in
// the reference.
int hg_set_chunking(int enable);

/* ---- products on host memory ------------------------------------------ */

// mpz-*/ntt (src/ntt-multiply.lisp:174-254): |x| * |y| through the three-prime
// NTT.  Replaces the Lisp function of that name.
int hg_mul(const uint64_t *x, size_t nx, const uint64_t *y, size_t ny, uint64_t *out, size_t nout);

/* mpz-square (src/ntt-multiply.lisp:101-172): |x|^2. */
int hg_sqr(const uint64_t *x, size_t nx, uint64_t *out, size_t nout);

/* Many NTT products or squares (mpz-*-ntt and mpz-square, src/ntt-multiply.lisp:101-254) on
 * host memory in one call, pipelined: while one product's result is copied
 * down, the next product's operands go up and its transforms run, in a
 * second set of device buffers.  Each product is computed exactly as hg_mul
 * (hg_sqr when y is NULL) computes it; out receives the product and zeros
 * up to nout.  Returns once every result is in host memory.  The copies
 * overlap only for page-locked (pinned) buffers.  Products that share an
 * output buffer must be at least two apart in the list (products two apart
 * are written in list order); the first product of a new size allocates
 * that size's device buffers. */
typedef struct hg_host_product {
    const uint64_t *x; /* host limbs                          */
    size_t nx;
    const uint64_t *y; /* host limbs; NULL squares x          */
    size_t ny;
    uint64_t *out;     /* host result, nout >= nx + ny limbs (2nx square) */
    size_t nout;
} hg_host_product;
int hg_mul_host_pipeline(const hg_host_product *prods, size_t n);

/* %multiply-storage/schoolboy (src/mpz-ram.lisp:404-431): |x| * |y| by the
 * quadratic method, used by mpz-* when the smaller operand has at most
 * *ntt-multiply-threshold* limbs (src/multiply.lisp:37-42). */
int hg_mul_schoolboy(const uint64_t *x, size_t nx, const uint64_t *y, size_t ny, uint64_t *out, size_t nout);

/* mpz-multiply-by-digit! (src/mpz-ram.lisp:367-395) as mpz-* uses it for a
 * one-limb operand (src/multiply.lisp:23-36): |x| * d. */
int hg_mul_digit(const uint64_t *x, size_t nx, uint64_t d, uint64_t *out, size_t nout);

/* The whole mpz-* method on two mpz/ram (src/multiply.lisp:12-49), signs
 * included: zero, by-digit, schoolboy (smaller operand <= threshold limbs),
 * squaring when same_object (the (eq x y) test), else the NTT product.
 * Writes the trimmed magnitude to out, its length to *nres and the sign
 * (+1/-1; +1 for zero) to *sres.  sx, sy are +1 or -1. */
int hg_mpz_mul(const uint64_t *x, size_t nx, int sx, const uint64_t *y, size_t ny, int sy, int same_object,
               size_t threshold, uint64_t *out, size_t nout, size_t *nres, int *sres);

/* ---- products on device memory ---------------------------------------- */

/* hg_mul / hg_sqr / hg_mul_schoolboy on device pointers, enqueued on stream. */
int hg_mul_device(const uint64_t *x, size_t nx, const uint64_t *y, size_t ny, uint64_t *out, size_t nout,
                  void *stream);
int hg_sqr_device(const uint64_t *x, size_t nx, uint64_t *out, size_t nout, void *stream);
int hg_mul_schoolboy_device(const uint64_t *x, size_t nx, const uint64_t *y, size_t ny, uint64_t *out,
                            size_t nout, void *stream);

/* ---- products without allocation -------------------------------------- */

/* Largest product (nx + ny limbs, transform length 2^16) that
 * hg_mul_device_noalloc accepts. */
#define HG_NOALLOC_MAX_LIMBS 65536

/* No counterpart in the reference: hypergeometrica allocates its transform
 * storage per product.  Same result as hg_mul_device (hg_sqr_device when y
 * is NULL) for products of at most HG_NOALLOC_MAX_LIMBS limbs, computed in a
 * 3 MiB scratch array compiled into the library, so the call makes no
 * device or pinned allocation.  It is for callers that must not allocate
 * while they run: a cudaMalloc or cudaFree synchronises the whole device,
 * and a process that has handed its device memory to its own pool or arena
 * may have none left for the library's grow-only workspace.
 *
 *  - hg_init must have succeeded first (HG_ERR_NOT_INIT otherwise); the call
 *    never initialises the library itself, because that allocates.
 *  - The first call on a device does a one-time setup: with the library's
 *    device current it looks up the scratch array's device address
 *    (cudaGetSymbolAddress).  Make that first call before any stream
 *    capture begins.  A call with another device current is HG_ERR_ARG.
 *  - nx + ny > HG_NOALLOC_MAX_LIMBS is rejected with HG_ERR_ARG before
 *    anything is enqueued.
 *  - The carry scan's ticket and flag words in the scratch must be zero
 *    when its kernel starts; the call clears them on stream itself
 *    (cudaMemsetAsync), so the caller zeroes nothing.
 *  - There is one scratch array per device, shared by every call: calls
 *    whose work can overlap on the GPU (different streams without an event
 *    between them, or several host threads) race and corrupt each other's
 *    results.  Issue them on one stream, or order them with events.
 *    hg_mul_device and the batch API use other storage and do not race
 *    with it.
 *  - Errors found on the device (a carry out of the top of out, which no
 *    exact product causes) latch the library's device error word, which the
 *    next hg_sync reports; the call itself reports only host-side errors.
 *  - hg_shutdown forgets the scratch address: after a reset of the device's
 *    context, call hg_shutdown and hg_init around it, and the next call looks
 *    the address up again. */
int hg_mul_device_noalloc(const uint64_t *x, size_t nx, const uint64_t *y, size_t ny, uint64_t *out, size_t nout,
                          void *stream);

/* No counterpart in the reference (measurement): the rate, in radix-2
 * butterflies per second, of a memory-free network of the library's modular
 * butterflies (half forward DIF, half inverse DIT) over every SM: the
 * integer-pipe ceiling the NTT passes are measured against. */
int hg_butterfly_peak(double *butterflies_per_s);

/* Wait for the library's work on stream (NULL = all of it) and report any
 * error latched on the device since the last hg_sync. */
int hg_sync(void *stream);

/* ---- batches of products on device memory ----------------------------
 * No counterpart in the reference, which multiplies one pair at a time.  Its
 * binary splitting issues thousands of independent products per tree level
 * (combine, src/binary-splitting.lisp:112-121); a batch runs them together:
 * products are grouped by transform length.  By default the whole batch
 * runs as one persistent launch: a fixed grid of CTAs walks a device work
 * list of (group, pass, tile) items, each group's passes in order and the
 * groups overlapping.  The per-pass schedule instead runs each group as one
 * launch per NTT pass.  HG_BATCH_AUTOTUNE times the candidate pass splits
 * of each length, and then both schedules on the whole batch, and keeps the
 * fastest.  hg_batch_run enqueues kernels and memsets only, so it can be
 * captured in a CUDA graph and replayed; a batch owns its workspace, so
 * batches on different streams may overlap. */
typedef struct hg_product {
    const uint64_t *x; /* device limbs                                   */
    size_t nx;
    const uint64_t *y; /* device limbs; NULL squares x (mpz-square)      */
    size_t ny;
    uint64_t *out;     /* device result, nout >= nx + ny limbs (2nx square) */
    size_t nout;
} hg_product;

typedef struct hg_batch hg_batch;
#define HG_BATCH_AUTOTUNE 1   /* time the candidate pass splits and both schedules */
#define HG_BATCH_PER_PASS 2   /* run one launch per pass per group (no persistent launch) */
#define HG_BATCH_PERSISTENT 4 /* run as one persistent launch; HG_ERR_ARG if it cannot */

/* Plan a batch (sizes as given: device operands are not trimmed), allocate
 * its workspace and, with HG_BATCH_AUTOTUNE, run each group once per
 * candidate schedule to pick the fastest.  Must not be called while a
 * stream is being captured. */
int hg_batch_create(const hg_product *prods, size_t n, int flags, hg_batch **batch);
/* Enqueue every product of the batch on stream. */
int hg_batch_run(hg_batch *batch, void *stream);
/* The schedule a batch runs: *persistent = 1 for the one persistent launch,
 * 0 for one launch per pass; *launches = kernel launches per hg_batch_run. */
int hg_batch_schedule(const hg_batch *batch, int *persistent, size_t *launches);
/* Free a batch (after its work has completed). */
int hg_batch_destroy(hg_batch *batch);
/* One-shot: create (no tuning, schedules from earlier tuning are reused),
 * run on stream, wait, destroy. */
int hg_mul_batch_device(const hg_product *prods, size_t n, void *stream);

/* ---- sums and sizes of many device integers ---------------------------- */

/* One signed sum: out = sa*|a| + sb*|b| (magnitude), nout >= max(na, nb) + 1. */
typedef struct hg_sum {
    const uint64_t *a; /* device limbs */
    size_t na;
    const uint64_t *b; /* device limbs */
    size_t nb;
    uint64_t *out;     /* device limbs; written up to nout */
    size_t nout;
    int64_t sa, sb;    /* +1 or -1 */
} hg_sum;

/* mpz-+ (src/mpz-ram.lisp:292-306) on n pairs at once: result[2k] receives
 * the sign of sum k (+1 for zero) and result[2k + 1] its length without high
 * zero limbs (device int64 array of 2n entries).  Sums shorter than 2^15
 * limbs run one CTA each; longer ones run one at a time over the whole GPU
 * (a carry-lookahead scan ordered with the library's products). */
int hg_add_batch_device(const hg_sum *sums, size_t n, int64_t *result, void *stream);

/* Largest operand of hg_mul_small_batch_device. */
#define HG_SMALL_MAX_LIMBS 64

/* %multiply-storage/schoolboy (src/mpz-ram.lisp:404-431) on n small device
 * products at once (operands of at most HG_SMALL_MAX_LIMBS limbs; y NULL
 * squares x), one thread per product: out[0, nx + ny) the product, zeros up
 * to nout.  The mpz-* dispatch sends products with a smaller operand of at
 * most 100 limbs this way (src/multiply.lisp:37-42); binary splitting's
 * lowest tree levels consist of them. */
int hg_mul_small_batch_device(const hg_product *prods, size_t n, void *stream);

typedef struct hg_vec {
    const uint64_t *p; /* device limbs */
    size_t n;
} hg_vec;

/* mpz-size (vec-digit-length*, src/vec.lisp:218-229) of n device integers:
 * sizes[k] = length of vecs[k] without high zero limbs (device array). */
int hg_trim_batch_device(const hg_vec *vecs, size_t n, uint64_t *sizes, void *stream);

/* ---- binary-splitting base cases -------------------------------------- */

/* An integer polynomial coef[0] + coef[1] k + ... + coef[degree] k^degree
 * (degree 0..7); when has_zero_value is nonzero its value at k = 0 is
 * zero_value instead (the reference's "(if (zerop n) 1 ...)"). */
typedef struct hg_poly {
    int64_t coef[8];
    int32_t degree;
    int32_t has_zero_value;
    int64_t zero_value;
} hg_poly;

/* binary-split-base-case=1 (src/binary-splitting.lisp:102-110) for the
 * terms k = lower .. lower + count - 1 of a series whose a, b, p, q are the
 * polynomials polys[0..3]: P = p(k), Q = q(k), B = b(k), R = p(k) a(k).
 * Value j of term i goes to limbs[(j count + i) 4 .. + 3] (four limbs,
 * magnitude) and sign_size[(j count + i) 2] = sign (+1 for zero),
 * [.. + 1] = length without high zero limbs (device arrays).  Every value and
 * R must fit in 255 bits; the caller checks the bound. */
int hg_series_leaves_device(const hg_poly *polys, uint64_t lower, uint64_t count, uint64_t *limbs,
                            int64_t *sign_size, void *stream);

/* binary-split (src/binary-splitting.lisp:112-133) of whole nodes: the
 * partial P, Q, B, R over terms [ranges[2 i], ranges[2 i + 1]) for each of
 * the n nodes, one device thread per node folding its terms left to right
 * (a range's partial is the same integers however the range is split).
 * Value j of node i goes to limbs[(j n + i) width ..] (magnitude) and
 * sign_size[(j n + i) 2] = sign (+1 for zero), [.. + 1] = length without
 * high zero limbs, or -1 when a value would need more than width limbs.
 * scratch holds 2 n width words.  All arrays are device memory.  Every
 * term's values and p(k) a(k) must fit in 255 bits, as for
 * hg_series_leaves_device. */
int hg_series_nodes_device(const hg_poly *polys, const uint64_t *ranges, uint64_t n, uint64_t width,
                           uint64_t *limbs, int64_t *sign_size, uint64_t *scratch, void *stream);

/* ---- device-resident multiply service ---------------------------------- */

/* Replaces the one-product-at-a-time mpz-* calls that binary-split / combine
 * (src/binary-splitting.lisp:100-133) and the MPD Newton steps
 * (src/mpd-reciprocal.lisp:27-73, src/mpd-sqrt.lisp:40-90) make.  Operands
 * and results stay in device memory; a worker thread batches the submitted
 * products (continuous batching: products submitted while batches run join
 * the next batch as a slot frees up) and admits them by free workspace. */
typedef struct hg_svc hg_svc;

typedef struct hg_svc_report {
    uint64_t submitted, completed, failed, batches;
    uint64_t pending, in_flight;          /* at the time of the call             */
    uint64_t peak_batch_products;         /* since the last reset                */
    uint64_t peak_batch_workspace_bytes;  /* since the last reset                */
    uint64_t slot_workspace_bytes;
    uint64_t latency_samples;             /* products completed since the reset  */
    int slots;
    double p50_us, p99_us, mean_us, max_us; /* submit-to-completion latency     */
    double products_per_s;  /* completed since the reset / (last completion - first submission) */
} hg_svc_report;

/* Open a service with `slots` CUDA streams (1..8) sharing workspace_bytes of
 * device memory (0: half the free memory, at most 8 GiB), allocated now;
 * max_batch products per batch (0: 2^20).  Needs hg_init; close every
 * service before hg_shutdown. */
int hg_svc_open(size_t workspace_bytes, int slots, size_t max_batch, hg_svc **svc);
/* Queue n products (device pointers, as hg_product); they get the tickets
 * *first_ticket .. *first_ticket + n - 1.  All are checked before any is
 * queued: a product whose transform workspace exceeds one slot is
 * HG_ERR_ARG.  The service's streams are not ordered after the caller's:
 * the operands must be complete in device memory when this is called (for
 * example, synchronise the stream that wrote them), and operands and outputs
 * must stay valid until the product is done.  Thread-safe. */
int hg_svc_submit(hg_svc *svc, const hg_product *prods, size_t n, uint64_t *first_ticket);
/* 1 done, 0 pending, < 0 the HG_ERR_* code the product failed with. */
int hg_svc_status(hg_svc *svc, uint64_t ticket);
/* Wait for one product (timeout_s < 0: no limit); HG_ERR_TIMEOUT when the
 * time runs out first. */
int hg_svc_wait(hg_svc *svc, uint64_t ticket, double timeout_s);
/* Wait for every product submitted so far. */
int hg_svc_wait_all(hg_svc *svc, double timeout_s);
/* Counters and latency percentiles; reset != 0 starts a new latency window. */
int hg_svc_stats(hg_svc *svc, hg_svc_report *out, int reset);
/* Finish the queued products, stop the worker, free the service. */
int hg_svc_close(hg_svc *svc);

/* ---- spectra (parity hooks) -------------------------------------------- */

/* ntt-forward (src/number-theoretic-transform.lisp:40-90) in place on n
 * device residues (each < the modulus) for scheme modulus mod_num: natural
 * order in, bit-reversed order out, the same values the reference computes. */
int hg_ntt_forward_device(uint64_t *a, size_t n, int mod_num, void *stream);

/* ntt-reverse (src/number-theoretic-transform.lisp:93-143) in place:
 * bit-reversed in, natural out, scaled by 1/n like the reference. */
int hg_ntt_reverse_device(uint64_t *a, size_t n, int mod_num, void *stream);

/* ---- instrumentation ---------------------------------------------------
 * No counterpart in the reference (its *verbose* stage timers,
 * src/ntt-multiply.lisp:109-114, print wall-clock milliseconds).  Kernel
 * classes index the arrays below. */
#define HG_KC_NTT_FORWARD 0 /* forward NTT passes (the first also reduces limbs) */
#define HG_KC_NTT_INVERSE 1 /* inverse NTT passes                               */
#define HG_KC_MIDDLE 2      /* last forward pass + pointwise product + first     */
                            /* inverse pass, fused                               */
#define HG_KC_CARRY 3       /* reconstruction + carry scan                      */
#define HG_KC_SMALL 4       /* schoolboy / by-digit products                    */
#define HG_KC_OTHER 5       /* scaling and other helpers                        */
#define HG_KC_BATCH 6       /* a whole batch in one persistent launch           */
#define HG_KC_COUNT 7

/* Record a CUDA event pair around every kernel launch from now on (on != 0)
 * or stop recording (on == 0). */
int hg_profile_enable(int on);

/* Totals per kernel class since the last read, then reset: launches, device
 * milliseconds (only while recording) and the algorithmic bytes those
 * launches move (each input read once, each output written once).
 * Synchronises on the recorded events. */
int hg_profile_read(uint64_t *launches, double *ms, double *bytes, int cap);

#ifdef __cplusplus
}
#endif
#endif
