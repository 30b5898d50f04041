/*
 * hg_oracle.c -- CPU restatement of hypergeometrica's exact multiplication
 * path (see hg_oracle.h).  TEST INFRASTRUCTURE ONLY: the checker for the
 * CUDA library, never linked into it.
 *
 * The code follows the reference's loops and arithmetic step by step so that
 * intermediate arrays (residues, bit-reversed spectra, inverse outputs) are
 * the same values the reference computes, not merely the same final product.
 * 128-bit intermediates use unsigned __int128, which gcc provides on both
 * x86-64 and aarch64.
 */
#include "hg_oracle.h"

#include <pthread.h>
#include <stdlib.h>
#include <string.h>

typedef unsigned __int128 u128;

#define HGO_ERR_ARG (-1)
#define HGO_ERR_MODULI (-2)
#define HGO_ERR_OOM (-3)
#define HGO_ERR_INCONSISTENT (-4)

/* ------------------------------------------------------------------------ */
/* Scalars: digit.lisp, modular-arithmetic.lisp                             */
/* ------------------------------------------------------------------------ */

static inline uint64_t mul_hi(uint64_t a, uint64_t b) { return (uint64_t)(((u128)a * b) >> 64); }

/* m- (modular-arithmetic.lisp:25-35). */
uint64_t hgo_m_sub(uint64_t a, uint64_t b, uint64_t m) {
    return (a < b) ? (m - b) + a : a - b;
}

/* m+ (modular-arithmetic.lisp:37-48): b = 0 returns a, else a - (m - b). */
uint64_t hgo_m_add(uint64_t a, uint64_t b, uint64_t m) {
    return (b == 0) ? a : hgo_m_sub(a, m - b, m);
}

/* m* (modular-arithmetic.lisp:81-88): mul128 then div128 remainder. */
uint64_t hgo_m_mul(uint64_t a, uint64_t b, uint64_t m) {
    return (uint64_t)(((u128)a * b) % m);
}

/* inv-mod (modular-arithmetic.lisp:90-99): extended Euclid, egcd(x, m, 0, 1). */
uint64_t hgo_inv_mod(uint64_t x, uint64_t m) {
    /* egcd(x, b, a, u): if x = 0 -> (b == 1 ? a mod m : error)
     * else (q, r) = floor(b, x); egcd(r, x, u, a - u*q).  Track a, u as
     * signed 128-bit values; they stay bounded by m in magnitude. */
    __int128 a = 0, u = 1;
    uint64_t b = m;
    x %= m;
    while (x != 0) {
        uint64_t q = b / x, r = b % x;
        __int128 na = u, nu = a - u * (__int128)q;
        b = x;
        x = r;
        a = na;
        u = nu;
    }
    if (b != 1) return 0; /* not invertible: the reference signals an error */
    __int128 res = a % (__int128)m;
    if (res < 0) res += m;
    return (uint64_t)res;
}

/* expt-mod (modular-arithmetic.lisp:118-133), square-and-multiply with m*. */
uint64_t hgo_expt_mod(uint64_t a, uint64_t n, uint64_t m) {
    uint64_t result = 1 % m;
    a %= m;
    for (;;) {
        if (n & 1) result = hgo_m_mul(result, a, m);
        n >>= 1;
        if (n == 0) return result;
        a = hgo_m_mul(a, a, m);
    }
}

/* expt-mod/2^n (modular-arithmetic.lisp:136-144): n squarings. */
static uint64_t expt_mod_2n(uint64_t a, int n, uint64_t m) {
    for (int i = 0; i < n; i++) a = hgo_m_mul(a, a, m);
    return a;
}

/* The modulus width used by mod128/fast: +lg-modulus+ = 62
 * (modular-arithmetic.lisp:12-14). */
#define HGO_LG_MODULUS 62

/* mod128/fast (modular-arithmetic.lisp:167-188).
 *   a1 = bits [62, 126) of (hi:lo)                 (dpb/ash, :177-179)
 *   q  = hi64(a1 * m~)                             (:180)
 *   (hi:lo) -= q*m ; (hi:lo) -= 2m                 (:182-185)
 *   (hi:lo) += m & (hi >> 1)                       (:187)
 *   return lo + (m & hi)                           (:188)
 * sub128/add128 are the portable definitions (digit.lisp:404-431): plain
 * arithmetic modulo 2^128. */
uint64_t hgo_mod128_fast(uint64_t lo, uint64_t hi, uint64_t m, uint64_t minv) {
    const uint64_t mask = (((uint64_t)1) << HGO_LG_MODULUS) - 1;
    uint64_t a1 = ((hi & mask) << (64 - HGO_LG_MODULUS)) | (lo >> HGO_LG_MODULUS);
    uint64_t q = mul_hi(a1, minv);
    u128 v = ((u128)hi << 64) | lo;
    v -= (u128)q * m;
    v -= (u128)(m * 2);
    hi = (uint64_t)(v >> 64);
    v += (u128)(m & (hi >> 1));
    lo = (uint64_t)v;
    hi = (uint64_t)(v >> 64);
    return lo + (m & hi);
}

// m*/fast (modular-arithmetic.lisp:190-202).
uint64_t hgo_m_mul_fast(uint64_t a, uint64_t b, uint64_t m, uint64_t minv) {
    u128 p = (u128)a * b;
    return hgo_mod128_fast((uint64_t)p, (uint64_t)(p >> 64), m, minv);
}

/* calc-b-inv (modular-arithmetic.lisp:207-208): floor(b * 2^64 / m). */
uint64_t hgo_calc_b_inv(uint64_t b, uint64_t m) {
    return (uint64_t)(((u128)b << 64) / m);
}

// m*/fast2 (modular-arithmetic.lisp:211-231): Shoup multiplication by a
// precomputed b with companion b-inv, one conditional subtraction.
uint64_t hgo_m_mul_fast2(uint64_t b, uint64_t binv, uint64_t a, uint64_t m) {
    uint64_t q = mul_hi(a, binv);
    uint64_t r = a * b - q * m;
    if (r >= m) r -= m;
    return r;
}

/* ------------------------------------------------------------------------ */
/* moduli.lisp                                                               */
/* ------------------------------------------------------------------------ */

/* primep (moduli.lisp:23-45).  The reference draws K=10 random Miller-Rabin
 * bases; this restatement uses the fixed bases 2..37, which decide every
 * 64-bit input exactly, so it agrees with the reference wherever the
 * reference's randomized answer is right (always, for the primes it uses). */
int hgo_primep(uint64_t n) {
    if (n == 1 || n == 0) return 0;
    if (n < 4) return 1;
    if ((n & 1) == 0) return 0;
    static const uint64_t bases[] = {2, 3, 5, 7, 11, 13, 17, 19, 23, 29, 31, 37};
    for (size_t i = 0; i < sizeof bases / sizeof bases[0]; i++)
        if (n == bases[i]) return 1;
    for (size_t i = 0; i < sizeof bases / sizeof bases[0]; i++)
        if (n % bases[i] == 0) return 0;
    /* factor-out (n-1, 2) (moduli.lisp:12-18) */
    uint64_t d = n - 1;
    int s = 0;
    while ((d & 1) == 0) {
        d >>= 1;
        s++;
    }
    for (size_t i = 0; i < sizeof bases / sizeof bases[0]; i++) {
        uint64_t x = hgo_expt_mod(bases[i], d, n);
        if (x == 1 || x == n - 1) continue;
        int witness = 1;
        for (int r = 1; r < s; r++) {
            x = hgo_m_mul(x, x, n);
            if (x == n - 1) {
                witness = 0;
                break;
            }
        }
        if (witness) return 0;
    }
    return 1;
}

/* next-prime (moduli.lisp:47-53). */
uint64_t hgo_next_prime(uint64_t n) {
    uint64_t i = (n & 1) ? n : n - 1;
    for (i += 2;; i += 2)
        if (hgo_primep(i)) return i;
}

static int integer_length(uint64_t n) {
    int l = 0;
    while (n) {
        l++;
        n >>= 1;
    }
    return l;
}

/* next-power-of-two (math-utilities.lisp:12-16): least k with n <= 2^k. */
static int next_power_of_two_bits(uint64_t n) {
    int is_pow2 = n && !(n & (n - 1));
    return is_pow2 ? integer_length(n) - 1 : integer_length(n);
}

/* find-suitable-moduli (moduli.lisp:109-124): p = i*2^k + 1 for i = 1, 2, ...
 * keeping primes whose p-1 has at least k factors of two. */
int hgo_find_suitable_moduli(uint64_t transform_length, int count, uint64_t *out) {
    int min_power = next_power_of_two_bits(transform_length);
    if (min_power >= 64) return 0;
    uint64_t min = ((uint64_t)1) << min_power;
    int found = 0;
    for (uint64_t i = 1; found < count; i++) {
        u128 p = (u128)i * min + 1;
        if (p >> 64) break;
        uint64_t q = (uint64_t)p;
        if (hgo_primep(q)) {
            uint64_t pm1 = q - 1;
            int power = 0;
            while ((pm1 & 1) == 0) {
                pm1 >>= 1;
                power++;
            }
            if (power >= min_power) out[found++] = q;
        }
    }
    return found;
}

/* factorize (moduli.lisp:64-77), distinct prime factors only (which is all
 * generator-test-function uses, :164-171). */
static int distinct_prime_factors(uint64_t n, uint64_t *f, int cap) {
    int k = 0;
    if (n > 1 && hgo_primep(n)) {
        f[k++] = n;
        return k;
    }
    for (uint64_t p = 2; n > 1; p = hgo_next_prime(p)) {
        if (n % p == 0) {
            if (k < cap) f[k++] = p;
            while (n % p == 0) n /= p;
            if (n > 1 && hgo_primep(n)) {
                if (k < cap) f[k++] = n;
                break;
            }
        }
    }
    return k;
}

/* find-finite-field-generator (moduli.lisp:173-179): the smallest prime g
 * with g^((m-1)/f) != 1 for every prime factor f of m-1. */
uint64_t hgo_find_generator(uint64_t m) {
    uint64_t f[64];
    int nf = distinct_prime_factors(m - 1, f, 64);
    for (uint64_t p = 2;; p = hgo_next_prime(p)) {
        int ok = 1;
        for (int i = 0; i < nf; i++)
            if (hgo_expt_mod(p, (m - 1) / f[i], m) == 1) {
                ok = 0;
                break;
            }
        if (ok) return p;
    }
}

/* primitive-root-from-generator / find-primitive-root (moduli.lisp:181-191). */
uint64_t hgo_primitive_root(uint64_t n, uint64_t m) {
    return hgo_expt_mod(hgo_find_generator(m), (m - 1) / n, m);
}

static int cmp_desc(const void *a, const void *b) {
    uint64_t x = *(const uint64_t *)a, y = *(const uint64_t *)b;
    return (x < y) - (x > y);
}

/* default-moduli (moduli.lisp:257-264): the suitable moduli for 2^55 whose
 * integer-length is +modulus-bits+ = 63, deduplicated, descending.  The
 * reference asks for the first 1000 suitable moduli; every 63-bit one is
 * among them (they are i*2^55+1 with 128 <= i < 256, found before any larger
 * i), so scanning i < 256 yields the same set. */
int hgo_default_moduli(uint64_t *out, int cap) {
    int n = 0;
    for (uint64_t i = 1; i < 256; i++) {
        uint64_t p = (i << 55) + 1;
        if (integer_length(p) == 63 && hgo_primep(p) && n < cap) out[n++] = p;
    }
    qsort(out, (size_t)n, sizeof(uint64_t), cmp_desc);
    return n;
}

static int ctz64(uint64_t n) {
    int z = 0;
    while (!(n & 1)) {
        n >>= 1;
        z++;
    }
    return z;
}

#define RIDX(s, power, i, kk, w) \
    ((((size_t)(power) * (s)->k + (i)) * ((s)->max_trans + 1) + (kk)) * 2 + (w))
#define LIDX(s, power, i, w) ((((size_t)(power) * (s)->k + (i)) * 2) + (w))

/* make-modular-scheme (moduli.lisp:302-353). */
hgo_scheme *hgo_scheme_make(const uint64_t *moduli, int k) {
    if (k < 1 || k > HGO_MAXK) return NULL;
    hgo_scheme *s = (hgo_scheme *)calloc(1, sizeof *s);
    if (!s) return NULL;
    s->k = k;
    memcpy(s->moduli, moduli, sizeof(uint64_t) * (size_t)k);
    qsort(s->moduli, (size_t)k, sizeof(uint64_t), cmp_desc);
    /* max-transform-length-bits (:266-267) and the lg minimum (:307-308). */
    s->max_trans = 64;
    s->lg_modulus = 64;
    for (int i = 0; i < k; i++) {
        int t = ctz64(s->moduli[i] - 1);
        if (t < s->max_trans) s->max_trans = t;
        int lg = integer_length(s->moduli[i]) - 1;
        if (lg < s->lg_modulus) s->lg_modulus = lg;
    }
    size_t P = (size_t)s->max_trans + 1;
    s->roots = (uint64_t *)calloc(P * k * P * 2, sizeof(uint64_t));
    s->inv_roots = (uint64_t *)calloc(P * k * P * 2, sizeof(uint64_t));
    s->inv_lengths = (uint64_t *)calloc(P * k * 2, sizeof(uint64_t));
    if (!s->roots || !s->inv_roots || !s->inv_lengths) {
        hgo_scheme_free(s);
        return NULL;
    }
    for (int i = 0; i < k; i++) {
        uint64_t m = s->moduli[i];
        uint64_t g = hgo_find_generator(m);
        for (size_t power = 0; power < P; power++) {
            /* find-primitive-root (2^power, m) and its inverse (:322-325). */
            uint64_t w = hgo_expt_mod(g, (m - 1) >> power, m);
            uint64_t wi = hgo_inv_mod(w, m);
            for (size_t kk = 0; kk < P; kk++) {
                uint64_t wk = expt_mod_2n(w, (int)kk, m);
                uint64_t wik = expt_mod_2n(wi, (int)kk, m);
                s->roots[RIDX(s, power, i, kk, 0)] = wk;
                s->roots[RIDX(s, power, i, kk, 1)] = hgo_calc_b_inv(wk, m);
                s->inv_roots[RIDX(s, power, i, kk, 0)] = wik;
                s->inv_roots[RIDX(s, power, i, kk, 1)] = hgo_calc_b_inv(wik, m);
            }
        }
        /* reciprocal lengths (:334-340) */
        for (size_t kk = 0; kk < P; kk++) {
            uint64_t invn = hgo_inv_mod(hgo_expt_mod(2, kk, m), m);
            s->inv_lengths[LIDX(s, kk, i, 0)] = invn;
            s->inv_lengths[LIDX(s, kk, i, 1)] = hgo_calc_b_inv(invn, m);
        }
        /* %inverse (:343-345): floor(2^(64 + lg-modulus) / m). */
        s->inverses[i] = (uint64_t)(((u128)1 << (64 + s->lg_modulus)) / m);
    }
    return s;
}

void hgo_scheme_free(hgo_scheme *s) {
    if (!s) return;
    free(s->roots);
    free(s->inv_roots);
    free(s->inv_lengths);
    free(s);
}

uint64_t hgo_scheme_root(const hgo_scheme *s, int power, int i, int kk, int which) {
    return s->roots[RIDX(s, power, i, kk, which)];
}
uint64_t hgo_scheme_inv_root(const hgo_scheme *s, int power, int i, int kk, int which) {
    return s->inv_roots[RIDX(s, power, i, kk, which)];
}
uint64_t hgo_scheme_inv_length(const hgo_scheme *s, int power, int i, int which) {
    return s->inv_lengths[LIDX(s, power, i, which)];
}

static pthread_once_t g_scheme_once = PTHREAD_ONCE_INIT;
static hgo_scheme *g_scheme;
static void make_default_scheme(void) {
    uint64_t m[HGO_MAXK];
    int n = hgo_default_moduli(m, HGO_MAXK);
    g_scheme = hgo_scheme_make(m, n);
}
const hgo_scheme *hgo_default_scheme(void) {
    pthread_once(&g_scheme_once, make_default_scheme);
    return g_scheme;
}

/* num-moduli-needed-for-bits (moduli.lisp:356-372). */
int hgo_num_moduli_needed_for_bits(const hgo_scheme *s, uint64_t bits) {
    int needed = 0;
    long long remaining = (long long)bits;
    while (remaining > 0) {
        if (needed == s->k) return -1; /* the reference's assert fires */
        remaining -= integer_length(s->moduli[needed]);
        needed++;
    }
    return needed;
}

/* ------------------------------------------------------------------------ */
/* number-theoretic-transform.lisp                                           */
/* ------------------------------------------------------------------------ */

static int lg_size(size_t n) {
    int l = 0;
    while (((size_t)1 << l) < n) l++;
    return l;
}

/* ntt-forward (number-theoretic-transform.lisp:40-90). */
void hgo_ntt_forward(uint64_t *a, size_t n, const hgo_scheme *s, int mod_num) {
    const uint64_t m = s->moduli[mod_num];
    const uint64_t minv = s->inverses[mod_num];
    const int ln = lg_size(n);
    for (int lsubn = ln; lsubn >= 2; lsubn--) {
        size_t subn = (size_t)1 << lsubn;
        size_t half = subn / 2;
        uint64_t dw = hgo_scheme_root(s, ln, mod_num, ln - lsubn, 0);
        uint64_t dwi = hgo_scheme_root(s, ln, mod_num, ln - lsubn, 1);
        uint64_t wj = 1;
        for (size_t j = 0; j < half; j++) {
            for (size_t r = 0; r <= n - subn; r += subn) {
                size_t p = r + j, q = p + half;
                uint64_t u = a[p], v = a[q];
                a[p] = hgo_m_add(u, v, m);
                a[q] = hgo_m_mul_fast(wj, hgo_m_sub(u, v, m), m, minv);
            }
            wj = hgo_m_mul_fast2(dw, dwi, wj, m);
        }
    }
    if (ln > 0) {
        for (size_t r = 0; r < n; r += 2) {
            uint64_t u = a[r], v = a[r + 1];
            a[r] = hgo_m_add(u, v, m);
            a[r + 1] = hgo_m_sub(u, v, m);
        }
    }
}

/* ntt-reverse (number-theoretic-transform.lisp:93-143). */
void hgo_ntt_reverse(uint64_t *a, size_t n, const hgo_scheme *s, int mod_num) {
    const uint64_t m = s->moduli[mod_num];
    const uint64_t minv = s->inverses[mod_num];
    const int ldn = lg_size(n);
    uint64_t invn = hgo_scheme_inv_length(s, ldn, mod_num, 0);
    uint64_t invni = hgo_scheme_inv_length(s, ldn, mod_num, 1);
    if (ldn > 0) {
        for (size_t r = 0; r < n; r += 2) {
            uint64_t u = a[r], v = a[r + 1];
            a[r] = hgo_m_mul_fast2(invn, invni, hgo_m_add(u, v, m), m);
            a[r + 1] = hgo_m_mul_fast2(invn, invni, hgo_m_sub(u, v, m), m);
        }
    }
    for (int ldm = 2; ldm <= ldn; ldm++) {
        size_t subn = (size_t)1 << ldm;
        size_t half = subn / 2;
        uint64_t dw = hgo_scheme_inv_root(s, ldn, mod_num, ldn - ldm, 0);
        uint64_t dwi = hgo_scheme_inv_root(s, ldn, mod_num, ldn - ldm, 1);
        uint64_t wj = 1;
        for (size_t j = 0; j < half; j++) {
            for (size_t r = 0; r <= n - subn; r += subn) {
                size_t p = r + j, q = p + half;
                uint64_t u = a[p];
                uint64_t v = hgo_m_mul_fast(wj, a[q], m, minv);
                a[p] = hgo_m_add(u, v, m);
                a[q] = hgo_m_sub(u, v, m);
            }
            wj = hgo_m_mul_fast2(dw, dwi, wj, m);
        }
    }
}

/* bit-reversed-permute-vec! (strandh-elster-reversal.lisp:198-206). */
void hgo_bit_reverse_permute(uint64_t *a, size_t n) {
    int bits = lg_size(n);
    for (size_t i = 0; i < n; i++) {
        size_t r = 0;
        for (int b = 0; b < bits; b++)
            if (i & ((size_t)1 << b)) r |= (size_t)1 << (bits - 1 - b);
        if (r > i) {
            uint64_t t = a[i];
            a[i] = a[r];
            a[r] = t;
        }
    }
}

/* ------------------------------------------------------------------------ */
/* Per-modulus task parallelism: with-parallel-work / with-task              */
/* (ntt-multiply.lisp:64-86) and pdotimes (:97, :141)                        */
/* ------------------------------------------------------------------------ */

static int g_threads = 1;
void hgo_set_threads(int n) { g_threads = n < 1 ? 1 : n; }
int hgo_get_threads(void) { return g_threads; }

typedef struct {
    int kind; /* 0 forward, 1 reverse, 2 pointwise, 3 square */
    uint64_t *a, *b;
    size_t n;
    const hgo_scheme *s;
    int mod;
} task_t;

static void run_task(task_t *t) {
    const uint64_t m = t->s->moduli[t->mod], mi = t->s->inverses[t->mod];
    switch (t->kind) {
    case 0: hgo_ntt_forward(t->a, t->n, t->s, t->mod); break;
    case 1: hgo_ntt_reverse(t->a, t->n, t->s, t->mod); break;
    case 2: /* multiply-pointwise! (ntt-multiply.lisp:88-99) */
        for (size_t i = 0; i < t->n; i++) t->a[i] = hgo_m_mul_fast(t->a[i], t->b[i], m, mi);
        break;
    case 3: /* mpz-square pointwise squaring (ntt-multiply.lisp:136-144) */
        for (size_t i = 0; i < t->n; i++) t->a[i] = hgo_m_mul_fast(t->a[i], t->a[i], m, mi);
        break;
    }
}

static void *task_entry(void *p) {
    run_task((task_t *)p);
    return NULL;
}

/* Run the tasks, at most g_threads at a time. */
static void run_tasks(task_t *tasks, int n) {
    if (g_threads <= 1) {
        for (int i = 0; i < n; i++) run_task(&tasks[i]);
        return;
    }
    for (int base = 0; base < n; base += g_threads) {
        int cnt = n - base < g_threads ? n - base : g_threads;
        pthread_t th[64];
        int started[64] = {0};
        for (int i = 0; i < cnt; i++)
            started[i] = pthread_create(&th[i], NULL, task_entry, &tasks[base + i]) == 0;
        for (int i = 0; i < cnt; i++) {
            if (started[i])
                pthread_join(th[i], NULL);
            else
                run_task(&tasks[base + i]);
        }
    }
}

/* ------------------------------------------------------------------------ */
/* ntt-multiply.lisp                                                         */
/* ------------------------------------------------------------------------ */

/* least-power-of-two->= (math-utilities.lisp:18-22). */
static size_t least_pow2_ge(size_t n) {
    if (n && !(n & (n - 1))) return n;
    size_t r = 1;
    while (r < n) r <<= 1;
    return r == 0 ? 1 : r;
}

size_t hgo_ntt_length(size_t nx, size_t ny) { return least_pow2_ge(nx + ny); }

/* mpz-size: vec-digit-length* (vec.lisp:218-229). */
static size_t trimmed(const uint64_t *x, size_t n) {
    while (n > 0 && x[n - 1] == 0) n--;
    return n;
}

/* integer-length of N * (2^64 - 1)^2 for N = 2^L (ntt-multiply.lisp:177). */
static uint64_t bound_bits(size_t length) {
    /* (2^64-1)^2 = 2^128 - 2^65 + 1 has integer-length 128; times 2^L adds L. */
    return 128 + (uint64_t)lg_size(length);
}

/* %make-ntt-work (number-theoretic-transform.lisp:7-22): residues of the
 * operand's digits, zero elsewhere. */
static void make_ntt_work(uint64_t *dst, const uint64_t *x, size_t nx, size_t length, uint64_t m) {
    size_t i = 0;
    for (; i < nx; i++) dst[i] = x[i] % m;
    for (; i < length; i++) dst[i] = 0;
}

/* Small fixed-width unsigned integers, little-endian 64-bit limbs, for the
 * CRT block (ntt-multiply.lisp:242-253). */
#define BW 6
typedef struct {
    uint64_t w[BW];
} big_t;

static void big_zero(big_t *a) { memset(a, 0, sizeof *a); }
static void big_mul_small(big_t *r, const big_t *a, uint64_t b) {
    uint64_t carry = 0;
    for (int i = 0; i < BW; i++) {
        u128 t = (u128)a->w[i] * b + carry;
        r->w[i] = (uint64_t)t;
        carry = (uint64_t)(t >> 64);
    }
}
static void big_add(big_t *r, const big_t *a, const big_t *b) {
    uint64_t c = 0;
    for (int i = 0; i < BW; i++) {
        u128 t = (u128)a->w[i] + b->w[i] + c;
        r->w[i] = (uint64_t)t;
        c = (uint64_t)(t >> 64);
    }
}
static int big_cmp(const big_t *a, const big_t *b) {
    for (int i = BW - 1; i >= 0; i--)
        if (a->w[i] != b->w[i]) return a->w[i] < b->w[i] ? -1 : 1;
    return 0;
}
static void big_sub(big_t *r, const big_t *a, const big_t *b) {
    uint64_t br = 0;
    for (int i = 0; i < BW; i++) {
        u128 t = (u128)a->w[i] - b->w[i] - br;
        r->w[i] = (uint64_t)t;
        br = (uint64_t)(t >> 64) ? 1 : 0;
    }
}
static int big_bits(const big_t *a) {
    for (int i = BW - 1; i >= 0; i--)
        if (a->w[i]) return 64 * i + integer_length(a->w[i]);
    return 0;
}
static void big_shl(big_t *r, const big_t *a, int sh) {
    big_t t;
    big_zero(&t);
    int ls = sh / 64, bs = sh % 64;
    for (int i = BW - 1; i >= 0; i--) {
        int j = i - ls;
        if (j < 0) continue;
        uint64_t v = a->w[j] << bs;
        if (bs && j - 1 >= 0) v |= a->w[j - 1] >> (64 - bs);
        t.w[i] = v;
    }
    *r = t;
}
static u128 big_top(const big_t *a, int sh) { /* (a >> sh) truncated to 128 bits */
    big_t t;
    big_zero(&t);
    int ls = sh / 64, bs = sh % 64;
    for (int i = 0; i + ls < BW; i++) {
        uint64_t v = a->w[i + ls] >> bs;
        if (bs && i + ls + 1 < BW) v |= a->w[i + ls + 1] << (64 - bs);
        t.w[i] = v;
    }
    return ((u128)t.w[1] << 64) | t.w[0];
}

/* a = a mod m.  The quotient is estimated from the top bits,
 * q' = floor((a >> s) / ((m >> s) + 1)) <= q, with s chosen so that
 * m >> s has 63-64 bits; then a -= q' m and a few exact subtractions
 * finish.  Same remainder as long division. */
static void big_mod(big_t *a, const big_t *m) {
    int mb = big_bits(m);
    if (big_cmp(a, m) < 0) return;
    int sh = mb > 64 ? mb - 64 : 0;
    u128 mt = big_top(m, sh) + 1;
    while (big_cmp(a, m) >= 0) {
        u128 at = big_top(a, sh);
        if (big_bits(a) - sh > 128) { /* far too large for one estimate: shift-subtract */
            int d = big_bits(a) - mb - 1;
            big_t t;
            big_shl(&t, m, d);
            big_sub(a, a, &t);
            continue;
        }
        u128 q = at / mt;
        if (q == 0) {
            big_sub(a, a, m);
            continue;
        }
        big_t t, t2;
        big_mul_small(&t, m, (uint64_t)q);
        if (q >> 64) {
            big_mul_small(&t2, m, (uint64_t)(q >> 64));
            big_shl(&t2, &t2, 64);
            big_add(&t, &t, &t2);
        }
        big_sub(a, a, &t);
    }
}

typedef struct {
    int k;
    big_t composite;
    big_t factors[HGO_MAXK];
} crt_t;

/* moduli / composite / complements / inverses / factors
 * (ntt-multiply.lisp:242-246). */
static void crt_setup(crt_t *c, const hgo_scheme *s, int k) {
    c->k = k;
    big_zero(&c->composite);
    c->composite.w[0] = 1;
    for (int j = 0; j < k; j++) big_mul_small(&c->composite, &c->composite, s->moduli[j]);
    for (int j = 0; j < k; j++) {
        /* complement = composite / m_j = product of the others */
        big_t comp;
        big_zero(&comp);
        comp.w[0] = 1;
        for (int l = 0; l < k; l++)
            if (l != j) big_mul_small(&comp, &comp, s->moduli[l]);
        /* complement mod m_j, then its inverse */
        uint64_t cm = 1;
        for (int l = 0; l < k; l++)
            if (l != j) cm = hgo_m_mul(cm, s->moduli[l] % s->moduli[j], s->moduli[j]);
        uint64_t inv = hgo_inv_mod(cm, s->moduli[j]);
        big_mul_small(&c->factors[j], &comp, inv);
    }
}

/* add-big-digit (ntt-multiply.lisp:10-51): storage += digit * 2^(64 i) with
 * carry ripple; adding a nonzero amount past the end is the reference's
 * "grave inconsistency" error. */
static int add_big_digit(const big_t *digit, uint64_t *storage, size_t len, size_t i) {
    uint64_t carry = 0;
    int top = BW - 1;
    while (top >= 0 && digit->w[top] == 0) top--;
    if (top < 0) return 0;
    size_t pos = i;
    for (int j = 0; j <= top || carry; j++, pos++) {
        uint64_t add = (j <= top) ? digit->w[j] : 0;
        if (pos >= len) {
            if (add || carry) return HGO_ERR_INCONSISTENT;
            break;
        }
        u128 t = (u128)storage[pos] + add + carry;
        storage[pos] = (uint64_t)t;
        carry = (uint64_t)(t >> 64);
    }
    return 0;
}

/* The CRT loop (ntt-multiply.lisp:248-253 and :160-171). */
static int crt_unpack(uint64_t *const *ntts, int k, const hgo_scheme *s, uint64_t *result, size_t length) {
    crt_t c;
    crt_setup(&c, s, k);
    for (size_t i = 0; i < length; i++) {
        big_t sum, t;
        big_zero(&sum);
        for (int j = 0; j < k; j++) {
            big_mul_small(&t, &c.factors[j], ntts[j][i]);
            big_add(&sum, &sum, &t);
        }
        big_mod(&sum, &c.composite);
        int rc = add_big_digit(&sum, result, length, i);
        if (rc) return rc;
    }
    return 0;
}

// mpz-*/ntt (ntt-multiply.lisp:174-254), magnitudes only.
int hgo_mpz_mul_ntt(const uint64_t *x, size_t nx, const uint64_t *y, size_t ny, uint64_t *out, size_t nout) {
    const hgo_scheme *s = hgo_default_scheme();
    if (!s) return HGO_ERR_OOM;
    nx = trimmed(x, nx);
    ny = trimmed(y, ny);
    size_t length = least_pow2_ge(nx + ny);
    if (nout < length) return HGO_ERR_ARG;
    int k = hgo_num_moduli_needed_for_bits(s, bound_bits(length));
    if (k < 0 || lg_size(length) > s->max_trans) return HGO_ERR_MODULI;
    /* make-ntt-work allocates a work vector per scheme modulus (:180-181). */
    uint64_t *wx[HGO_MAXK], *wy[HGO_MAXK];
    int ok = 1;
    for (int j = 0; j < s->k; j++) {
        wx[j] = (uint64_t *)malloc(length * sizeof(uint64_t));
        wy[j] = (uint64_t *)malloc(length * sizeof(uint64_t));
        if (!wx[j] || !wy[j]) ok = 0;
    }
    int rc = 0;
    if (!ok) {
        rc = HGO_ERR_OOM;
        goto done;
    }
    for (int j = 0; j < s->k; j++) {
        make_ntt_work(wx[j], x, nx, length, s->moduli[j]);
        make_ntt_work(wy[j], y, ny, length, s->moduli[j]);
    }
    {
        task_t t[2 * HGO_MAXK];
        for (int j = 0; j < k; j++) { /* forward (:202-209) */
            t[2 * j] = (task_t){0, wx[j], NULL, length, s, j};
            t[2 * j + 1] = (task_t){0, wy[j], NULL, length, s, j};
        }
        run_tasks(t, 2 * k);
        for (int j = 0; j < k; j++) t[j] = (task_t){2, wx[j], wy[j], length, s, j}; /* pointwise (:215-220) */
        run_tasks(t, k);
        for (int j = 0; j < k; j++) t[j] = (task_t){1, wx[j], NULL, length, s, j}; /* reverse (:230-234) */
        run_tasks(t, k);
    }
    /* The result reuses y's first work vector, cleared (:184, :225). */
    memset(out, 0, nout * sizeof(uint64_t));
    rc = crt_unpack(wx, k, s, out, length);
done:
    for (int j = 0; j < s->k; j++) {
        free(wx[j]);
        free(wy[j]);
    }
    return rc;
}

/* mpz-square (ntt-multiply.lisp:101-172). */
int hgo_mpz_square(const uint64_t *x, size_t nx, uint64_t *out, size_t nout) {
    const hgo_scheme *s = hgo_default_scheme();
    if (!s) return HGO_ERR_OOM;
    nx = trimmed(x, nx);
    size_t length = least_pow2_ge(2 * nx);
    if (nout < length) return HGO_ERR_ARG;
    int k = hgo_num_moduli_needed_for_bits(s, bound_bits(length));
    if (k < 0 || lg_size(length) > s->max_trans) return HGO_ERR_MODULI;
    uint64_t *wx[HGO_MAXK];
    int ok = 1;
    for (int j = 0; j < s->k; j++) {
        wx[j] = (uint64_t *)malloc(length * sizeof(uint64_t));
        if (!wx[j]) ok = 0;
    }
    int rc = 0;
    if (!ok) {
        rc = HGO_ERR_OOM;
        goto done;
    }
    for (int j = 0; j < s->k; j++) make_ntt_work(wx[j], x, nx, length, s->moduli[j]);
    {
        task_t t[HGO_MAXK];
        for (int j = 0; j < k; j++) t[j] = (task_t){0, wx[j], NULL, length, s, j};
        run_tasks(t, k);
        for (int j = 0; j < k; j++) t[j] = (task_t){3, wx[j], NULL, length, s, j};
        run_tasks(t, k);
        for (int j = 0; j < k; j++) t[j] = (task_t){1, wx[j], NULL, length, s, j};
        run_tasks(t, k);
    }
    memset(out, 0, nout * sizeof(uint64_t));
    rc = crt_unpack(wx, k, s, out, length);
done:
    for (int j = 0; j < s->k; j++) free(wx[j]);
    return rc;
}

/* ------------------------------------------------------------------------ */
/* mpz-ram.lisp small products                                               */
/* ------------------------------------------------------------------------ */

/* mpz-multiply-by-digit! (mpz-ram.lisp:367-395) on the first `size` limbs of
 * v, writing the final carry to v[size]. */
static void multiply_by_digit_inplace(uint64_t *v, size_t size, uint64_t d) {
    uint64_t carry = 0;
    for (size_t i = 0; i < size; i++) {
        u128 p = (u128)d * v[i];
        uint64_t lo = (uint64_t)p, hi = (uint64_t)(p >> 64);
        u128 s = (u128)lo + carry;
        v[i] = (uint64_t)s;
        carry = hi + (uint64_t)(s >> 64);
    }
    if (carry) v[size] = carry;
}

int hgo_mul_by_digit(const uint64_t *x, size_t nx, uint64_t d, uint64_t *out, size_t nout) {
    nx = trimmed(x, nx);
    if (nout < nx + 2) return HGO_ERR_ARG;
    memset(out, 0, nout * sizeof(uint64_t));
    memcpy(out, x, nx * sizeof(uint64_t));
    if (d == 0) {
        memset(out, 0, nout * sizeof(uint64_t));
        return 0;
    }
    if (d == 1) return 0;
    multiply_by_digit_inplace(out, nx, d);
    return 0;
}

/* %multiply-storage/schoolboy (mpz-ram.lisp:404-431): for each nonzero b_i,
 * temp = a * 2^(64 i) * b_i, r += temp. */
int hgo_mul_schoolboy(const uint64_t *x, size_t nx, const uint64_t *y, size_t ny, uint64_t *out, size_t nout) {
    size_t length = 1 + nx + ny;
    if (nout < length || nx < ny) return HGO_ERR_ARG;
    memset(out, 0, nout * sizeof(uint64_t));
    uint64_t *temp = (uint64_t *)malloc(length * sizeof(uint64_t));
    if (!temp) return HGO_ERR_OOM;
    for (size_t i = 0; i < ny; i++) {
        uint64_t bi = y[i];
        if (bi == 0) continue;
        memset(temp, 0, length * sizeof(uint64_t));
        memcpy(temp + i, x, nx * sizeof(uint64_t));
        multiply_by_digit_inplace(temp, trimmed(temp, length), bi);
        /* %add-storages/unsafe r r length temp length */
        uint64_t c = 0;
        for (size_t j = 0; j < length; j++) {
            u128 t = (u128)out[j] + temp[j] + c;
            out[j] = (uint64_t)t;
            c = (uint64_t)(t >> 64);
        }
    }
    free(temp);
    return 0;
}

/* mpz-* (multiply.lisp:12-49). */
int hgo_mpz_mul(const uint64_t *x, size_t nx, int sx, const uint64_t *y, size_t ny, int sy, int same_object,
                size_t threshold, uint64_t *out, size_t nout, size_t *nres, int *sres) {
    nx = trimmed(x, nx);
    ny = trimmed(y, ny);
    if (nx < ny) { /* rotatef so |x| >= |y| (:15-16) */
        const uint64_t *tp = x;
        x = y;
        y = tp;
        size_t tn = nx;
        nx = ny;
        ny = tn;
        int ts = sx;
        sx = sy;
        sy = ts;
    }
    int rc = 0;
    *sres = sx * sy;
    if (ny == 0) { /* zero (:21-22) */
        *nres = 0;
        *sres = 1;
        return 0;
    } else if (ny == 1) { /* by digit (:23-36) */
        uint64_t d = y[0];
        if (d == 1) {
            if (nout < nx) return HGO_ERR_ARG;
            memcpy(out, x, nx * sizeof(uint64_t));
            *sres = (sy == -1) ? -sx : sx;
        } else {
            rc = hgo_mul_by_digit(x, nx, d, out, nout);
        }
    } else if (ny <= threshold) { /* schoolboy (:37-42) */
        rc = hgo_mul_schoolboy(x, nx, y, ny, out, nout);
    } else if (same_object) { /* square (:43-44); mpz-square returns sign +1 */
        rc = hgo_mpz_square(x, nx, out, nout);
        *sres = 1;
    } else { /* NTT (:48-49) */
        rc = hgo_mpz_mul_ntt(x, nx, y, ny, out, nout);
    }
    if (rc) return rc;
    *nres = trimmed(out, nout);
    if (*nres == 0) *sres = 1;
    return 0;
}
