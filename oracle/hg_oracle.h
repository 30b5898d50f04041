/*
 * hg_oracle.h -- CPU restatement of hypergeometrica's exact multiplication path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker: tests/, the smoke
 * test and bench.py's CPU-baseline leg load it to compare against or to time
 * beside the CUDA path.  Nothing in the shipped package links or calls it.
 *
 * Every function restates the Common Lisp reference (file:line given with
 * each declaration, paths relative to the hypergeometrica source tree).
 * Parity of this restatement is pinned by
 *   - golden fixtures written by an independent pure-Python restatement
 *     (tests/golden/make_golden.py), which is itself checked against the
 *     matrix / direct DFT definitions the reference's own tests use
 *     (tests/ntt.lisp:12-155) and against exact Python integer products;
 *   - the known answers embedded in the reference: the default moduli
 *     #x6280000000000001 #x5700000000000001 #x4180000000000001
 *     (logs/24apr21-999-ram.txt:199), the suitable-moduli listing and the
 *     generator 11 of 180143985094819841 (src/moduli.lisp:213-231).
 */
#ifndef HG_ORACLE_H
#define HG_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- digit.lisp / modular-arithmetic.lisp scalars ---------------------- */
int      hgo_primep(uint64_t n);                                   /* moduli.lisp:23-45 */
uint64_t hgo_next_prime(uint64_t n);                               /* moduli.lisp:47-53 */
uint64_t hgo_m_add(uint64_t a, uint64_t b, uint64_t m);            /* modular-arithmetic.lisp:37-48 */
uint64_t hgo_m_sub(uint64_t a, uint64_t b, uint64_t m);            /* modular-arithmetic.lisp:25-35 */
uint64_t hgo_m_mul(uint64_t a, uint64_t b, uint64_t m);            /* modular-arithmetic.lisp:81-88 */
uint64_t hgo_inv_mod(uint64_t x, uint64_t m);                      /* modular-arithmetic.lisp:90-99 */
uint64_t hgo_expt_mod(uint64_t a, uint64_t n, uint64_t m);         /* modular-arithmetic.lisp:118-133 */
uint64_t hgo_mod128_fast(uint64_t lo, uint64_t hi, uint64_t m, uint64_t minv); /* :167-188 */
uint64_t hgo_m_mul_fast(uint64_t a, uint64_t b, uint64_t m, uint64_t minv);   /* :190-202 */
uint64_t hgo_calc_b_inv(uint64_t b, uint64_t m);                   /* :207-208 */
uint64_t hgo_m_mul_fast2(uint64_t b, uint64_t binv, uint64_t a, uint64_t m);  /* :220-231 */

/* ---- moduli.lisp ---------------------------------------------------------- */
/* find-suitable-moduli (moduli.lisp:109-124); returns how many were found
 * (fewer than count only when the next candidate would not fit 64 bits). */
int      hgo_find_suitable_moduli(uint64_t transform_length, int count, uint64_t *out);
uint64_t hgo_find_generator(uint64_t m);                           /* moduli.lisp:173-179 */
uint64_t hgo_primitive_root(uint64_t n, uint64_t m);               /* moduli.lisp:181-191 */
int      hgo_default_moduli(uint64_t *out, int cap);               /* moduli.lisp:257-264 */

/* The modular scheme of make-modular-scheme (moduli.lisp:302-353). */
#define HGO_MAXK 8
typedef struct hgo_scheme {
    int k;                       /* number of moduli                     */
    int max_trans;               /* max-transform-length (bits)          */
    int lg_modulus;              /* min over moduli of lg(m)             */
    uint64_t moduli[HGO_MAXK];   /* descending                           */
    uint64_t inverses[HGO_MAXK]; /* floor(2^(64+lg_modulus)/m)           */
    uint64_t *roots;             /* [(max+1)][k][(max+1)][2]             */
    uint64_t *inv_roots;         /* same shape, 1/w                      */
    uint64_t *inv_lengths;       /* [(max+1)][k][2]                      */
} hgo_scheme;

/* Build a scheme from the given moduli (any order; sorted descending like
 * the reference).  Returns NULL on failure.  Free with hgo_scheme_free. */
hgo_scheme *hgo_scheme_make(const uint64_t *moduli, int k);
void        hgo_scheme_free(hgo_scheme *s);
/* The global **scheme** (ntt-multiply.lisp:8), built on first use. */
const hgo_scheme *hgo_default_scheme(void);
uint64_t hgo_scheme_root(const hgo_scheme *s, int power, int i, int kk, int which);
uint64_t hgo_scheme_inv_root(const hgo_scheme *s, int power, int i, int kk, int which);
uint64_t hgo_scheme_inv_length(const hgo_scheme *s, int power, int i, int which);
/* num-moduli-needed-for-bits (moduli.lisp:356-372); -1 when not enough. */
int hgo_num_moduli_needed_for_bits(const hgo_scheme *s, uint64_t bits);

/* ---- number-theoretic-transform.lisp ------------------------------------ */
/* ntt-forward (number-theoretic-transform.lisp:40-90): natural in,
 * bit-reversed out, in place.  n must be a power of two. */
void hgo_ntt_forward(uint64_t *a, size_t n, const hgo_scheme *s, int mod_num);
/* ntt-reverse (number-theoretic-transform.lisp:93-143): bit-reversed in,
 * natural out, 1/N applied in the first stage. */
void hgo_ntt_reverse(uint64_t *a, size_t n, const hgo_scheme *s, int mod_num);
/* bit-reversed-permute-vec! (strandh-elster-reversal.lisp:198-206). */
void hgo_bit_reverse_permute(uint64_t *a, size_t n);

/* ---- ntt-multiply.lisp / multiply.lisp / mpz-ram.lisp ------------------- */
// Transform length chosen by mpz-*/ntt for operand sizes nx, ny
// (ntt-multiply.lisp:175-176); mpz-square uses 2*nx (:103).
size_t hgo_ntt_length(size_t nx, size_t ny);

// mpz-*/ntt (ntt-multiply.lisp:174-254) on magnitudes.  Sizes are the
// storage lengths; high zero limbs are trimmed first (mpz-size).  Writes the
// full transform-length storage the reference returns into out (nout must
// be >= hgo_ntt_length(trimmed sizes)); limbs past it up to nout are zeroed.
// Returns 0, or a negative error code.
int hgo_mpz_mul_ntt(const uint64_t *x, size_t nx, const uint64_t *y, size_t ny,
                    uint64_t *out, size_t nout);
/* mpz-square (ntt-multiply.lisp:101-172). */
int hgo_mpz_square(const uint64_t *x, size_t nx, uint64_t *out, size_t nout);
/* %multiply-storage/schoolboy (mpz-ram.lisp:404-431): out has
 * 1 + nx + ny limbs (requires nx >= ny). */
int hgo_mul_schoolboy(const uint64_t *x, size_t nx, const uint64_t *y, size_t ny,
                      uint64_t *out, size_t nout);
/* mpz-multiply-by-digit! (mpz-ram.lisp:367-395) applied to a copy of x in a
 * storage of nx + 2 limbs (multiply.lisp:34-38). */
int hgo_mul_by_digit(const uint64_t *x, size_t nx, uint64_t d, uint64_t *out, size_t nout);

/* mpz-* dispatch (multiply.lisp:12-49) on signed operands.  same_object
 * reproduces the (eq x y) test.  threshold is *ntt-multiply-threshold*.
 * The trimmed magnitude goes to out (*nres limbs) and its sign to *sres. */
int hgo_mpz_mul(const uint64_t *x, size_t nx, int sx, const uint64_t *y, size_t ny, int sy,
                int same_object, size_t threshold,
                uint64_t *out, size_t nout, size_t *nres, int *sres);

/* Number of host threads used by the per-modulus task parallelism of
 * with-parallel-work (ntt-multiply.lisp:64-86); 1 disables it. */
void hgo_set_threads(int n);
int  hgo_get_threads(void);

#ifdef __cplusplus
}
#endif
#endif
