/*
 * CPU oracle for the BLS12-381 G1 MSM and G1 FFT hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain C11 restatement of the reference
 * library's algorithms (category-blst), used by tests/, the smoke check and
 * bench.py's CPU-baseline leg to check results.  The product library never
 * links, loads or calls anything declared here.
 *
 * Parity of this restatement is pinned against the reference library built
 * from its own sources (oracle/_ref/libblst_ref.so) and against the golden
 * vectors under tests/golden/, which were produced by that library.
 *
 * Data layouts are the reference ABI layouts (bindings/blst_types.h:84-103):
 *   fp   : 6 x u64 little-endian limbs, Montgomery form, R = 2^384
 *   fr   : 4 x u64 little-endian limbs, Montgomery form, R = 2^256
 *   p1   : Jacobian {x, y, z} (144 B); infinity <=> z == 0
 *   p1a  : affine {x, y} (96 B); infinity <=> all zero
 */
#ifndef CATMSM_ORACLE_H
#define CATMSM_ORACLE_H

#include <stddef.h>
#include <stdint.h>
#include <stdbool.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct { uint64_t l[6]; } ofp;
typedef struct { uint64_t l[4]; } ofr;
typedef struct { ofp x, y, z; } op1;
typedef struct { ofp x, y; } op1a;
typedef struct { ofp x, y, zz, zzz; } op1xyzz;

/* ---- constants / init (fp.c) ---- */
void oracle_init(void);

/* ---- Fp / Fr (fp.c) ---- */
void ofp_mul(ofp *o, const ofp *a, const ofp *b);
void ofp_sqr(ofp *o, const ofp *a);
void ofp_add(ofp *o, const ofp *a, const ofp *b);
void ofp_sub(ofp *o, const ofp *a, const ofp *b);
void ofp_neg(ofp *o, const ofp *a);
void ofp_inv(ofp *o, const ofp *a);
void ofp_from_mont(ofp *o, const ofp *a);
void ofp_to_mont(ofp *o, const ofp *a);
bool ofp_is_zero(const ofp *a);
bool ofp_eq(const ofp *a, const ofp *b);
const ofp *ofp_one(void);

void ofr_mul(ofr *o, const ofr *a, const ofr *b);
void ofr_sqr(ofr *o, const ofr *a);
void ofr_inv(ofr *o, const ofr *a);
void ofr_from_mont(ofr *o, const ofr *a);
void ofr_to_mont(ofr *o, const ofr *a);
void ofr_from_u64(ofr *o, uint64_t v);
bool ofr_eq(const ofr *a, const ofr *b);
const ofr *ofr_one(void);
const ofr *ofr_modulus(void);
const ofp *ofp_modulus(void);

/* ---- G1 (g1.c) ---- */
void op1_generator(op1 *o);
bool op1_is_inf(const op1 *p);
void op1_from_affine(op1 *o, const op1a *a);
void op1_to_affine(op1a *o, const op1 *p);
void op1_neg(op1 *o, const op1 *p);
void op1_dadd(op1 *o, const op1 *a, const op1 *b);
void op1_double(op1 *o, const op1 *a);
void op1_mult_vartime(op1 *o, const op1 *p, const uint8_t *scalar, size_t nbits);
void op1_compress(uint8_t out[48], const op1 *p);
void op1_serialize(uint8_t out[96], const op1 *p);
void op1_affine_serialize(uint8_t out[96], const op1a *p);
bool op1_on_curve(const op1 *p);
void oxyzz_madd(op1xyzz *o, const op1xyzz *a, const op1a *b, int subtract);
void oxyzz_add(op1xyzz *o, const op1xyzz *a, const op1xyzz *b);
void oxyzz_to_jacobian(op1 *o, const op1xyzz *a);

/* ---- MSM (msm.c): restates c_api.cpp:1371-1418, multi_scalar.cpp:730-923 ---- */
size_t oracle_pippenger_window_size(size_t npoints);
size_t oracle_p1s_mult_pippenger_scratch_sizeof(size_t npoints);
void oracle_p1s_mult_pippenger(op1 *ret, const op1a *const points[], size_t npoints,
                               const uint8_t *const scalars[], size_t nbits,
                               uint64_t *scratch);
void oracle_p1s_mult_pippenger_window(op1 *ret, const op1a *const points[], size_t npoints,
                                      const uint8_t *const scalars[], size_t nbits,
                                      uint64_t *scratch, size_t window);
void oracle_p1s_tile_pippenger(op1 *ret, const op1a *const points[], size_t npoints,
                               const uint8_t *const scalars[], size_t nbits,
                               uint64_t *scratch, size_t bit0, size_t window);
/* Naive sum of k_i * P_i (the reference tests' algorithmic oracle). */
void oracle_p1s_mult_naive(op1 *ret, const op1a *points, size_t npoints,
                           const uint8_t *scalars, size_t nbits);

/* ---- fixed-table MSM (wbits.c): restates c_api.cpp:1310-1369,
 *      multi_scalar.h:245-315, multi_scalar.cpp:481-720 ---- */
size_t oracle_p1s_mult_wbits_precompute_sizeof(size_t wbits, size_t npoints);
void oracle_p1s_mult_wbits_precompute(op1a *table, size_t wbits, const op1a *const points[], size_t npoints);
size_t oracle_p1s_mult_wbits_scratch_sizeof(size_t npoints);
void oracle_p1s_mult_wbits(op1 *ret, const op1a *table, size_t wbits, size_t npoints,
                           const uint8_t *const scalars[], size_t nbits, uint64_t *scratch);

/* ---- FFT (fft.c): restates fft_c_api.cpp:51-220, ctFft.h, domain.h ---- */
size_t oracle_fr_fft_domain_len(size_t n);
bool oracle_fr_fft_domain_init(ofr *domain, size_t domain_len, size_t n);
bool oracle_p1_fft(op1 *values, size_t n, bool inverse);
bool oracle_p1_fft_with_domain(op1 *values, size_t n, const ofr *domain, size_t domain_len, bool inverse);
bool oracle_p1_ifft_unscaled_with_domain(op1 *values, size_t n, const ofr *domain, size_t domain_len);
bool oracle_p1_fft_truncated_prefix(op1 *values, size_t n, size_t xn, const ofr *domain, size_t domain_len);
bool oracle_fr_fft(ofr *values, size_t n, bool inverse);
bool oracle_fr_fft_with_domain(ofr *values, size_t n, const ofr *domain, size_t domain_len, bool inverse);
void oracle_fr_root_of_unity(ofr *o, size_t log2n);

/* ---- seeded synthetic inputs (gen.c) ---- */
uint64_t oracle_splitmix64(uint64_t *state);
/* kind 0: uniform Fr (255-bit, rejection), 1: uniform 64-bit, 2: uniform Fr
 * with a seeded 10% of scalars set to zero.  32 bytes LE per scalar. */
void oracle_gen_scalars(uint64_t seed, size_t n, int kind, uint8_t *out32);
/* P_i = k_i * G for 32-byte LE scalars k_i, affine output; nthreads >= 1. */
void oracle_points_from_scalars(const uint8_t *k32, size_t n, op1a *out, int nthreads);
/* Replace a seeded 5% of points by copies of other (seeded) points. */
void oracle_duplicate_points(uint64_t seed, size_t n, op1a *points);
/* Randomize affine points into Jacobian form with seeded nonzero z. */
void oracle_jacobian_randomize(uint64_t seed, size_t n, const op1a *in, op1 *out);

#ifdef __cplusplus
}
#endif
#endif
