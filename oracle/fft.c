/*
 * Oracle G1 / Fr FFT (test infrastructure only; see oracle.h).
 *
 * Restates:
 *   fft_c_api.cpp:51-66   group_fft (one-shot: roots = powers of the primitive
 *                         root, or of its inverse; inverse scales by 1/n)
 *   fft_c_api.cpp:68-103  group_fft_with_domain (length n+2, tag domain[n+1]
 *                         == n, inverse reads forward roots at n - idx, then
 *                         scales by domain[n]; the unscaled call skips it)
 *   fft_c_api.cpp:128-146 domain length / init
 *   fft/ctFft.h:20-124    valid sizes, bit_reverse, fft_butterflies, fft_scale
 *   fft/domain.h:18-100   fill_roots / initialize_domain / transform_with_domain
 *   fft/context.h:182-215 GroupFftCoeffCtx: plus = dadd, minus = neg + dadd,
 *                         mult = from_mont + mult_vartime(.., 256)
 *   fft/primitive_root.h:29-62,142-152  2^k-th roots: derived here from
 *                         7^((r-1)/2^32) by repeated squaring
 */
#include "oracle.h"
#include <stdlib.h>
#include <string.h>
#include <limits.h>

static int valid_size(size_t n)
{
    return n != 0 && (n & (n - 1)) == 0 && n <= (size_t)INT_MAX;
}

static int log2_size(size_t n)
{
    int k = 0;
    while (((size_t)1 << k) < n) k++;
    return k;
}

static ofr ROOTS[33];
static int roots_ready;

static void roots_init(void)
{
    if (roots_ready) return;
    /* e = (r - 1) / 2^32 */
    const uint64_t *r = ofr_modulus()->l;
    uint64_t e[4];
    for (int i = 0; i < 4; i++) e[i] = r[i];
    e[0] -= 1;
    for (int i = 0; i < 4; i++) e[i] = (e[i] >> 32) | (i < 3 ? e[i + 1] << 32 : 0);
    ofr seven, acc = *ofr_one();
    ofr_from_u64(&seven, 7);
    for (int i = 255; i >= 0; i--) {
        ofr_sqr(&acc, &acc);
        if ((e[i / 64] >> (i % 64)) & 1) ofr_mul(&acc, &acc, &seven);
    }
    ROOTS[32] = acc;
    for (int k = 31; k >= 0; k--) ofr_sqr(&ROOTS[k], &ROOTS[k + 1]);
    roots_ready = 1;
}

void oracle_fr_root_of_unity(ofr *o, size_t log2n)
{
    roots_init();
    *o = ROOTS[log2n];
}

size_t oracle_fr_fft_domain_len(size_t n) { return valid_size(n) ? n + 2 : 0; }

static void fill_roots(ofr *roots, size_t n, int inverse)
{
    roots_init();
    ofr prim = ROOTS[log2_size(n)];
    if (inverse) ofr_inv(&prim, &prim);
    ofr cur = *ofr_one();
    for (size_t i = 0; i < n; i++) {
        roots[i] = cur;
        ofr_mul(&cur, &cur, &prim);
    }
}

bool oracle_fr_fft_domain_init(ofr *domain, size_t domain_len, size_t n)
{
    size_t req = oracle_fr_fft_domain_len(n);
    if (!domain || req == 0 || domain_len != req) return false;
    fill_roots(domain, n, 0);
    ofr nn;
    ofr_from_u64(&nn, n);
    ofr_inv(&domain[n], &nn);
    domain[n + 1] = nn;
    return true;
}

/* ---- generic radix-2 DIT over G1 (Jacobian) ---- */
static void p1_bit_reverse(op1 *a, size_t n)
{
    for (size_t i = 1, j = 0; i < n; i++) {
        size_t bit = n >> 1;
        for (; j & bit; bit >>= 1) j ^= bit;
        j ^= bit;
        if (i < j) { op1 t = a[i]; a[i] = a[j]; a[j] = t; }
    }
}

static void p1_mult_fr(op1 *o, const op1 *a, const ofr *w)
{
    ofr c;
    uint8_t bytes[32];
    ofr_from_mont(&c, w);
    for (int i = 0; i < 32; i++) bytes[i] = (uint8_t)(c.l[i / 8] >> (8 * (i % 8)));
    op1_mult_vartime(o, a, bytes, 256);
}

static void p1_butterflies(op1 *a, size_t n, const ofr *roots, int inverse_from_forward)
{
    p1_bit_reverse(a, n);
    for (size_t len = 2; len <= n; len <<= 1) {
        size_t half = len / 2;
        for (size_t i = 0; i < n; i += len) {
            op1 u = a[i], t = a[i + half], nt;
            op1_dadd(&a[i], &u, &t);
            op1_neg(&nt, &t);
            op1_dadd(&a[i + half], &u, &nt);
            for (size_t j = 1; j < half; j++) {
                size_t idx = j * (n / len);
                if (inverse_from_forward) idx = n - idx;
                u = a[i + j];
                p1_mult_fr(&t, &a[i + j + half], &roots[idx]);
                op1_dadd(&a[i + j], &u, &t);
                op1_neg(&nt, &t);
                op1_dadd(&a[i + j + half], &u, &nt);
            }
        }
    }
}

static void p1_scale(op1 *a, size_t n, const ofr *s)
{
    for (size_t i = 0; i < n; i++) p1_mult_fr(&a[i], &a[i], s);
}

bool oracle_p1_fft(op1 *values, size_t n, bool inverse)
{
    if (!values || !valid_size(n)) return false;
    ofr *roots = (ofr *)malloc(n * sizeof(ofr));
    if (!roots) return false;
    fill_roots(roots, n, inverse);
    p1_butterflies(values, n, roots, 0);
    if (inverse) {
        ofr nn, inv;
        ofr_from_u64(&nn, n);
        ofr_inv(&inv, &nn);
        p1_scale(values, n, &inv);
    }
    free(roots);
    return true;
}

static bool domain_ok(size_t n, const ofr *domain, size_t domain_len)
{
    size_t req = oracle_fr_fft_domain_len(n);
    if (!domain || req == 0 || domain_len != req) return false;
    ofr tag;
    ofr_from_u64(&tag, n);
    return ofr_eq(&domain[n + 1], &tag);
}

bool oracle_p1_fft_with_domain(op1 *values, size_t n, const ofr *domain, size_t domain_len, bool inverse)
{
    if (!values || !domain_ok(n, domain, domain_len)) return false;
    if (inverse) {
        p1_butterflies(values, n, domain, 1);
        p1_scale(values, n, &domain[n]);
    } else {
        p1_butterflies(values, n, domain, 0);
    }
    return true;
}

/* ---- truncated-prefix forward transform (fft/ctFft.h:132-150 declaration,
 * :384-460 make_fft_truncated_forward_plan, :575-646 the transform).  Inputs
 * [xn, n) are the identity.  After the bit reversal a position is active iff
 * it holds an input below xn; a butterfly runs iff either of its positions is
 * active, and both are active afterwards.  The outputs equal the full forward
 * transform (the reference's TruncatedForwardPrefixMatchesFullG1 test).  Like
 * the reference, the identity tail is the caller's precondition. ---- */
bool oracle_p1_fft_truncated_prefix(op1 *values, size_t n, size_t xn, const ofr *domain, size_t domain_len)
{
    if (!values || !domain_ok(n, domain, domain_len) || xn == 0 || xn > n) return false;
    unsigned char *act = (unsigned char *)calloc(n, 1), *nxt = (unsigned char *)calloc(n, 1);
    if (!act || !nxt) {
        free(act);
        free(nxt);
        return false;
    }
    p1_bit_reverse(values, n);
    for (size_t i = 0; i < n; i++) {
        size_t r = 0;
        for (size_t b = 1, m = n >> 1; b < n; b <<= 1, m >>= 1)
            if (i & b) r |= m;
        act[r] = i < xn;
    }
    for (size_t len = 2; len <= n; len <<= 1) {
        size_t half = len / 2;
        memset(nxt, 0, n);
        for (size_t i = 0; i < n; i += len) {
            for (size_t j = 0; j < half; j++) {
                size_t l = i + j, r = l + half;
                if (!act[l] && !act[r]) continue;
                op1 u = values[l], t = values[r], nt;
                if (j) p1_mult_fr(&t, &values[r], &domain[j * (n / len)]);
                op1_dadd(&values[l], &u, &t);
                op1_neg(&nt, &t);
                op1_dadd(&values[r], &u, &nt);
                nxt[l] = nxt[r] = 1;
            }
        }
        unsigned char *tmp = act;
        act = nxt;
        nxt = tmp;
    }
    free(act);
    free(nxt);
    return true;
}

bool oracle_p1_ifft_unscaled_with_domain(op1 *values, size_t n, const ofr *domain, size_t domain_len)
{
    if (!values || !domain_ok(n, domain, domain_len)) return false;
    p1_butterflies(values, n, domain, 1);
    return true;
}

/* ---- Fr FFT (fft_c_api.cpp:109-182; FrCoeffCtx context.h:25-64) ---- */
static void fr_butterflies(ofr *a, size_t n, const ofr *roots, int inverse_from_forward)
{
    for (size_t i = 1, j = 0; i < n; i++) {
        size_t bit = n >> 1;
        for (; j & bit; bit >>= 1) j ^= bit;
        j ^= bit;
        if (i < j) { ofr t = a[i]; a[i] = a[j]; a[j] = t; }
    }
    const uint64_t *r = ofr_modulus()->l;
    for (size_t len = 2; len <= n; len <<= 1) {
        size_t half = len / 2;
        for (size_t i = 0; i < n; i += len) {
            for (size_t j = 0; j < half; j++) {
                ofr u = a[i + j], t;
                size_t idx = j * (n / len);
                if (inverse_from_forward && j) idx = n - idx;
                if (j) ofr_mul(&t, &a[i + j + half], &roots[idx]);
                else t = a[i + j + half];
                /* u + t, u - t mod r */
                unsigned __int128 c = 0;
                ofr s, d;
                for (int k = 0; k < 4; k++) { c += (unsigned __int128)u.l[k] + t.l[k]; s.l[k] = (uint64_t)c; c >>= 64; }
                int ge = (int)c;
                if (!ge) { ge = 1; for (int k = 3; k >= 0; k--) { if (s.l[k] != r[k]) { ge = s.l[k] > r[k]; break; } } }
                if (ge) { unsigned __int128 b = 0; for (int k = 0; k < 4; k++) { unsigned __int128 x = (unsigned __int128)s.l[k] - r[k] - b; s.l[k] = (uint64_t)x; b = (x >> 64) & 1; } }
                unsigned __int128 b = 0;
                for (int k = 0; k < 4; k++) { unsigned __int128 x = (unsigned __int128)u.l[k] - t.l[k] - b; d.l[k] = (uint64_t)x; b = (x >> 64) & 1; }
                if (b) { c = 0; for (int k = 0; k < 4; k++) { c += (unsigned __int128)d.l[k] + r[k]; d.l[k] = (uint64_t)c; c >>= 64; } }
                a[i + j] = s;
                a[i + j + half] = d;
            }
        }
    }
}

bool oracle_fr_fft(ofr *a, size_t n, bool inverse)
{
    if (!a || !valid_size(n)) return false;
    ofr *roots = (ofr *)malloc(n * sizeof(ofr));
    if (!roots) return false;
    fill_roots(roots, n, inverse);
    fr_butterflies(a, n, roots, 0);
    if (inverse) {
        ofr nn, inv;
        ofr_from_u64(&nn, n);
        ofr_inv(&inv, &nn);
        for (size_t i = 0; i < n; i++) ofr_mul(&a[i], &a[i], &inv);
    }
    free(roots);
    return true;
}

bool oracle_fr_fft_with_domain(ofr *a, size_t n, const ofr *domain, size_t domain_len, bool inverse)
{
    if (!a || !domain_ok(n, domain, domain_len)) return false;
    fr_butterflies(a, n, domain, inverse ? 1 : 0);
    if (inverse)
        for (size_t i = 0; i < n; i++) ofr_mul(&a[i], &a[i], &domain[n]);
    return true;
}
