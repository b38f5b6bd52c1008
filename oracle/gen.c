/*
 * Seeded synthetic inputs for the checks (test infrastructure only).
 *
 * Scalars: splitmix64 stream, four outputs per candidate (little-endian
 * limbs), top bit cleared, accepted iff < r (uniform Fr, at most 255 bits).
 * Points: P_i = k_i * G via a fixed-base byte comb (32 tables of 255 affine
 * multiples of 2^(8j) G), then batch normalisation to affine.  The affine
 * Montgomery bytes of k*G are unique, so any correct generator (the device
 * one included) yields the same bytes.
 */
#include "oracle.h"
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

uint64_t oracle_splitmix64(uint64_t *state)
{
    uint64_t z = (*state += 0x9e3779b97f4a7c15ULL);
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
    return z ^ (z >> 31);
}

static int lt_r(const uint64_t l[4])
{
    const uint64_t *r = ofr_modulus()->l;
    for (int i = 3; i >= 0; i--) {
        if (l[i] != r[i]) return l[i] < r[i];
    }
    return 0;
}

static void put_le(uint8_t *out, const uint64_t l[4])
{
    for (int i = 0; i < 32; i++) out[i] = (uint8_t)(l[i / 8] >> (8 * (i % 8)));
}

void oracle_gen_scalars(uint64_t seed, size_t n, int kind, uint8_t *out32)
{
    oracle_init();
    uint64_t st = seed;
    for (size_t i = 0; i < n; i++) {
        uint64_t l[4] = {0, 0, 0, 0};
        if (kind == 1) {
            l[0] = oracle_splitmix64(&st);
        } else {
            do {
                for (int k = 0; k < 4; k++) l[k] = oracle_splitmix64(&st);
                l[3] &= 0x7fffffffffffffffULL;
            } while (!lt_r(l));
        }
        put_le(out32 + 32 * i, l);
    }
    if (kind == 2) {
        uint64_t st2 = seed ^ 0x5eed5eed5eed5eedULL;
        for (size_t i = 0; i < n; i++) {
            if (oracle_splitmix64(&st2) % 10 == 0) memset(out32 + 32 * i, 0, 32);
        }
    }
}

void oracle_duplicate_points(uint64_t seed, size_t n, op1a *points)
{
    uint64_t st = seed ^ 0xd0b1ed0b1ed0b1edULL;
    for (size_t i = 0; i < n; i++) {
        uint64_t u = oracle_splitmix64(&st);
        uint64_t v = oracle_splitmix64(&st);
        if (u % 20 == 0) points[i] = points[v % n];
    }
}

/* ---- fixed-base comb ---- */
static op1a *COMB;          /* 32 x 256 entries; entry 0 of each row = infinity */
static pthread_mutex_t comb_lock = PTHREAD_MUTEX_INITIALIZER;

static void batch_to_affine(op1a *out, const op1 *in, size_t n)
{
    ofp *pref = (ofp *)malloc((n + 1) * sizeof(ofp));
    ofp acc = *ofp_one();
    for (size_t i = 0; i < n; i++) {
        pref[i] = acc;
        if (!op1_is_inf(&in[i])) ofp_mul(&acc, &acc, &in[i].z);
    }
    ofp inv;
    ofp_inv(&inv, &acc);
    for (size_t i = n; i-- > 0;) {
        if (op1_is_inf(&in[i])) { memset(&out[i], 0, sizeof(op1a)); continue; }
        ofp zi, zi2, zi3;
        ofp_mul(&zi, &inv, &pref[i]);
        ofp_mul(&inv, &inv, &in[i].z);
        ofp_sqr(&zi2, &zi);
        ofp_mul(&zi3, &zi2, &zi);
        ofp_mul(&out[i].x, &in[i].x, &zi2);
        ofp_mul(&out[i].y, &in[i].y, &zi3);
    }
    free(pref);
}

static void comb_init(void)
{
    pthread_mutex_lock(&comb_lock);
    if (!COMB) {
        oracle_init();
        op1 *jac = (op1 *)malloc(32 * 256 * sizeof(op1));
        op1 base;
        op1_generator(&base);
        for (int j = 0; j < 32; j++) {
            memset(&jac[j * 256], 0, sizeof(op1));
            jac[j * 256 + 1] = base;
            for (int b = 2; b < 256; b++) op1_dadd(&jac[j * 256 + b], &jac[j * 256 + b - 1], &base);
            for (int d = 0; d < 8; d++) op1_double(&base, &base);
        }
        op1a *t = (op1a *)malloc(32 * 256 * sizeof(op1a));
        batch_to_affine(t, jac, 32 * 256);
        free(jac);
        COMB = t;
    }
    pthread_mutex_unlock(&comb_lock);
}

typedef struct { const uint8_t *k; op1a *out; size_t lo, hi; } gen_job;

static void *gen_worker(void *arg)
{
    gen_job *j = (gen_job *)arg;
    size_t m = j->hi - j->lo;
    op1 *jac = (op1 *)malloc((m ? m : 1) * sizeof(op1));
    for (size_t i = 0; i < m; i++) {
        const uint8_t *k = j->k + 32 * (j->lo + i);
        op1xyzz acc;
        memset(&acc, 0, sizeof(acc));
        for (int b = 0; b < 32; b++) {
            if (k[b]) oxyzz_madd(&acc, &acc, &COMB[b * 256 + k[b]], 0);
        }
        oxyzz_to_jacobian(&jac[i], &acc);
    }
    batch_to_affine(j->out + j->lo, jac, m);
    free(jac);
    return NULL;
}

void oracle_points_from_scalars(const uint8_t *k32, size_t n, op1a *out, int nthreads)
{
    comb_init();
    if (nthreads < 1) nthreads = 1;
    if ((size_t)nthreads > n) nthreads = n ? (int)n : 1;
    pthread_t *th = (pthread_t *)malloc(sizeof(pthread_t) * (size_t)nthreads);
    gen_job *jobs = (gen_job *)malloc(sizeof(gen_job) * (size_t)nthreads);
    for (int t = 0; t < nthreads; t++) {
        jobs[t].k = k32;
        jobs[t].out = out;
        jobs[t].lo = n * (size_t)t / (size_t)nthreads;
        jobs[t].hi = n * (size_t)(t + 1) / (size_t)nthreads;
        pthread_create(&th[t], NULL, gen_worker, &jobs[t]);
    }
    for (int t = 0; t < nthreads; t++) pthread_join(th[t], NULL);
    free(th);
    free(jobs);
}

void oracle_jacobian_randomize(uint64_t seed, size_t n, const op1a *in, op1 *out)
{
    oracle_init();
    uint64_t st = seed ^ 0x1ac0b1a11ac0b1a1ULL;
    for (size_t i = 0; i < n; i++) {
        if (ofp_is_zero(&in[i].x) && ofp_is_zero(&in[i].y)) { memset(&out[i], 0, sizeof(op1)); continue; }
        ofp z, zm, z2, z3;
        do {
            for (int k = 0; k < 6; k++) z.l[k] = oracle_splitmix64(&st);
            z.l[5] &= 0x0fffffffffffffffULL;
        } while (ofp_is_zero(&z) || !(z.l[5] < ofp_modulus()->l[5]));
        ofp_to_mont(&zm, &z);
        ofp_sqr(&z2, &zm);
        ofp_mul(&z3, &z2, &zm);
        ofp_mul(&out[i].x, &in[i].x, &z2);
        ofp_mul(&out[i].y, &in[i].y, &z3);
        out[i].z = zm;
    }
}
