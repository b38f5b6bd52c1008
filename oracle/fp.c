/*
 * Oracle field arithmetic (test infrastructure only; see oracle.h).
 *
 * Restates the reference's Montgomery arithmetic on 64-bit limbs:
 *   Fp: scalar/fields/Fp.h:290-330 (add/sub/mul/sqr), backend_portable.h:386
 *       (cc_mul_mont_n, CIOS) and :510 (cc_redc_mont_n).  R = 2^384.
 *   Fr: scalar/fields/Fr.h:44-125, :587 (mul).  R = 2^256.
 * Outputs are fully reduced ([0, modulus)), as in the reference, so the
 * Montgomery bytes are directly comparable with the reference ABI types.
 * The Montgomery constants are derived at start-up from the moduli alone.
 */
#include "oracle.h"
#include <string.h>

typedef unsigned __int128 u128;

static uint64_t P[6], P_R[6], P_R2[6], P_N0;
static uint64_t Q[4], Q_R[4], Q_R2[4], Q_N0;
static int inited;

static void from_hex(uint64_t *out, int n, const char *hex)
{
    memset(out, 0, 8 * (size_t)n);
    size_t len = strlen(hex);
    for (size_t i = 0; i < len; i++) {
        char c = hex[len - 1 - i];
        uint64_t v = (c >= '0' && c <= '9') ? (uint64_t)(c - '0')
                   : (c >= 'a' && c <= 'f') ? (uint64_t)(c - 'a' + 10)
                   : (uint64_t)(c - 'A' + 10);
        out[i / 16] |= v << (4 * (i % 16));
    }
}

static int geq_n(const uint64_t *a, const uint64_t *b, int n)
{
    for (int i = n - 1; i >= 0; i--) {
        if (a[i] != b[i]) return a[i] > b[i];
    }
    return 1;
}

static uint64_t sub_n(uint64_t *o, const uint64_t *a, const uint64_t *b, int n)
{
    uint64_t borrow = 0;
    for (int i = 0; i < n; i++) {
        u128 d = (u128)a[i] - b[i] - borrow;
        o[i] = (uint64_t)d;
        borrow = (uint64_t)(d >> 64) & 1;
    }
    return borrow;
}

static uint64_t add_n(uint64_t *o, const uint64_t *a, const uint64_t *b, int n)
{
    uint64_t carry = 0;
    for (int i = 0; i < n; i++) {
        u128 s = (u128)a[i] + b[i] + carry;
        o[i] = (uint64_t)s;
        carry = (uint64_t)(s >> 64);
    }
    return carry;
}

/* o = 2*a mod m, a < m */
static void dbl_mod(uint64_t *o, const uint64_t *a, const uint64_t *m, int n)
{
    uint64_t t[8];
    uint64_t carry = add_n(t, a, a, n);
    if (carry || geq_n(t, m, n)) sub_n(t, t, m, n);
    memcpy(o, t, 8 * (size_t)n);
}

static uint64_t neg_inv64(uint64_t m0)
{
    /* Newton iteration for m0^-1 mod 2^64, then negate. */
    uint64_t x = m0;               /* correct to 3 bits for odd m0 */
    for (int i = 0; i < 6; i++) x *= 2 - m0 * x;
    return (uint64_t)0 - x;
}

/* CIOS Montgomery multiplication, n <= 6 limbs: o = a*b*2^(-64n) mod m. */
static void mont_mul(uint64_t *o, const uint64_t *a, const uint64_t *b,
                     const uint64_t *m, uint64_t n0, int n)
{
    uint64_t t[8] = {0};
    for (int i = 0; i < n; i++) {
        u128 c = 0;
        for (int j = 0; j < n; j++) {
            c += (u128)a[j] * b[i] + t[j];
            t[j] = (uint64_t)c;
            c >>= 64;
        }
        c += t[n];
        t[n] = (uint64_t)c;
        t[n + 1] = (uint64_t)(c >> 64);

        uint64_t mm = t[0] * n0;
        c = (u128)mm * m[0] + t[0];
        c >>= 64;
        for (int j = 1; j < n; j++) {
            c += (u128)mm * m[j] + t[j];
            t[j - 1] = (uint64_t)c;
            c >>= 64;
        }
        c += t[n];
        t[n - 1] = (uint64_t)c;
        t[n] = t[n + 1] + (uint64_t)(c >> 64);
    }
    if (t[n] || geq_n(t, m, n)) sub_n(t, t, m, n);
    memcpy(o, t, 8 * (size_t)n);
}

void oracle_init(void)
{
    if (inited) return;
    from_hex(P, 6, "1a0111ea397fe69a4b1ba7b6434bacd764774b84f38512bf6730d2a0f6b0f6241eabfffeb153ffffb9feffffffffaaab");
    from_hex(Q, 4, "73eda753299d7d483339d80809a1d80553bda402fffe5bfeffffffff00000001");
    P_N0 = neg_inv64(P[0]);
    Q_N0 = neg_inv64(Q[0]);
    /* R mod m by doubling 1 (64n) times; R^2 by doubling a further 64n times. */
    uint64_t t[8] = {1};
    for (int i = 0; i < 384; i++) dbl_mod(t, t, P, 6);
    memcpy(P_R, t, 48);
    for (int i = 0; i < 384; i++) dbl_mod(t, t, P, 6);
    memcpy(P_R2, t, 48);
    uint64_t u[8] = {1};
    for (int i = 0; i < 256; i++) dbl_mod(u, u, Q, 4);
    memcpy(Q_R, u, 32);
    for (int i = 0; i < 256; i++) dbl_mod(u, u, Q, 4);
    memcpy(Q_R2, u, 32);
    inited = 1;
}

const ofp *ofp_modulus(void) { return (const ofp *)P; }
const ofr *ofr_modulus(void) { return (const ofr *)Q; }
const ofp *ofp_one(void) { return (const ofp *)P_R; }
const ofr *ofr_one(void) { return (const ofr *)Q_R; }

void ofp_mul(ofp *o, const ofp *a, const ofp *b) { mont_mul(o->l, a->l, b->l, P, P_N0, 6); }
void ofp_sqr(ofp *o, const ofp *a) { mont_mul(o->l, a->l, a->l, P, P_N0, 6); }

void ofp_add(ofp *o, const ofp *a, const ofp *b)
{
    uint64_t t[6];
    uint64_t c = add_n(t, a->l, b->l, 6);
    if (c || geq_n(t, P, 6)) sub_n(t, t, P, 6);
    memcpy(o->l, t, 48);
}

void ofp_sub(ofp *o, const ofp *a, const ofp *b)
{
    uint64_t t[6];
    if (sub_n(t, a->l, b->l, 6)) add_n(t, t, P, 6);
    memcpy(o->l, t, 48);
}

bool ofp_is_zero(const ofp *a)
{
    uint64_t acc = 0;
    for (int i = 0; i < 6; i++) acc |= a->l[i];
    return acc == 0;
}

bool ofp_eq(const ofp *a, const ofp *b) { return memcmp(a, b, 48) == 0; }

void ofp_neg(ofp *o, const ofp *a)
{
    if (ofp_is_zero(a)) { memset(o, 0, 48); return; }
    sub_n(o->l, P, a->l, 6);
}

void ofp_from_mont(ofp *o, const ofp *a)
{
    uint64_t one[6] = {1};
    mont_mul(o->l, a->l, one, P, P_N0, 6);
}

void ofp_to_mont(ofp *o, const ofp *a) { mont_mul(o->l, a->l, P_R2, P, P_N0, 6); }

/* Fermat inversion a^(p-2); inverse of zero is zero. */
void ofp_inv(ofp *o, const ofp *a)
{
    uint64_t e[6];
    uint64_t two[6] = {2};
    sub_n(e, P, two, 6);
    ofp r = *ofp_one();
    ofp b = *a;
    for (int i = 0; i < 384; i++) {
        if ((e[i / 64] >> (i % 64)) & 1) ofp_mul(&r, &r, &b);
        ofp_sqr(&b, &b);
    }
    *o = r;
}

void ofr_mul(ofr *o, const ofr *a, const ofr *b) { mont_mul(o->l, a->l, b->l, Q, Q_N0, 4); }
void ofr_sqr(ofr *o, const ofr *a) { mont_mul(o->l, a->l, a->l, Q, Q_N0, 4); }

void ofr_from_mont(ofr *o, const ofr *a)
{
    uint64_t one[4] = {1};
    mont_mul(o->l, a->l, one, Q, Q_N0, 4);
}

void ofr_to_mont(ofr *o, const ofr *a) { mont_mul(o->l, a->l, Q_R2, Q, Q_N0, 4); }

void ofr_from_u64(ofr *o, uint64_t v)
{
    ofr t = {{v, 0, 0, 0}};
    ofr_to_mont(o, &t);
}

bool ofr_eq(const ofr *a, const ofr *b) { return memcmp(a, b, 32) == 0; }

void ofr_inv(ofr *o, const ofr *a)
{
    uint64_t e[4];
    uint64_t two[4] = {2};
    sub_n(e, Q, two, 4);
    ofr r = *ofr_one();
    ofr b = *a;
    for (int i = 0; i < 256; i++) {
        if ((e[i / 64] >> (i % 64)) & 1) ofr_mul(&r, &r, &b);
        ofr_sqr(&b, &b);
    }
    *o = r;
}
