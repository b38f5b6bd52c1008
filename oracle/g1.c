/*
 * Oracle G1 arithmetic (test infrastructure only; see oracle.h).
 *
 * Restates scalar/curve/point.cpp:
 *   neg :618, from_jacobian/to_affine :628-660, compress/serialize :765-905,
 *   Jacobian add (Point::dadd) :1623, doubling :1898, mult_vartime :1546
 *   (window for nbits < 176, else GLV + wNAF-5, :1319/:1419),
 *   XYZZ add :1939, XYZZ mixed add/sub :2028-2103, XYZZ->Jacobian :2109.
 * The Jacobian add here is the textbook add with explicit infinity/doubling/
 * opposite branches; its affine results equal the reference's unified add.
 */
#include "oracle.h"
#include <string.h>

typedef unsigned __int128 u128;

static const char *GX = "17f1d3a73197d7942695638c4fa9ac0fc3688c4f9774b905a14e3a3f171bac586c55e83ff97a1aeffb3af00adb22c6bb";
static const char *GY = "08b3f481e3aaa0f1a09e30ed741d8ae4fcf5e095d5d00af600db18cb2c04b3edd03cc744a2888ae40caa232946c5e7e1";

static void hex_le(uint64_t *out, int n, const char *hex)
{
    memset(out, 0, 8 * (size_t)n);
    size_t len = strlen(hex);
    for (size_t i = 0; i < len; i++) {
        char c = hex[len - 1 - i];
        uint64_t v = (c >= '0' && c <= '9') ? (uint64_t)(c - '0') : (uint64_t)(c - 'a' + 10);
        out[i / 16] |= v << (4 * (i % 16));
    }
}

void op1_generator(op1 *o)
{
    ofp x, y;
    hex_le(x.l, 6, GX);
    hex_le(y.l, 6, GY);
    ofp_to_mont(&o->x, &x);
    ofp_to_mont(&o->y, &y);
    o->z = *ofp_one();
}

bool op1_is_inf(const op1 *p) { return ofp_is_zero(&p->z); }

void op1_from_affine(op1 *o, const op1a *a)
{
    o->x = a->x;
    o->y = a->y;
    if (ofp_is_zero(&a->x) && ofp_is_zero(&a->y)) memset(&o->z, 0, 48);
    else o->z = *ofp_one();
}

void op1_to_affine(op1a *o, const op1 *p)
{
    if (op1_is_inf(p)) { memset(o, 0, sizeof(*o)); return; }
    ofp zi, zi2, zi3;
    ofp_inv(&zi, &p->z);
    ofp_sqr(&zi2, &zi);
    ofp_mul(&zi3, &zi2, &zi);
    ofp_mul(&o->x, &p->x, &zi2);
    ofp_mul(&o->y, &p->y, &zi3);
}

void op1_neg(op1 *o, const op1 *p)
{
    o->x = p->x;
    ofp_neg(&o->y, &p->y);
    o->z = p->z;
}

/* dbl-2009-l for a = 0 */
void op1_double(op1 *o, const op1 *p)
{
    if (op1_is_inf(p)) { *o = *p; return; }
    ofp A, B, C, D, E, F, t;
    ofp_sqr(&A, &p->x);
    ofp_sqr(&B, &p->y);
    ofp_sqr(&C, &B);
    ofp_add(&t, &p->x, &B);
    ofp_sqr(&t, &t);
    ofp_sub(&t, &t, &A);
    ofp_sub(&t, &t, &C);
    ofp_add(&D, &t, &t);
    ofp_add(&E, &A, &A);
    ofp_add(&E, &E, &A);
    ofp_sqr(&F, &E);
    ofp Z3;
    ofp_mul(&Z3, &p->y, &p->z);
    ofp_add(&Z3, &Z3, &Z3);
    ofp X3;
    ofp_sub(&X3, &F, &D);
    ofp_sub(&X3, &X3, &D);
    ofp Y3;
    ofp_sub(&t, &D, &X3);
    ofp_mul(&Y3, &E, &t);
    ofp_add(&C, &C, &C);
    ofp_add(&C, &C, &C);
    ofp_add(&C, &C, &C);
    ofp_sub(&Y3, &Y3, &C);
    o->x = X3; o->y = Y3; o->z = Z3;
}

void op1_dadd(op1 *o, const op1 *a, const op1 *b)
{
    if (op1_is_inf(a)) { *o = *b; return; }
    if (op1_is_inf(b)) { *o = *a; return; }
    ofp z1z1, z2z2, u1, u2, s1, s2, h, r, t;
    ofp_sqr(&z1z1, &a->z);
    ofp_sqr(&z2z2, &b->z);
    ofp_mul(&u1, &a->x, &z2z2);
    ofp_mul(&u2, &b->x, &z1z1);
    ofp_mul(&s1, &a->y, &b->z);
    ofp_mul(&s1, &s1, &z2z2);
    ofp_mul(&s2, &b->y, &a->z);
    ofp_mul(&s2, &s2, &z1z1);
    ofp_sub(&h, &u2, &u1);
    ofp_sub(&r, &s2, &s1);
    if (ofp_is_zero(&h)) {
        if (ofp_is_zero(&r)) { op1_double(o, a); return; }
        memset(o, 0, sizeof(*o));
        return;
    }
    ofp hh, hhh, v, X3, Y3, Z3;
    ofp_sqr(&hh, &h);
    ofp_mul(&hhh, &hh, &h);
    ofp_mul(&v, &u1, &hh);
    ofp_sqr(&X3, &r);
    ofp_sub(&X3, &X3, &hhh);
    ofp_sub(&X3, &X3, &v);
    ofp_sub(&X3, &X3, &v);
    ofp_sub(&t, &v, &X3);
    ofp_mul(&Y3, &r, &t);
    ofp_mul(&t, &s1, &hhh);
    ofp_sub(&Y3, &Y3, &t);
    ofp_mul(&Z3, &a->z, &b->z);
    ofp_mul(&Z3, &Z3, &h);
    o->x = X3; o->y = Y3; o->z = Z3;
}

bool op1_on_curve(const op1 *p)
{
    if (op1_is_inf(p)) return true;
    /* Y^2 = X^3 + 4 Z^6 */
    ofp y2, x3, z2, z6, four, t;
    ofp_sqr(&y2, &p->y);
    ofp_sqr(&x3, &p->x);
    ofp_mul(&x3, &x3, &p->x);
    ofp_sqr(&z2, &p->z);
    ofp_mul(&z6, &z2, &z2);
    ofp_mul(&z6, &z6, &z2);
    ofp_add(&four, ofp_one(), ofp_one());
    ofp_add(&four, &four, &four);
    ofp_mul(&t, &z6, &four);
    ofp_add(&t, &t, &x3);
    return ofp_eq(&t, &y2);
}

/* ---- XYZZ (point.cpp:1939-2113) ---- */
static bool xyzz_is_inf(const op1xyzz *p) { return ofp_is_zero(&p->zz) && ofp_is_zero(&p->zzz); }

void oxyzz_madd(op1xyzz *o, const op1xyzz *a, const op1a *b, int subtract)
{
    if (ofp_is_zero(&b->x) && ofp_is_zero(&b->y)) { *o = *a; return; }
    ofp by = b->y;
    if (subtract) ofp_neg(&by, &b->y);
    if (xyzz_is_inf(a)) {
        o->x = b->x; o->y = by; o->zz = *ofp_one(); o->zzz = *ofp_one();
        return;
    }
    ofp P, R;
    ofp_mul(&P, &b->x, &a->zz);
    ofp_mul(&R, &by, &a->zzz);
    ofp_sub(&P, &P, &a->x);
    ofp_sub(&R, &R, &a->y);
    if (!ofp_is_zero(&P)) {
        ofp PP, PPP, Qv, X3, Y3, t;
        ofp_sqr(&PP, &P);
        ofp_mul(&PPP, &PP, &P);
        ofp_mul(&Qv, &a->x, &PP);
        ofp_sqr(&X3, &R);
        ofp_sub(&X3, &X3, &PPP);
        ofp_sub(&X3, &X3, &Qv);
        ofp_sub(&X3, &X3, &Qv);
        ofp_sub(&t, &Qv, &X3);
        ofp_mul(&Y3, &t, &R);
        ofp_mul(&t, &a->y, &PPP);
        ofp_sub(&Y3, &Y3, &t);
        ofp_mul(&o->zz, &a->zz, &PP);
        ofp_mul(&o->zzz, &a->zzz, &PPP);
        o->x = X3; o->y = Y3;
    } else if (ofp_is_zero(&R)) {
        /* mdbl-2008-s on (b.x, by) */
        ofp U, V, W, S, M, X3, Y3, t;
        ofp_add(&U, &by, &by);
        ofp_sqr(&V, &U);
        ofp_mul(&W, &V, &U);
        ofp_mul(&S, &b->x, &V);
        ofp_sqr(&M, &b->x);
        ofp_add(&t, &M, &M);
        ofp_add(&M, &t, &M);
        ofp_sqr(&X3, &M);
        ofp_sub(&X3, &X3, &S);
        ofp_sub(&X3, &X3, &S);
        ofp_sub(&t, &S, &X3);
        ofp_mul(&Y3, &M, &t);
        ofp_mul(&t, &W, &by);
        ofp_sub(&Y3, &Y3, &t);
        o->x = X3; o->y = Y3; o->zz = V; o->zzz = W;
    } else {
        memset(o, 0, sizeof(*o));
    }
}

static void xyzz_dbl(op1xyzz *o, const op1xyzz *a)
{
    if (xyzz_is_inf(a)) { *o = *a; return; }
    ofp U, V, W, S, M, X3, Y3, t;
    ofp_add(&U, &a->y, &a->y);
    ofp_sqr(&V, &U);
    ofp_mul(&W, &V, &U);
    ofp_mul(&S, &a->x, &V);
    ofp_sqr(&M, &a->x);
    ofp_add(&t, &M, &M);
    ofp_add(&M, &t, &M);
    ofp_sqr(&X3, &M);
    ofp_sub(&X3, &X3, &S);
    ofp_sub(&X3, &X3, &S);
    ofp_sub(&t, &S, &X3);
    ofp_mul(&Y3, &M, &t);
    ofp_mul(&t, &W, &a->y);
    ofp_sub(&Y3, &Y3, &t);
    ofp_mul(&o->zz, &V, &a->zz);
    ofp_mul(&o->zzz, &W, &a->zzz);
    o->x = X3; o->y = Y3;
}

void oxyzz_add(op1xyzz *o, const op1xyzz *a, const op1xyzz *b)
{
    if (xyzz_is_inf(a)) { *o = *b; return; }
    if (xyzz_is_inf(b)) { *o = *a; return; }
    ofp U1, U2, S1, S2, P, R;
    ofp_mul(&U1, &a->x, &b->zz);
    ofp_mul(&U2, &b->x, &a->zz);
    ofp_mul(&S1, &a->y, &b->zzz);
    ofp_mul(&S2, &b->y, &a->zzz);
    ofp_sub(&P, &U2, &U1);
    ofp_sub(&R, &S2, &S1);
    if (ofp_is_zero(&P)) {
        if (ofp_is_zero(&R)) { xyzz_dbl(o, a); return; }
        memset(o, 0, sizeof(*o));
        return;
    }
    ofp PP, PPP, Qv, X3, Y3, t;
    ofp_sqr(&PP, &P);
    ofp_mul(&PPP, &PP, &P);
    ofp_mul(&Qv, &U1, &PP);
    ofp_sqr(&X3, &R);
    ofp_sub(&X3, &X3, &PPP);
    ofp_sub(&X3, &X3, &Qv);
    ofp_sub(&X3, &X3, &Qv);
    ofp_sub(&t, &Qv, &X3);
    ofp_mul(&Y3, &R, &t);
    ofp_mul(&t, &S1, &PPP);
    ofp_sub(&Y3, &Y3, &t);
    ofp_mul(&o->zz, &a->zz, &b->zz);
    ofp_mul(&o->zz, &o->zz, &PP);
    ofp_mul(&o->zzz, &a->zzz, &b->zzz);
    ofp_mul(&o->zzz, &o->zzz, &PPP);
    o->x = X3; o->y = Y3;
}

void oxyzz_to_jacobian(op1 *o, const op1xyzz *a)
{
    if (xyzz_is_inf(a)) { memset(o, 0, sizeof(*o)); return; }
    ofp_mul(&o->x, &a->x, &a->zz);
    ofp_mul(&o->y, &a->y, &a->zzz);
    o->z = a->zz;
}

/* ---- serialization (point.cpp:765-905) ---- */
static void be48(uint8_t *out, const ofp *mont)
{
    ofp t;
    ofp_from_mont(&t, mont);
    for (int i = 0; i < 48; i++) out[47 - i] = (uint8_t)(t.l[i / 8] >> (8 * (i % 8)));
}

/* 1 iff canonical y > (p-1)/2 */
static int y_is_large(const ofp *ymont)
{
    ofp y, ny;
    ofp_from_mont(&y, ymont);
    /* compare y with p - y */
    ofp_neg(&ny, &y);
    for (int i = 5; i >= 0; i--) {
        if (y.l[i] != ny.l[i]) return y.l[i] > ny.l[i];
    }
    return 0;
}

void op1_compress(uint8_t out[48], const op1 *p)
{
    if (op1_is_inf(p)) { memset(out, 0, 48); out[0] = 0xc0; return; }
    op1a a;
    op1_to_affine(&a, p);
    be48(out, &a.x);
    out[0] |= (uint8_t)(0x80 | (y_is_large(&a.y) << 5));
}

void op1_affine_serialize(uint8_t out[96], const op1a *a)
{
    if (ofp_is_zero(&a->x) && ofp_is_zero(&a->y)) { memset(out, 0, 96); out[0] = 0x40; return; }
    be48(out, &a->x);
    be48(out + 48, &a->y);
}

void op1_serialize(uint8_t out[96], const op1 *p)
{
    if (op1_is_inf(p)) { memset(out, 0, 96); out[0] = 0x40; return; }
    op1a a;
    op1_to_affine(&a, p);
    be48(out, &a.x);
    be48(out + 48, &a.y);
}

/* ---- scalar multiplication (point.cpp:1546-1565) ---- */

/* Canonical 256-bit scalar: nbits-masked, then reduced mod r
 * (scalar/fields/Fr.h:326 canonical_scalar_256_vartime). */
static void canonical_scalar(uint64_t k[4], const uint8_t *scalar, size_t nbits)
{
    uint8_t masked[32] = {0};
    size_t nbytes = (nbits + 7) / 8;
    if (nbytes) {
        memcpy(masked, scalar, nbytes);
        if (nbits & 7) masked[nbytes - 1] &= (uint8_t)((1u << (nbits & 7)) - 1);
    }
    for (int i = 0; i < 4; i++) {
        k[i] = 0;
        for (int b = 0; b < 8; b++) k[i] |= (uint64_t)masked[8 * i + b] << (8 * b);
    }
    const uint64_t *r = ofr_modulus()->l;
    for (;;) {
        int ge = 1;
        for (int i = 3; i >= 0; i--) {
            if (k[i] != r[i]) { ge = k[i] > r[i]; break; }
        }
        if (!ge) break;
        uint64_t borrow = 0;
        for (int i = 0; i < 4; i++) {
            u128 d = (u128)k[i] - r[i] - borrow;
            k[i] = (uint64_t)d;
            borrow = (uint64_t)(d >> 64) & 1;
        }
    }
}

/* width-w NAF digits of a little-endian multi-limb integer; returns length */
static int wnaf(int8_t *digits, const uint64_t *k_in, int nlimbs, int w)
{
    uint64_t k[5] = {0};
    for (int i = 0; i < nlimbs; i++) k[i] = k_in[i];
    int len = 0;
    const int64_t half = (int64_t)1 << (w - 1), full = (int64_t)1 << w;
    for (;;) {
        int nz = 0;
        for (int i = 0; i < 5; i++) nz |= k[i] != 0;
        if (!nz) break;
        int8_t d = 0;
        if (k[0] & 1) {
            int64_t v = (int64_t)(k[0] & (uint64_t)(full - 1));
            if (v >= half) v -= full;
            d = (int8_t)v;
            /* k -= d */
            if (v > 0) {
                uint64_t borrow = (uint64_t)v;
                for (int i = 0; i < 5 && borrow; i++) { uint64_t o = k[i]; k[i] -= borrow; borrow = o < borrow; }
            } else {
                uint64_t carry = (uint64_t)(-v);
                for (int i = 0; i < 5 && carry; i++) { k[i] += carry; carry = k[i] < carry; }
            }
        }
        digits[len++] = d;
        for (int i = 0; i < 4; i++) k[i] = (k[i] >> 1) | (k[i + 1] << 63);
        k[4] >>= 1;
    }
    return len;
}

static ofp BETA;
static uint64_t LAMBDA[2];
static int glv_ready;

static void plain_mult(op1 *o, const op1 *p, const uint64_t *k, int nlimbs)
{
    /* wNAF-5 double-and-add, exact for any curve point */
    int8_t d[300];
    int len = wnaf(d, k, nlimbs, 5);
    op1 tbl[8], p2;
    tbl[0] = *p;
    op1_double(&p2, p);
    for (int i = 1; i < 8; i++) op1_dadd(&tbl[i], &tbl[i - 1], &p2);
    op1 acc;
    memset(&acc, 0, sizeof(acc));
    for (int i = len - 1; i >= 0; i--) {
        op1_double(&acc, &acc);
        if (d[i] > 0) op1_dadd(&acc, &acc, &tbl[(d[i] - 1) / 2]);
        else if (d[i] < 0) { op1 t; op1_neg(&t, &tbl[(-d[i] - 1) / 2]); op1_dadd(&acc, &acc, &t); }
    }
    *o = acc;
}

/* GLV set-up: lambda = z^2 - 1 (a cube root of unity mod r), beta a cube
 * root of unity in Fp chosen so that (beta*x, y) = lambda * (x, y) on G1. */
static void glv_init(void)
{
    if (glv_ready) return;
    LAMBDA[0] = 0x00000000ffffffffULL;
    LAMBDA[1] = 0xac45a4010001a402ULL;
    /* beta = g^((p-1)/3) for the first g giving a nontrivial cube root */
    uint64_t e[6];
    const uint64_t *pm = ofp_modulus()->l;
    /* e = (p-1)/3 */
    {
        u128 rem = 0;
        uint64_t pm1[6];
        memcpy(pm1, pm, 48);
        pm1[0] -= 1;
        for (int i = 5; i >= 0; i--) {
            u128 cur = (rem << 64) | pm1[i];
            e[i] = (uint64_t)(cur / 3);
            rem = cur % 3;
        }
    }
    for (uint64_t g = 2;; g++) {
        ofp gm, t = {{g}}, r = *ofp_one();
        ofp_to_mont(&gm, &t);
        for (int i = 383; i >= 0; i--) {
            ofp_sqr(&r, &r);
            if ((e[i / 64] >> (i % 64)) & 1) ofp_mul(&r, &r, &gm);
        }
        if (!ofp_eq(&r, ofp_one())) { BETA = r; break; }
    }
    op1 G, lg, bg;
    op1_generator(&G);
    uint64_t lam4[4] = {LAMBDA[0], LAMBDA[1], 0, 0};
    plain_mult(&lg, &G, lam4, 4);
    bg = G;
    ofp_mul(&bg.x, &G.x, &BETA);
    op1a a1, a2;
    op1_to_affine(&a1, &lg);
    op1_to_affine(&a2, &bg);
    if (!ofp_eq(&a1.x, &a2.x)) ofp_sqr(&BETA, &BETA);
    glv_ready = 1;
}

static void glv_mult(op1 *o, const op1 *p, const uint64_t k[4])
{
    glv_init();
    /* k = k1 + lambda*k2 by binary long division */
    uint64_t q[4] = {0}, rem[3] = {0};
    for (int i = 255; i >= 0; i--) {
        rem[2] = (rem[2] << 1) | (rem[1] >> 63);
        rem[1] = (rem[1] << 1) | (rem[0] >> 63);
        rem[0] = (rem[0] << 1) | ((k[i / 64] >> (i % 64)) & 1);
        int ge = rem[2] || rem[1] > LAMBDA[1] || (rem[1] == LAMBDA[1] && rem[0] >= LAMBDA[0]);
        if (ge) {
            u128 d = (u128)rem[0] - LAMBDA[0];
            rem[0] = (uint64_t)d;
            uint64_t b = (uint64_t)(d >> 64) & 1;
            d = (u128)rem[1] - LAMBDA[1] - b;
            rem[1] = (uint64_t)d;
            b = (uint64_t)(d >> 64) & 1;
            rem[2] -= b;
            q[i / 64] |= (uint64_t)1 << (i % 64);
        }
    }
    int8_t d1[300], d2[300];
    int l1 = wnaf(d1, rem, 2, 5);
    int l2 = wnaf(d2, q, 4, 5);
    op1 t1[8], t2[8], p2;
    t1[0] = *p;
    op1_double(&p2, p);
    for (int i = 1; i < 8; i++) op1_dadd(&t1[i], &t1[i - 1], &p2);
    for (int i = 0; i < 8; i++) { t2[i] = t1[i]; ofp_mul(&t2[i].x, &t1[i].x, &BETA); }
    int len = l1 > l2 ? l1 : l2;
    op1 acc;
    memset(&acc, 0, sizeof(acc));
    for (int i = len - 1; i >= 0; i--) {
        op1_double(&acc, &acc);
        int a = i < l1 ? d1[i] : 0, b = i < l2 ? d2[i] : 0;
        if (a > 0) op1_dadd(&acc, &acc, &t1[(a - 1) / 2]);
        else if (a < 0) { op1 t; op1_neg(&t, &t1[(-a - 1) / 2]); op1_dadd(&acc, &acc, &t); }
        if (b > 0) op1_dadd(&acc, &acc, &t2[(b - 1) / 2]);
        else if (b < 0) { op1 t; op1_neg(&t, &t2[(-b - 1) / 2]); op1_dadd(&acc, &acc, &t); }
    }
    *o = acc;
}

void op1_mult_vartime(op1 *o, const op1 *p, const uint8_t *scalar, size_t nbits)
{
    if (nbits == 0 || op1_is_inf(p)) { memset(o, 0, sizeof(*o)); return; }
    uint64_t k[4];
    canonical_scalar(k, scalar, nbits);
    if (nbits < 176) plain_mult(o, p, k, 4);
    else glv_mult(o, p, k);
}
