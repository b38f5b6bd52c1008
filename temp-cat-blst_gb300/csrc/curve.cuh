// G1 point arithmetic on sm_103a (y^2 = x^3 + 4 over Fp).
//
// Representations:
//   affine  {x, y}            96 B, all-zero = infinity (blst_p1_affine,
//                             bindings/blst_types.h:101)
//   jacobian{x, y, z}         144 B, z == 0 = infinity (blst_p1, :99)
//   xyzz    {x, y, zz, zzz}   x = X/ZZ, y = Y/ZZZ, ZZ^3 = ZZZ^2; zz == 0 =
//                             infinity.  Same coordinates the reference uses
//                             for its Pippenger buckets (scalar/curve/point.cpp
//                             :1939-2113).
// Formulas are the public explicit-formulas-database ones for a = 0:
//   xyzz madd-2008-s / mdbl-2008-s / add-2008-s / dbl-2008-s,
//   jacobian dbl-2009-l and add-2007-bl (with explicit special cases).
// Every addition handles infinity, doubling and opposite inputs, so the group
// law is complete and results are exact for any points on the curve.
#pragma once
#include "field.cuh"

namespace catmsm {

struct affine { fp x, y; };
struct jac { fp x, y, z; };
struct xyzz { fp x, y, zz, zzz; };

// Vectorised global loads and stores of points (16-byte aligned rows).
__device__ __forceinline__ void load_affine(fp& x, fp& y, const affine* p)
{
    const uint4* q = reinterpret_cast<const uint4*>(p);
    uint4 v[6];
#pragma unroll
    for (int k = 0; k < 6; k++) v[k] = __ldg(q + k);
#pragma unroll
    for (int k = 0; k < 3; k++) {
        x.v[4 * k + 0] = v[k].x; x.v[4 * k + 1] = v[k].y;
        x.v[4 * k + 2] = v[k].z; x.v[4 * k + 3] = v[k].w;
        y.v[4 * k + 0] = v[k + 3].x; y.v[4 * k + 1] = v[k + 3].y;
        y.v[4 * k + 2] = v[k + 3].z; y.v[4 * k + 3] = v[k + 3].w;
    }
}

__device__ __forceinline__ void store_xyzz(xyzz* dst, const xyzz& p)
{
    uint4* q = reinterpret_cast<uint4*>(dst);
    const uint32_t* s = reinterpret_cast<const uint32_t*>(&p);
#pragma unroll
    for (int k = 0; k < 12; k++) q[k] = make_uint4(s[4 * k], s[4 * k + 1], s[4 * k + 2], s[4 * k + 3]);
}

__device__ __forceinline__ void store_affine(affine* dst, const affine& p)
{
    uint4* q = reinterpret_cast<uint4*>(dst);
    const uint32_t* s = reinterpret_cast<const uint32_t*>(&p);
#pragma unroll
    for (int k = 0; k < 6; k++) q[k] = make_uint4(s[4 * k], s[4 * k + 1], s[4 * k + 2], s[4 * k + 3]);
}

__device__ __forceinline__ void load_xyzz(xyzz& p, const xyzz* src)
{
    const uint4* q = reinterpret_cast<const uint4*>(src);
    uint32_t* d = reinterpret_cast<uint32_t*>(&p);
#pragma unroll
    for (int k = 0; k < 12; k++) {
        uint4 v = q[k];
        d[4 * k] = v.x; d[4 * k + 1] = v.y; d[4 * k + 2] = v.z; d[4 * k + 3] = v.w;
    }
}

__device__ __forceinline__ bool aff_is_inf(const affine& a)
{
    return fp_is_zero_raw(a.x) && fp_is_zero_raw(a.y);
}

__device__ __forceinline__ void xyzz_set_inf(xyzz& p)
{
    fp_zero(p.x); fp_zero(p.y); fp_zero(p.zz); fp_zero(p.zzz);
}

__device__ __forceinline__ bool xyzz_is_inf(const xyzz& p) { return fp_is_zero(p.zz); }

// p = 2 * (ax, ay) for an affine point (mdbl-2008-s)
__device__ __forceinline__ void xyzz_dbl_affine(xyzz& p, const fp& ax, const fp& ay)
{
    fp U, V, W, S, M, t;
    fp_dbl(U, ay);
    fp_sqr(V, U);
    fp_mul(W, V, U);
    fp_mul(S, ax, V);
    fp_sqr(M, ax);
    fp_dbl(t, M);
    fp_add(M, t, M);
    fp_sqr(t, M);
    fp_sub(t, t, S);
    fp_sub(p.x, t, S);
    fp_sub(t, S, p.x);
    fp_neg(S, ay);
    fp_mul2(p.y, M, t, W, S);     // Y3 = M (S - X3) - W y, one reduction
    p.zz = V;
    p.zzz = W;
}

// p += (ax, +/-ay)   (madd-2008-s, 8M + 2S); ay already carries the sign
__device__ __forceinline__ void xyzz_madd(xyzz& p, const fp& ax, const fp& ay)
{
    if (xyzz_is_inf(p)) {
        p.x = ax; p.y = ay;
        fp_set_one(p.zz); fp_set_one(p.zzz);
        return;
    }
    fp P, R;
    fp_mul(P, ax, p.zz);
    fp_sub(P, P, p.x);
    fp_mul(R, ay, p.zzz);
    fp_sub(R, R, p.y);
    if (fp_is_zero(P)) {
        if (fp_is_zero(R)) xyzz_dbl_affine(p, ax, ay);
        else xyzz_set_inf(p);
        return;
    }
    fp PP, PPP, Q;
    fp_sqr(PP, P);
    fp_mul(PPP, PP, P);
    fp_mul(p.zz, p.zz, PP);
    fp_mul(p.zzz, p.zzz, PPP);
    fp_mul(Q, p.x, PP);
    fp_sqr(P, R);                 // P := R^2
    fp_sub(P, P, PPP);
    fp_sub(P, P, Q);
    fp_sub(p.x, P, Q);            // X3 = R^2 - PPP - 2Q
    fp_sub(Q, Q, p.x);
    fp_neg(PPP, PPP);
    fp_mul2(p.y, Q, R, p.y, PPP); // Y3 = R (Q - X3) - Y1 PPP, one reduction
}

// p = 2p (dbl-2008-s)
__device__ __forceinline__ void xyzz_dbl(xyzz& p)
{
    if (xyzz_is_inf(p)) return;
    fp U, V, W, S, M, t;
    fp_dbl(U, p.y);
    fp_sqr(V, U);
    fp_mul(W, V, U);
    fp_mul(S, p.x, V);
    fp_sqr(M, p.x);
    fp_dbl(t, M);
    fp_add(M, t, M);
    fp_mul(p.zz, p.zz, V);
    fp_mul(p.zzz, p.zzz, W);
    fp_sqr(t, M);
    fp_sub(t, t, S);
    fp_sub(p.x, t, S);
    fp_sub(t, S, p.x);
    fp_neg(W, W);
    fp_mul2(p.y, M, t, W, p.y);   // Y3 = M (S - X3) - W Y1, one reduction
}

// p += q (add-2008-s, 12M + 2S)
__device__ __forceinline__ void xyzz_add(xyzz& p, const xyzz& q)
{
    if (xyzz_is_inf(q)) return;
    if (xyzz_is_inf(p)) { p = q; return; }
    fp U1, S1, P, R;
    fp_mul(U1, p.x, q.zz);
    fp_mul(P, q.x, p.zz);
    fp_sub(P, P, U1);
    fp_mul(S1, p.y, q.zzz);
    fp_mul(R, q.y, p.zzz);
    fp_sub(R, R, S1);
    if (fp_is_zero(P)) {
        if (fp_is_zero(R)) xyzz_dbl(p);
        else xyzz_set_inf(p);
        return;
    }
    fp PP, PPP;
    fp_sqr(PP, P);
    fp_mul(PPP, PP, P);
    fp_mul(p.zz, p.zz, q.zz);
    fp_mul(p.zz, p.zz, PP);
    fp_mul(p.zzz, p.zzz, q.zzz);
    fp_mul(p.zzz, p.zzz, PPP);
    fp_mul(U1, U1, PP);           // Q = U1 PP
    fp_sqr(P, R);
    fp_sub(P, P, PPP);
    fp_sub(P, P, U1);
    fp_sub(p.x, P, U1);
    fp_sub(U1, U1, p.x);
    fp_neg(PPP, PPP);
    fp_mul2(p.y, U1, R, S1, PPP); // Y3 = R (Q - X3) - S1 PPP, one reduction
}

__device__ __forceinline__ void xyzz_neg(xyzz& p) { fp_neg(p.y, p.y); }

// Jacobian (X, Y, Z) = (x*zz, y*zzz, zz); reference point.cpp:2109
__device__ __forceinline__ void xyzz_to_jac(jac& o, const xyzz& p)
{
    if (xyzz_is_inf(p)) {
        fp_zero(o.x); fp_zero(o.y); fp_zero(o.z);
        return;
    }
    fp_mul(o.x, p.x, p.zz);
    fp_mul(o.y, p.y, p.zzz);
    o.z = p.zz;
}

// xyzz from Jacobian: zz = Z^2, zzz = Z^3
__device__ __forceinline__ void jac_to_xyzz(xyzz& o, const jac& p)
{
    if (fp_is_zero(p.z)) { xyzz_set_inf(o); return; }
    o.x = p.x;
    o.y = p.y;
    fp_sqr(o.zz, p.z);
    fp_mul(o.zzz, o.zz, p.z);
}

// Affine normalisation of an xyzz point: x = X / ZZ, y = Y / ZZZ.
// 1/ZZ and 1/ZZZ come from one inversion of ZZZ*ZZ... via (ZZ*ZZZ)^-1.
__device__ __forceinline__ void xyzz_to_affine(affine& o, const xyzz& p)
{
    if (xyzz_is_inf(p)) { fp_zero(o.x); fp_zero(o.y); return; }
    fp t, inv;
    fp_mul(t, p.zz, p.zzz);
    fp_inv(inv, t);
    fp_mul(t, inv, p.zzz);        // 1/ZZ
    fp_mul(o.x, p.x, t);
    fp_mul(t, inv, p.zz);         // 1/ZZZ
    fp_mul(o.y, p.y, t);
    fp_canon(o.x, o.x);
    fp_canon(o.y, o.y);
}


// ---------------------------------------------------------------- Jacobian
__device__ __forceinline__ bool jac_is_inf(const jac& p) { return fp_is_zero(p.z); }

__device__ __forceinline__ void jac_set_inf(jac& p) { fp_zero(p.x); fp_zero(p.y); fp_zero(p.z); }

// dbl-2009-l (a = 0): 2M + 5S
__device__ __forceinline__ void jac_dbl(jac& p)
{
    if (jac_is_inf(p)) return;
    fp A, B, C, D, E, t;
    fp_sqr(A, p.x);
    fp_sqr(B, p.y);
    fp_sqr(C, B);
    fp_add(t, p.x, B);
    fp_sqr(t, t);
    fp_sub(t, t, A);
    fp_sub(t, t, C);
    fp_dbl(D, t);
    fp_dbl(E, A);
    fp_add(E, E, A);
    fp_mul(p.z, p.y, p.z);
    fp_dbl(p.z, p.z);
    fp_sqr(t, E);
    fp_sub(t, t, D);
    fp_sub(p.x, t, D);
    fp_sub(t, D, p.x);
    fp_mul(t, E, t);
    fp_dbl(C, C);
    fp_dbl(C, C);
    fp_dbl(C, C);
    fp_sub(p.y, t, C);
}

// p += q, add-2007-bl style with explicit infinity / doubling / opposite cases
__device__ __forceinline__ void jac_add(jac& p, const jac& q)
{
    if (jac_is_inf(q)) return;
    if (jac_is_inf(p)) { p = q; return; }
    fp z1z1, z2z2, u1, h, s1, r, t;
    fp_sqr(z1z1, p.z);
    fp_sqr(z2z2, q.z);
    fp_mul(u1, p.x, z2z2);
    fp_mul(h, q.x, z1z1);
    fp_sub(h, h, u1);
    fp_mul(s1, p.y, q.z);
    fp_mul(s1, s1, z2z2);
    fp_mul(r, q.y, p.z);
    fp_mul(r, r, z1z1);
    fp_sub(r, r, s1);
    if (fp_is_zero(h)) {
        if (fp_is_zero(r)) jac_dbl(p);
        else jac_set_inf(p);
        return;
    }
    fp_mul(p.z, p.z, q.z);
    fp_mul(p.z, p.z, h);
    fp_sqr(t, h);                 // HH
    fp_mul(u1, u1, t);            // V = U1 HH
    fp_mul(t, t, h);              // HHH
    fp_sqr(z1z1, r);
    fp_sub(z1z1, z1z1, t);
    fp_sub(z1z1, z1z1, u1);
    fp_sub(p.x, z1z1, u1);        // X3 = R^2 - HHH - 2V
    fp_sub(u1, u1, p.x);
    fp_neg(t, t);
    fp_mul2(p.y, u1, r, s1, t);   // Y3 = R (V - X3) - S1 HHH, one reduction
}

__device__ __forceinline__ void jac_neg(jac& p) { fp_neg(p.y, p.y); }

// GLV endomorphism of G1: phi(x, y) = (beta x, y) = lambda (x, y) for
// lambda = z^2 - 1 = 0xac45a4010001a40200000000ffffffff (lambda^2 + lambda + 1 = r)
// and the cube root of unity beta below (Montgomery form).
__device__ __constant__ static const uint32_t FP_BETA[12] = {
    0x8671f071u, 0xcd03c9e4u, 0x1fcda5d2u, 0x5dab2246u, 0xd3851b95u, 0x587042afu,
    0x01bacb9eu, 0x8eb60ebeu, 0x83d050d2u, 0x03f97d6eu, 0x54638741u, 0x18f02065u};

// Signed fixed-window digits of a value below 2^128 (4 little-endian words):
// 26 digits d_i in [-15, 16] with value = sum_i d_i 32^i (window recoding
// with carry, as the MSM's digit recoding).  Every value uses the same 26
// windows, so lanes of a warp working on different scalars add at the same
// positions.  5-bit windows against 4-bit: 125 doublings and ~50 additions
// instead of 128 and ~62, for a 16-entry table (7% faster FFTs measured).
__device__ __forceinline__ void booth5_128(int8_t* d, const uint32_t* k)
{
    uint32_t carry = 0;
#pragma unroll
    for (int i = 0; i < 26; i++) {
        const uint32_t bit = 5 * i, word = bit >> 5, sh = bit & 31;
        uint32_t raw = word < 4 ? k[word] >> sh : 0u;
        if (sh > 27 && word + 1 < 4) raw |= k[word + 1] << (32 - sh);
        raw &= 31u;
        int v = (int)(raw + carry);
        if (v > 16) { v -= 32; carry = 1; }
        else carry = 0;
        d[i] = (int8_t)v;
    }
}
static __device__ __noinline__ void jac_mult_glv(jac& out, const jac& P, const uint32_t* k1, const uint32_t* k2)
{
    int8_t d1[26], d2[26];
    booth5_128(d1, k1);
    booth5_128(d2, k2);
    jac T[16];                                   // T[i] = (i + 1) P
    T[0] = P;
    T[1] = P; jac_dbl(T[1]);
#pragma unroll 1
    for (int i = 2; i < 16; i++) {
        if (i & 1) { T[i] = T[i / 2]; jac_dbl(T[i]); }         // (i+1) even: 2 ((i+1)/2) P
        else { T[i] = T[i - 1]; jac_add(T[i], P); }
    }
    fp beta;
#pragma unroll
    for (int i = 0; i < 12; i++) beta.v[i] = FP_BETA[i];
    jac acc;
    jac_set_inf(acc);
    for (int i = 25; i >= 0; i--) {
        if (i < 25) {
            jac_dbl(acc); jac_dbl(acc); jac_dbl(acc); jac_dbl(acc); jac_dbl(acc);
        }
        const int a = d1[i], b = d2[i];
        if (a) {
            jac t = T[(a > 0 ? a : -a) - 1];
            if (a < 0) jac_neg(t);
            jac_add(acc, t);
        }
        if (b) {
            jac t = T[(b > 0 ? b : -b) - 1];
            fp_mul(t.x, t.x, beta);
            if (b < 0) jac_neg(t);
            jac_add(acc, t);
        }
    }
    out = acc;
}

// Width-5 NAF of a value below 2^128 (4 little-endian words): digits d_i in
// {0, +-1, +-3, ..., +-15} with value = sum_i d_i 2^i and at most one nonzero
// digit in any five consecutive positions (density ~1/6).  Returns the number
// of digits, at most 129: subtracting a negative digit can carry the value
// past 2^128 once, after which every step halves it.
__device__ __forceinline__ int wnaf5_128(int8_t* d, const uint32_t* k)
{
    uint32_t w0 = k[0], w1 = k[1], w2 = k[2], w3 = k[3], w4 = 0;
    int len = 0;
#pragma unroll 1
    for (int i = 0; i < 130 && (w0 | w1 | w2 | w3 | w4); i++) {
        int v = 0;
        if (w0 & 1u) {
            v = (int)(w0 & 31u);
            if (v > 16) v -= 32;
            if (v > 0) {
                w0 -= (uint32_t)v;                   // the low five bits are v: no borrow
            } else {
                uint64_t s = (uint64_t)w0 + (uint32_t)(-v);
                w0 = (uint32_t)s;
                s = (s >> 32) + w1; w1 = (uint32_t)s;
                s = (s >> 32) + w2; w2 = (uint32_t)s;
                s = (s >> 32) + w3; w3 = (uint32_t)s;
                w4 += (uint32_t)(s >> 32);
            }
        }
        d[i] = (int8_t)v;
        len = i + 1;
        w0 = (w0 >> 1) | (w1 << 31);
        w1 = (w1 >> 1) | (w2 << 31);
        w2 = (w2 >> 1) | (w3 << 31);
        w3 = (w3 >> 1) | (w4 << 31);
        w4 >>= 1;
    }
    return len;
}

// jac_mult_glv for lanes that all multiply by one scalar (k1, k2): each half
// in width-5 NAF over the odd multiples P, 3P, ..., 15P (one doubling and
// seven additions) and phi of them, ~129 doublings and ~50 additions against
// 133 and ~57 for the fixed windows.  The digit positions depend on the
// scalar, so lanes with different scalars would diverge at every addition;
// jac_mult_glv serves those.
static __device__ __noinline__ void jac_mult_glv_shared(jac& out, const jac& P, const uint32_t* k1,
                                                        const uint32_t* k2)
{
    int8_t d1[130], d2[130];
    const int n1 = wnaf5_128(d1, k1), n2 = wnaf5_128(d2, k2);
    jac T[8];                                    // T[i] = (2 i + 1) P
    jac P2 = P;
    jac_dbl(P2);
    T[0] = P;
#pragma unroll 1
    for (int i = 1; i < 8; i++) {
        T[i] = T[i - 1];
        jac_add(T[i], P2);
    }
    fp beta;
#pragma unroll
    for (int i = 0; i < 12; i++) beta.v[i] = FP_BETA[i];
    jac acc;
    jac_set_inf(acc);
    for (int i = max(n1, n2) - 1; i >= 0; i--) {
        jac_dbl(acc);
        const int a = i < n1 ? d1[i] : 0, b = i < n2 ? d2[i] : 0;
        if (a) {
            jac t = T[(a > 0 ? a : -a) >> 1];
            if (a < 0) jac_neg(t);
            jac_add(acc, t);
        }
        if (b) {
            jac t = T[(b > 0 ? b : -b) >> 1];
            fp_mul(t.x, t.x, beta);
            if (b < 0) jac_neg(t);
            jac_add(acc, t);
        }
    }
    out = acc;
}

// ---------------------------------------------------------------------------
// Quad point operations: four consecutive lanes (a quad) hold the same
// operands and perform one XYZZ addition or doubling together.  At each step
// lane k of the quad computes one of the step's independent products (the
// same fp_mul_call on lane-selected operands, so the lanes never diverge) and
// the products are exchanged with width-4 shuffles under the quad's own mask.
// An addition becomes 4 dependent multiplications instead of ~11.5, a
// doubling 3 instead of ~8: for chains of few point operations in few
// threads (the reduction's upper levels, carry joins) latency, not
// multiplier throughput, is what costs.  Every lane ends with the result.
// All control flow below depends only on the quad's shared operands, so the
// four lanes stay converged; callers keep the quad's lanes together.
struct quad_lane {
    uint32_t k;      // position in the quad
    uint32_t mask;   // the quad's four lanes
};

__device__ __forceinline__ quad_lane quad_of(uint32_t lane)
{
    return quad_lane{lane & 3u, 0xfu << (lane & 28u)};
}

__device__ __forceinline__ fp fp_bcast(const fp& v, int src, const quad_lane& q)
{
    fp r;
#pragma unroll
    for (int i = 0; i < 12; i++) r.v[i] = __shfl_sync(q.mask, v.v[i], src, 4);
    return r;
}

// Operand k of four, by masks: a chain of conditional selects on a per-lane
// k measured ~1.7k cycles per pick on sm_103a against ~60 for this form.
__device__ __forceinline__ fp fp_pick(uint32_t k, const fp& a0, const fp& a1, const fp& a2, const fp& a3)
{
    const uint32_t m0 = 0u - (k == 0), m1 = 0u - (k == 1), m2 = 0u - (k == 2), m3 = 0u - (k == 3);
    fp r;
#pragma unroll
    for (int i = 0; i < 12; i++) r.v[i] = (a0.v[i] & m0) | (a1.v[i] & m1) | (a2.v[i] & m2) | (a3.v[i] & m3);
    return r;
}

// dbl-2008-s as xyzz_dbl: V = U^2, M = 3 X^2 | W = U V, S = X V, M^2, ZZ V |
// M (S - X3), W Y, ZZZ W.
__device__ __forceinline__ void xyzz_dbl_quad(xyzz& p, const quad_lane& q)
{
    if (xyzz_is_inf(p)) return;
    fp U, r;
    fp_dbl(U, p.y);
    r = fp_mul_call(fp_pick(q.k, U, p.x, U, p.x), fp_pick(q.k, U, p.x, U, p.x));
    const fp V = fp_bcast(r, 0, q);
    fp M = fp_bcast(r, 1, q), t;
    fp_dbl(t, M);
    fp_add(M, t, M);
    r = fp_mul_call(fp_pick(q.k, V, p.x, M, p.zz), fp_pick(q.k, U, V, M, V));
    const fp W = fp_bcast(r, 0, q), S = fp_bcast(r, 1, q), MM = fp_bcast(r, 2, q);
    p.zz = fp_bcast(r, 3, q);
    fp_sub(t, MM, S);
    fp_sub(p.x, t, S);
    fp_sub(t, S, p.x);
    r = fp_mul_call(fp_pick(q.k, M, W, p.zzz, p.zzz), fp_pick(q.k, t, p.y, W, W));
    const fp a = fp_bcast(r, 0, q), b = fp_bcast(r, 1, q);
    p.zzz = fp_bcast(r, 2, q);
    fp_sub(p.y, a, b);
}

// p += q, add-2008-s as xyzz_add: U1, U2, S1, S2 | P^2, R^2, ZZ1 ZZ2,
// ZZZ1 ZZZ2 | P PP, U1 PP, ZZ1 ZZ2 PP | R (Q - X3), S1 PPP, ZZZ1 ZZZ2 PPP.
__device__ __forceinline__ void xyzz_add_quad(xyzz& p, const xyzz& o, const quad_lane& q)
{
    if (xyzz_is_inf(o)) return;
    if (xyzz_is_inf(p)) {
        p = o;
        return;
    }
    fp r = fp_mul_call(fp_pick(q.k, p.x, o.x, p.y, o.y), fp_pick(q.k, o.zz, p.zz, o.zzz, p.zzz));
    const fp U1 = fp_bcast(r, 0, q), S1 = fp_bcast(r, 2, q);
    fp P = fp_bcast(r, 1, q), R = fp_bcast(r, 3, q);
    fp_sub(P, P, U1);
    fp_sub(R, R, S1);
    if (fp_is_zero(P)) {
        if (fp_is_zero(R)) xyzz_dbl_quad(p, q);
        else xyzz_set_inf(p);
        return;
    }
    r = fp_mul_call(fp_pick(q.k, P, R, p.zz, p.zzz), fp_pick(q.k, P, R, o.zz, o.zzz));
    const fp PP = fp_bcast(r, 0, q), RR = fp_bcast(r, 1, q), T1 = fp_bcast(r, 2, q), T2 = fp_bcast(r, 3, q);
    r = fp_mul_call(fp_pick(q.k, P, U1, T1, T1), PP);
    const fp PPP = fp_bcast(r, 0, q), Qv = fp_bcast(r, 1, q);
    p.zz = fp_bcast(r, 2, q);
    fp t;
    fp_sub(t, RR, PPP);
    fp_sub(t, t, Qv);
    fp_sub(p.x, t, Qv);
    fp_sub(t, Qv, p.x);
    r = fp_mul_call(fp_pick(q.k, R, S1, T2, T2), fp_pick(q.k, t, PPP, PPP, PPP));
    const fp a = fp_bcast(r, 0, q), b = fp_bcast(r, 1, q);
    p.zzz = fp_bcast(r, 2, q);
    fp_sub(p.y, a, b);
}

// dbl-2009-l as jac_dbl: X^2, Y^2, Y Z | B^2, (X + B)^2, E^2 | E (D - X3).
__device__ __forceinline__ void jac_dbl_quad(jac& p, const quad_lane& q)
{
    if (jac_is_inf(p)) return;
    fp r = fp_mul_call(fp_pick(q.k, p.x, p.y, p.y, p.y), fp_pick(q.k, p.x, p.y, p.z, p.z));
    const fp A = fp_bcast(r, 0, q), B = fp_bcast(r, 1, q), YZ = fp_bcast(r, 2, q);
    fp XB, E, t, D;
    fp_add(XB, p.x, B);
    fp_dbl(E, A);
    fp_add(E, E, A);
    r = fp_mul_call(fp_pick(q.k, B, XB, E, E), fp_pick(q.k, B, XB, E, E));
    const fp C = fp_bcast(r, 0, q), T = fp_bcast(r, 1, q), F = fp_bcast(r, 2, q);
    fp_sub(t, T, A);
    fp_sub(t, t, C);
    fp_dbl(D, t);
    fp_sub(t, F, D);
    fp_sub(p.x, t, D);
    fp_sub(t, D, p.x);
    fp_dbl(p.z, YZ);
    r = fp_mul_call(E, t);                      // the same product on every lane
    fp C8;
    fp_dbl(C8, C);
    fp_dbl(C8, C8);
    fp_dbl(C8, C8);
    fp_sub(p.y, r, C8);
}

// p += o as jac_add: Z1^2, Z2^2, Y1 Z2, Y2 Z1 | U1, U2, S1, S2 | H^2, R^2,
// Z1 Z2 | U1 HH, H HH, Z1 Z2 H | R (V - X3), S1 HHH.
__device__ __forceinline__ void jac_add_quad(jac& p, const jac& o, const quad_lane& q)
{
    if (jac_is_inf(o)) return;
    if (jac_is_inf(p)) {
        p = o;
        return;
    }
    fp r = fp_mul_call(fp_pick(q.k, p.z, o.z, p.y, o.y), fp_pick(q.k, p.z, o.z, o.z, p.z));
    const fp z1z1 = fp_bcast(r, 0, q), z2z2 = fp_bcast(r, 1, q), s1a = fp_bcast(r, 2, q), ra = fp_bcast(r, 3, q);
    r = fp_mul_call(fp_pick(q.k, p.x, o.x, s1a, ra), fp_pick(q.k, z2z2, z1z1, z2z2, z1z1));
    const fp u1 = fp_bcast(r, 0, q), s1 = fp_bcast(r, 2, q);
    fp h = fp_bcast(r, 1, q), R = fp_bcast(r, 3, q);
    fp_sub(h, h, u1);
    fp_sub(R, R, s1);
    if (fp_is_zero(h)) {
        if (fp_is_zero(R)) jac_dbl_quad(p, q);
        else jac_set_inf(p);
        return;
    }
    r = fp_mul_call(fp_pick(q.k, h, R, p.z, p.z), fp_pick(q.k, h, R, o.z, o.z));
    const fp HH = fp_bcast(r, 0, q), RR = fp_bcast(r, 1, q), Z12 = fp_bcast(r, 2, q);
    r = fp_mul_call(fp_pick(q.k, u1, h, Z12, Z12), fp_pick(q.k, HH, HH, h, h));
    const fp V = fp_bcast(r, 0, q), HHH = fp_bcast(r, 1, q);
    p.z = fp_bcast(r, 2, q);
    fp t;
    fp_sub(t, RR, HHH);
    fp_sub(t, t, V);
    fp_sub(p.x, t, V);
    fp_sub(t, V, p.x);
    r = fp_mul_call(fp_pick(q.k, R, s1, s1, s1), fp_pick(q.k, t, HHH, HHH, HHH));
    const fp a = fp_bcast(r, 0, q), b = fp_bcast(r, 1, q);
    fp_sub(p.y, a, b);
}

// jac_mult_glv with quad operations: every lane of the quad passes the same
// point and scalar and ends with the product.
static __device__ __noinline__ void jac_mult_glv_quad(jac& out, const jac& P, const uint32_t* k1, const uint32_t* k2,
                                                      const quad_lane q)
{
    int8_t d1[26], d2[26];
    booth5_128(d1, k1);
    booth5_128(d2, k2);
    jac T[16];                                   // T[i] = (i + 1) P
    T[0] = P;
    T[1] = P;
    jac_dbl_quad(T[1], q);
#pragma unroll 1
    for (int i = 2; i < 16; i++) {
        if (i & 1) { T[i] = T[i / 2]; jac_dbl_quad(T[i], q); }
        else { T[i] = T[i - 1]; jac_add_quad(T[i], P, q); }
    }
    fp beta;
#pragma unroll
    for (int i = 0; i < 12; i++) beta.v[i] = FP_BETA[i];
    jac acc;
    jac_set_inf(acc);
    for (int i = 25; i >= 0; i--) {
        if (i < 25)
            for (int k = 0; k < 5; k++) jac_dbl_quad(acc, q);
        const int a = d1[i], b = d2[i];
        if (a) {
            jac t = T[(a > 0 ? a : -a) - 1];
            if (a < 0) jac_neg(t);
            jac_add_quad(acc, t, q);
        }
        if (b) {
            jac t = T[(b > 0 ? b : -b) - 1];
            fp_mul(t.x, t.x, beta);
            if (b < 0) jac_neg(t);
            jac_add_quad(acc, t, q);
        }
    }
    out = acc;
}

}  // namespace catmsm
