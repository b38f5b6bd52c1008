// Host-side G1 arithmetic for the short serial epilogues of the device
// pipelines: folding the per-window MSM sums (c*(D-1) doublings and D adds,
// a strictly sequential chain of ~2-3k field multiplications that one CPU core
// finishes ~10x faster than one GPU thread) and normalising the single MSM
// result to affine.  6 x 64-bit Montgomery limbs (same bytes as blst_fp).
// Device values arrive lazily reduced in [0, 2p) and are canonicalised first.
#pragma once
#include <cstdint>
#include <cstring>

namespace catmsm_host {

typedef unsigned __int128 u128;

struct hfp { uint64_t l[6]; };
struct hjac { hfp x, y, z; };

static const uint64_t HP[6] = {0xb9feffffffffaaabULL, 0x1eabfffeb153ffffULL, 0x6730d2a0f6b0f624ULL,
                               0x64774b84f38512bfULL, 0x4b1ba7b6434bacd7ULL, 0x1a0111ea397fe69aULL};
static const uint64_t HONE[6] = {0x760900000002fffdULL, 0xebf4000bc40c0002ULL, 0x5f48985753c758baULL,
                                 0x77ce585370525745ULL, 0x5c071a97a256ec6dULL, 0x15f65ec3fa80e493ULL};
static const uint64_t HN0 = 0x89f3fffcfffcfffdULL;

inline bool geq(const uint64_t* a, const uint64_t* b)
{
    for (int i = 5; i >= 0; i--)
        if (a[i] != b[i]) return a[i] > b[i];
    return true;
}

inline void sub_p(uint64_t* a)
{
    uint64_t br = 0;
    for (int i = 0; i < 6; i++) {
        u128 d = (u128)a[i] - HP[i] - br;
        a[i] = (uint64_t)d;
        br = (uint64_t)(d >> 64) & 1;
    }
}

inline void canon(hfp& a)
{
    while (geq(a.l, HP)) sub_p(a.l);
}

inline bool is_zero(const hfp& a)
{
    uint64_t z = 0;
    for (int i = 0; i < 6; i++) z |= a.l[i];
    return z == 0;
}

// o = a b R^-1 mod p for canonical a, b (CIOS, the multiplication and the
// reduction of each word of b in one pass).  With a, b < p the running value
// t stays below 2p < 2^382, so the carry chains of the products (A) and of
// the reduction (C) meet in t[5] without overflow and no carry words beyond
// six are needed.  Measured on the Grace host: 43 ns against 51 for separate
// multiply and reduce passes, and 41 ns as the squaring against 51 for a
// dedicated squaring (the halved cross products do not pay at 6 words).
inline void mul(hfp& o, const hfp& a, const hfp& b)
{
    uint64_t t[6] = {0, 0, 0, 0, 0, 0};
#pragma GCC unroll 6
    for (int i = 0; i < 6; i++) {
        const uint64_t bi = b.l[i];
        u128 c = (u128)a.l[0] * bi + t[0];
        uint64_t A = (uint64_t)(c >> 64);
        const uint64_t t0 = (uint64_t)c;
        const uint64_t m = t0 * HN0;
        uint64_t C = (uint64_t)(((u128)m * HP[0] + t0) >> 64);
#pragma GCC unroll 5
        for (int j = 1; j < 6; j++) {
            c = (u128)a.l[j] * bi + t[j] + A;
            A = (uint64_t)(c >> 64);
            const u128 d = (u128)m * HP[j] + (uint64_t)c + C;
            t[j - 1] = (uint64_t)d;
            C = (uint64_t)(d >> 64);
        }
        t[5] = C + A;
    }
    if (geq(t, HP)) sub_p(t);
    std::memcpy(o.l, t, 48);
}

inline void add(hfp& o, const hfp& a, const hfp& b)
{
    uint64_t t[6];
    uint64_t c = 0;
    for (int i = 0; i < 6; i++) {
        u128 s = (u128)a.l[i] + b.l[i] + c;
        t[i] = (uint64_t)s;
        c = (uint64_t)(s >> 64);
    }
    if (c || geq(t, HP)) sub_p(t);
    std::memcpy(o.l, t, 48);
}

inline void sub(hfp& o, const hfp& a, const hfp& b)
{
    uint64_t t[6];
    uint64_t br = 0;
    for (int i = 0; i < 6; i++) {
        u128 d = (u128)a.l[i] - b.l[i] - br;
        t[i] = (uint64_t)d;
        br = (uint64_t)(d >> 64) & 1;
    }
    if (br) {
        uint64_t c = 0;
        for (int i = 0; i < 6; i++) {
            u128 s = (u128)t[i] + HP[i] + c;
            t[i] = (uint64_t)s;
            c = (uint64_t)(s >> 64);
        }
    }
    std::memcpy(o.l, t, 48);
}

// o = a^2 (Montgomery), canonical a.
inline void sqr(hfp& o, const hfp& a) { mul(o, a, a); }

// R^3 mod p (R = 2^384): a Montgomery multiplication by it maps U^-1 to U^-1 R^2.
static const uint64_t HR3[6] = {0xed48ac6bd94ca1e0ULL, 0x315f831e03a7adf8ULL, 0x9a53352a615e29ddULL,
                                0x34c04e5e921e1761ULL, 0x2512d43565724728ULL, 0x0aa6346091755d4dULL};

inline void limbs6_shr(uint64_t* x, unsigned t)
{
    while (t >= 64) {
        for (int i = 0; i < 5; i++) x[i] = x[i + 1];
        x[5] = 0;
        t -= 64;
    }
    if (t) {
        for (int i = 0; i < 5; i++) x[i] = (x[i] >> t) | (x[i + 1] << (64 - t));
        x[5] >>= t;
    }
}

inline void limbs6_shl(uint64_t* x, unsigned t)
{
    while (t >= 64) {
        for (int i = 5; i > 0; i--) x[i] = x[i - 1];
        x[0] = 0;
        t -= 64;
    }
    if (t) {
        for (int i = 5; i > 0; i--) x[i] = (x[i] << t) | (x[i - 1] >> (64 - t));
        x[0] <<= t;
    }
}

inline uint64_t limbs6_sub(uint64_t* d, const uint64_t* a, const uint64_t* b)
{
    uint64_t br = 0;
    for (int i = 0; i < 6; i++) {
        const u128 x = (u128)a[i] - b[i] - br;
        d[i] = (uint64_t)x;
        br = (uint64_t)(x >> 64) & 1;
    }
    return br;
}

inline void limbs6_add(uint64_t* d, const uint64_t* a, const uint64_t* b)
{
    uint64_t c = 0;
    for (int i = 0; i < 6; i++) {
        const u128 x = (u128)a[i] + b[i] + c;
        d[i] = (uint64_t)x;
        c = (uint64_t)(x >> 64);
    }
}

inline unsigned ctz6(const uint64_t* x)
{
    unsigned t = 0;
    for (int i = 0; i < 6; i++) {
        if (x[i]) return t + (unsigned)__builtin_ctzll(x[i]);
        t += 64;
    }
    return t;
}

// o = a^-1 in Montgomery form (zero maps to zero), variable time: Kaliski's
// almost Montgomery inverse (phase 1, every run of trailing zeros in one step)
// on the Montgomery representation U of a gives X = U^-1 2^k; X 2^-k comes
// from k / 64 word-wise Montgomery reductions and k % 64 halvings mod p, and
// one multiplication by R^3 gives U^-1 R^2 = a^-1 R.  ~270 subtract-and-shift
// steps against ~570 multiplications for a^(p-2).
inline void inv(hfp& o, const hfp& a)
{
    hfp c = a;
    canon(c);
    if (is_zero(c)) {
        std::memset(o.l, 0, 48);
        return;
    }
    uint64_t u[6], v[6], r[6] = {0}, s[6] = {1, 0, 0, 0, 0, 0}, d[6];
    std::memcpy(u, HP, 48);
    std::memcpy(v, c.l, 48);
    unsigned k = ctz6(v);
    limbs6_shr(v, k);
    for (int iter = 0; iter < 2048; iter++) {     // at most ~390 for 381-bit inputs
        if (limbs6_sub(d, u, v) == 0) {
            uint64_t z = 0;
            for (int i = 0; i < 6; i++) z |= d[i];
            if (z == 0) {                          // u == v == 1
                limbs6_add(s, r, s);
                limbs6_shl(r, 1);
                k += 1;
                break;
            }
            const unsigned t = ctz6(d);            // u > v: u = (u - v) >> t, r += s, s <<= t
            limbs6_shr(d, t);
            std::memcpy(u, d, 48);
            limbs6_add(r, r, s);
            limbs6_shl(s, t);
            k += t;
        } else {
            limbs6_sub(d, v, u);                   // u < v: v = (v - u) >> t, s += r, r <<= t
            const unsigned t = ctz6(d);
            limbs6_shr(d, t);
            std::memcpy(v, d, 48);
            limbs6_add(s, r, s);
            limbs6_shl(r, t);
            k += t;
        }
    }
    if (geq(r, HP)) sub_p(r);                      // r in (0, 2p): X = p - r
    hfp X;
    limbs6_sub(X.l, HP, r);
    // X 2^-k: whole words by Montgomery reduction steps, the rest by halvings
    for (; k >= 64; k -= 64) {
        const uint64_t m = X.l[0] * HN0;
        u128 acc = ((u128)m * HP[0] + X.l[0]) >> 64;
        for (int j = 1; j < 6; j++) {
            acc += (u128)m * HP[j] + X.l[j];
            X.l[j - 1] = (uint64_t)acc;
            acc >>= 64;
        }
        X.l[5] = (uint64_t)acc;                   // X + m p < 2^448: the quotient fits 6 words, < 2p
        if (geq(X.l, HP)) sub_p(X.l);
    }
    for (; k > 0; k--) {
        uint64_t top = 0;
        if (X.l[0] & 1) {
            uint64_t cy = 0;
            for (int i = 0; i < 6; i++) {
                const u128 x = (u128)X.l[i] + HP[i] + cy;
                X.l[i] = (uint64_t)x;
                cy = (uint64_t)(x >> 64);
            }
            top = cy;
        }
        for (int i = 0; i < 5; i++) X.l[i] = (X.l[i] >> 1) | (X.l[i + 1] << 63);
        X.l[5] = (X.l[5] >> 1) | (top << 63);
    }
    hfp r3;
    std::memcpy(r3.l, HR3, 48);
    mul(o, X, r3);
}

inline bool jac_is_inf(const hjac& p) { return is_zero(p.z); }

// dbl-2009-l (a = 0)
inline void jac_dbl(hjac& o, const hjac& p)
{
    if (jac_is_inf(p)) { o = p; return; }
    hfp A, B, C, D, E, F, t, X3, Y3, Z3;
    sqr(A, p.x);
    sqr(B, p.y);
    sqr(C, B);
    add(t, p.x, B);
    sqr(t, t);
    sub(t, t, A);
    sub(t, t, C);
    add(D, t, t);
    add(E, A, A);
    add(E, E, A);
    sqr(F, E);
    mul(Z3, p.y, p.z);
    add(Z3, Z3, Z3);
    sub(X3, F, D);
    sub(X3, X3, D);
    sub(t, D, X3);
    mul(Y3, E, t);
    add(C, C, C);
    add(C, C, C);
    add(C, C, C);
    sub(Y3, Y3, C);
    o.x = X3; o.y = Y3; o.z = Z3;
}

inline void jac_add(hjac& o, const hjac& a, const hjac& b)
{
    if (jac_is_inf(a)) { o = b; return; }
    if (jac_is_inf(b)) { o = a; return; }
    hfp z1z1, z2z2, u1, u2, s1, s2, h, r, t;
    sqr(z1z1, a.z);
    sqr(z2z2, b.z);
    mul(u1, a.x, z2z2);
    mul(u2, b.x, z1z1);
    mul(s1, a.y, b.z);
    mul(s1, s1, z2z2);
    mul(s2, b.y, a.z);
    mul(s2, s2, z1z1);
    sub(h, u2, u1);
    sub(r, s2, s1);
    if (is_zero(h)) {
        if (is_zero(r)) { jac_dbl(o, a); return; }
        std::memset(&o, 0, sizeof(o));
        return;
    }
    hfp hh, hhh, v, X3, Y3, Z3;
    sqr(hh, h);
    mul(hhh, hh, h);
    mul(v, u1, hh);
    sqr(X3, r);
    sub(X3, X3, hhh);
    sub(X3, X3, v);
    sub(X3, X3, v);
    sub(t, v, X3);
    mul(Y3, r, t);
    mul(t, s1, hhh);
    sub(Y3, Y3, t);
    mul(Z3, a.z, b.z);
    mul(Z3, Z3, h);
    o.x = X3; o.y = Y3; o.z = Z3;
}

// xyzz image from the device (x, y, zz, zzz; lazily reduced) -> Jacobian
inline void from_device_xyzz(hjac& o, const uint64_t* w /* 24 limbs */)
{
    hfp x, y, zz, zzz;
    std::memcpy(x.l, w, 48);
    std::memcpy(y.l, w + 6, 48);
    std::memcpy(zz.l, w + 12, 48);
    std::memcpy(zzz.l, w + 18, 48);
    canon(x); canon(y); canon(zz); canon(zzz);
    if (is_zero(zz)) { std::memset(&o, 0, sizeof(o)); return; }
    mul(o.x, x, zz);
    mul(o.y, y, zzz);
    o.z = zz;
}

// Normalise to Z = 1 (Montgomery one) so the Jacobian output bytes are the
// affine coordinates; infinity is written as all-zero.
inline void normalize(hjac& o, const hjac& p)
{
    if (jac_is_inf(p)) { std::memset(&o, 0, sizeof(o)); return; }
    hfp zi, zi2, zi3;
    inv(zi, p.z);
    sqr(zi2, zi);
    mul(zi3, zi2, zi);
    mul(o.x, p.x, zi2);
    mul(o.y, p.y, zi3);
    std::memcpy(o.z.l, HONE, 48);
}

}  // namespace catmsm_host
