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

inline void mul(hfp& o, const hfp& a, const hfp& b)
{
    uint64_t t[8] = {0};
    for (int i = 0; i < 6; i++) {
        u128 c = 0;
        for (int j = 0; j < 6; j++) {
            c += (u128)a.l[j] * b.l[i] + t[j];
            t[j] = (uint64_t)c;
            c >>= 64;
        }
        c += t[6];
        t[6] = (uint64_t)c;
        t[7] = (uint64_t)(c >> 64);
        uint64_t m = t[0] * HN0;
        c = ((u128)m * HP[0] + t[0]) >> 64;
        for (int j = 1; j < 6; j++) {
            c += (u128)m * HP[j] + t[j];
            t[j - 1] = (uint64_t)c;
            c >>= 64;
        }
        c += t[6];
        t[5] = (uint64_t)c;
        t[6] = t[7] + (uint64_t)(c >> 64);
    }
    if (t[6] || geq(t, HP)) sub_p(t);
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

inline void inv(hfp& o, const hfp& a)
{
    uint64_t e[6];
    std::memcpy(e, HP, 48);
    e[0] -= 2;
    hfp r, b = a;
    std::memcpy(r.l, HONE, 48);
    for (int i = 0; i < 381; i++) {
        if ((e[i / 64] >> (i % 64)) & 1) mul(r, r, b);
        mul(b, b, b);
    }
    o = r;
}

inline bool jac_is_inf(const hjac& p) { return is_zero(p.z); }

// dbl-2009-l (a = 0)
inline void jac_dbl(hjac& o, const hjac& p)
{
    if (jac_is_inf(p)) { o = p; return; }
    hfp A, B, C, D, E, F, t, X3, Y3, Z3;
    mul(A, p.x, p.x);
    mul(B, p.y, p.y);
    mul(C, B, B);
    add(t, p.x, B);
    mul(t, t, t);
    sub(t, t, A);
    sub(t, t, C);
    add(D, t, t);
    add(E, A, A);
    add(E, E, A);
    mul(F, E, E);
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
    mul(z1z1, a.z, a.z);
    mul(z2z2, b.z, b.z);
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
    mul(hh, h, h);
    mul(hhh, hh, h);
    mul(v, u1, hh);
    mul(X3, r, r);
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
    mul(zi2, zi, zi);
    mul(zi3, zi2, zi);
    mul(o.x, p.x, zi2);
    mul(o.y, p.y, zi3);
    std::memcpy(o.z.l, HONE, 48);
}

}  // namespace catmsm_host
