// Host-side Fr (4 x 64-bit Montgomery limbs, R = 2^256; same bytes as
// blst_fr) for the O(1) root constants of the FFT entry points: the primitive
// 2^k-th root (derived from 7^((r-1)/2^32) by repeated squaring, the rule the
// reference's root table follows, fft/primitive_root.h:29-62), its inverse,
// 1/n and the size tag n.
#pragma once
#include <cstdint>
#include <cstring>

namespace catmsm_host {

struct hfr { uint64_t l[4]; };

static const uint64_t HR[4] = {0xffffffff00000001ULL, 0x53bda402fffe5bfeULL, 0x3339d80809a1d805ULL,
                               0x73eda753299d7d48ULL};
static const uint64_t HR_ONE[4] = {0x00000001fffffffeULL, 0x5884b7fa00034802ULL, 0x998c4fefecbc4ff5ULL,
                                   0x1824b159acc5056fULL};
static const uint64_t HR_R2[4] = {0xc999e990f3f29c6dULL, 0x2b6cedcb87925c23ULL, 0x05d314967254398fULL,
                                  0x0748d9d99f59ff11ULL};
static const uint64_t HR_N0 = 0xfffffffeffffffffULL;

inline bool fr_geq(const uint64_t* a, const uint64_t* b)
{
    for (int i = 3; i >= 0; i--)
        if (a[i] != b[i]) return a[i] > b[i];
    return true;
}

inline void fr_mul(hfr& o, const hfr& a, const hfr& b)
{
    typedef unsigned __int128 u128;
    uint64_t t[6] = {0};
    for (int i = 0; i < 4; i++) {
        u128 c = 0;
        for (int j = 0; j < 4; j++) {
            c += (u128)a.l[j] * b.l[i] + t[j];
            t[j] = (uint64_t)c;
            c >>= 64;
        }
        c += t[4];
        t[4] = (uint64_t)c;
        t[5] = (uint64_t)(c >> 64);
        uint64_t m = t[0] * HR_N0;
        c = ((u128)m * HR[0] + t[0]) >> 64;
        for (int j = 1; j < 4; j++) {
            c += (u128)m * HR[j] + t[j];
            t[j - 1] = (uint64_t)c;
            c >>= 64;
        }
        c += t[4];
        t[3] = (uint64_t)c;
        t[4] = t[5] + (uint64_t)(c >> 64);
    }
    if (t[4] || fr_geq(t, HR)) {
        uint64_t br = 0;
        for (int i = 0; i < 4; i++) {
            u128 d = (u128)t[i] - HR[i] - br;
            t[i] = (uint64_t)d;
            br = (uint64_t)(d >> 64) & 1;
        }
    }
    std::memcpy(o.l, t, 32);
}

inline hfr fr_one() { hfr o; std::memcpy(o.l, HR_ONE, 32); return o; }

inline hfr fr_from_u64(uint64_t v)
{
    hfr a = {{v, 0, 0, 0}}, r2, o;
    std::memcpy(r2.l, HR_R2, 32);
    fr_mul(o, a, r2);
    return o;
}

// a^e for a 256-bit little-endian exponent
inline hfr fr_pow(const hfr& a, const uint64_t* e)
{
    hfr acc = fr_one(), b = a;
    for (int i = 0; i < 256; i++) {
        if ((e[i / 64] >> (i % 64)) & 1) fr_mul(acc, acc, b);
        fr_mul(b, b, b);
    }
    return acc;
}

inline hfr fr_inv(const hfr& a)
{
    uint64_t e[4];
    std::memcpy(e, HR, 32);
    e[0] -= 2;
    return fr_pow(a, e);
}

// primitive 2^logn-th root of unity (Montgomery), logn <= 32
inline hfr fr_root_of_unity(unsigned logn)
{
    uint64_t e[4];
    std::memcpy(e, HR, 32);
    e[0] -= 1;
    for (int i = 0; i < 4; i++) e[i] = (e[i] >> 32) | (i < 3 ? e[i + 1] << 32 : 0);
    hfr w = fr_pow(fr_from_u64(7), e);
    for (unsigned k = 32; k > logn; k--) fr_mul(w, w, w);
    return w;
}

}  // namespace catmsm_host
