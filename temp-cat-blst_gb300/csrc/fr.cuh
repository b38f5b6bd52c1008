// BLS12-381 scalar field Fr on device: 8 x 32-bit limbs, Montgomery form with
// R = 2^256 (same bytes as the reference's 4 x u64 blst_fr, scalar/fields/
// Fr.h:44-125).  Used only to prepare FFT roots (powers, from_mont, GLV split),
// which is O(n) work next to O(n log n) group operations, so a plain CIOS with
// 64-bit accumulators suffices here.
#pragma once
#include <cstdint>

namespace catmsm {

__device__ __constant__ static const uint32_t FR_R[8] = {
    0x00000001u, 0xffffffffu, 0xfffe5bfeu, 0x53bda402u, 0x09a1d805u, 0x3339d808u, 0x299d7d48u, 0x73eda753u};
__device__ __constant__ static const uint32_t FR_ONE_MONT[8] = {
    // 2^256 mod r
    0xfffffffeu, 0x00000001u, 0x00034802u, 0x5884b7fau, 0xecbc4ff5u, 0x998c4fefu, 0xacc5056fu, 0x1824b159u};
constexpr uint32_t FR_N0 = 0xffffffffu;
// lambda = 0xac45a4010001a40200000000ffffffff (GLV eigenvalue, lambda^2 + lambda + 1 = r)
__device__ __constant__ static const uint32_t FR_LAMBDA[4] = {0xffffffffu, 0x00000000u, 0x0001a402u, 0xac45a401u};

__device__ __forceinline__ bool fr_geq(const uint32_t* a, const uint32_t* b)
{
    for (int i = 7; i >= 0; i--)
        if (a[i] != b[i]) return a[i] > b[i];
    return true;
}

__device__ __forceinline__ void fr_sub_r(uint32_t* a)
{
    uint64_t br = 0;
    for (int i = 0; i < 8; i++) {
        uint64_t d = (uint64_t)a[i] - FR_R[i] - br;
        a[i] = (uint32_t)d;
        br = (d >> 63) & 1;
    }
}

// o = a * b * 2^-256 mod r (reduced)
__device__ __forceinline__ void fr_mul(uint32_t* o, const uint32_t* a, const uint32_t* b)
{
    uint32_t t[10];
    for (int i = 0; i < 10; i++) t[i] = 0;
    for (int i = 0; i < 8; i++) {
        uint64_t c = 0;
        for (int j = 0; j < 8; j++) {
            c += (uint64_t)a[j] * b[i] + t[j];
            t[j] = (uint32_t)c;
            c >>= 32;
        }
        c += t[8];
        t[8] = (uint32_t)c;
        t[9] = (uint32_t)(c >> 32);
        const uint32_t m = t[0] * FR_N0;
        c = ((uint64_t)m * FR_R[0] + t[0]) >> 32;
        for (int j = 1; j < 8; j++) {
            c += (uint64_t)m * FR_R[j] + t[j];
            t[j - 1] = (uint32_t)c;
            c >>= 32;
        }
        c += t[8];
        t[7] = (uint32_t)c;
        t[8] = t[9] + (uint32_t)(c >> 32);
    }
    if (t[8] || fr_geq(t, FR_R)) fr_sub_r(t);
    for (int i = 0; i < 8; i++) o[i] = t[i];
}

// o = a + b mod r, o = a - b mod r (reduced inputs and outputs)
__device__ __forceinline__ void fr_add(uint32_t* o, const uint32_t* a, const uint32_t* b)
{
    uint32_t t[8];
    uint64_t c = 0;
    for (int i = 0; i < 8; i++) {
        c += (uint64_t)a[i] + b[i];
        t[i] = (uint32_t)c;
        c >>= 32;
    }
    if (c || fr_geq(t, FR_R)) fr_sub_r(t);
    for (int i = 0; i < 8; i++) o[i] = t[i];
}

__device__ __forceinline__ void fr_sub(uint32_t* o, const uint32_t* a, const uint32_t* b)
{
    uint32_t t[8];
    uint64_t br = 0;
    for (int i = 0; i < 8; i++) {
        const uint64_t d = (uint64_t)a[i] - b[i] - br;
        t[i] = (uint32_t)d;
        br = (d >> 63) & 1;
    }
    if (br) {
        uint64_t c = 0;
        for (int i = 0; i < 8; i++) {
            c += (uint64_t)t[i] + FR_R[i];
            t[i] = (uint32_t)c;
            c >>= 32;
        }
    }
    for (int i = 0; i < 8; i++) o[i] = t[i];
}

__device__ __forceinline__ void fr_from_mont(uint32_t* o, const uint32_t* a)
{
    const uint32_t one[8] = {1, 0, 0, 0, 0, 0, 0, 0};
    fr_mul(o, a, one);
}

// o = base^e (Montgomery in/out), e < 2^32
__device__ __forceinline__ void fr_pow_u32(uint32_t* o, const uint32_t* base, uint32_t e)
{
    uint32_t acc[8], b[8];
    for (int i = 0; i < 8; i++) { acc[i] = FR_ONE_MONT[i]; b[i] = base[i]; }
    while (e) {
        if (e & 1) fr_mul(acc, acc, b);
        fr_mul(b, b, b);
        e >>= 1;
    }
    for (int i = 0; i < 8; i++) o[i] = acc[i];
}

// floor(2^256 / lambda), 129 bits, little-endian words
__device__ __constant__ static const uint32_t FR_LAMBDA_MU[5] = {0xf6cfee30u, 0x63f6e522u, 0xe01faaddu, 0x7c6becf1u,
                                                                 0x00000001u};

// GLV split of a canonical k < r: k = k1 + lambda * k2, 0 <= k1 < lambda,
// k2 = floor(k / lambda) <= lambda + 1 (both fit 128 bits).  Barrett
// quotient q = floor(floor(k / 2^127) * mu / 2^129) with mu = floor(2^256 /
// lambda) is at most two below floor(k / lambda); the remainder is corrected
// by at most two subtractions.
__device__ __forceinline__ void fr_glv_split(uint32_t* k1, uint32_t* k2, const uint32_t* k)
{
    uint32_t a[4];
#pragma unroll
    for (int i = 0; i < 4; i++) a[i] = (k[i + 3] >> 31) | (k[i + 4] << 1);   // k >> 127 (k < 2^255)
    uint32_t prod[9];
#pragma unroll
    for (int i = 0; i < 9; i++) prod[i] = 0;
#pragma unroll
    for (int i = 0; i < 4; i++) {
        uint64_t c = 0;
#pragma unroll
        for (int j = 0; j < 5; j++) {
            c += (uint64_t)a[i] * FR_LAMBDA_MU[j] + prod[i + j];
            prod[i + j] = (uint32_t)c;
            c >>= 32;
        }
        prod[i + 5] = (uint32_t)c;
    }
    uint32_t q[4];
#pragma unroll
    for (int i = 0; i < 4; i++) q[i] = (prod[i + 4] >> 1) | (prod[i + 5] << 31);   // >> 129
    // rem = k - q * lambda (< 3 lambda: five words)
    uint32_t t[8];
#pragma unroll
    for (int i = 0; i < 8; i++) t[i] = 0;
#pragma unroll
    for (int i = 0; i < 4; i++) {
        uint64_t c = 0;
#pragma unroll
        for (int j = 0; j < 4; j++) {
            c += (uint64_t)q[i] * FR_LAMBDA[j] + t[i + j];
            t[i + j] = (uint32_t)c;
            c >>= 32;
        }
        t[i + 4] = (uint32_t)c;
    }
    uint32_t rem[5];
    uint64_t br = 0;
#pragma unroll
    for (int i = 0; i < 5; i++) {
        const uint64_t d = (uint64_t)k[i] - t[i] - br;
        rem[i] = (uint32_t)d;
        br = (d >> 63) & 1;
    }
    for (int it = 0; it < 3; it++) {
        bool ge = rem[4] != 0;
        if (!ge) {
            ge = true;
            for (int w = 3; w >= 0; w--) {
                if (rem[w] != FR_LAMBDA[w]) { ge = rem[w] > FR_LAMBDA[w]; break; }
            }
        }
        if (!ge) break;
        br = 0;
#pragma unroll
        for (int w = 0; w < 4; w++) {
            const uint64_t d = (uint64_t)rem[w] - FR_LAMBDA[w] - br;
            rem[w] = (uint32_t)d;
            br = (d >> 63) & 1;
        }
        rem[4] -= (uint32_t)br;
        for (int w = 0; w < 4 && ++q[w] == 0; w++) {}
    }
#pragma unroll
    for (int w = 0; w < 4; w++) { k1[w] = rem[w]; k2[w] = q[w]; }
}

// (lambda + 1) / 2 and lambda + 1, little-endian words (lambda = z^2 - 1,
// lambda^2 + lambda + 1 = r)
__device__ __constant__ static const uint32_t GLV_HALF[4] = {0x80000000u, 0x00000000u, 0x8000d201u, 0x5622d200u};
__device__ __constant__ static const uint32_t GLV_LAMBDA1[4] = {0x00000000u, 0x00000001u, 0x0001a402u, 0xac45a401u};

__device__ __forceinline__ bool ge4(const uint32_t* a, const uint32_t* b)
{
    for (int i = 3; i >= 0; i--)
        if (a[i] != b[i]) return a[i] > b[i];
    return true;
}

__device__ __forceinline__ void sub4(uint32_t* o, const uint32_t* a, const uint32_t* b)
{
    uint64_t br = 0;
    for (int i = 0; i < 4; i++) {
        const uint64_t d = (uint64_t)a[i] - b[i] - br;
        o[i] = (uint32_t)d;
        br = (d >> 63) & 1;
    }
}

__device__ __forceinline__ void inc4(uint32_t* a)
{
    for (int i = 0; i < 4 && ++a[i] == 0; i++) {}
}

__device__ __forceinline__ void dec4(uint32_t* a)
{
    for (int i = 0; i < 4 && a[i]-- == 0; i++) {}
}


// Balanced GLV split of any k < 2^256 (the MSM pipelines): k mod r = s1 m1 +
// s2 m2 lambda with m1, m2 <= (lambda + 1) / 2 < 2^127 (s = true: negative).
//   k1 >= (lambda+1)/2:  k1 -> k1 - lambda,  k2 -> k2 + 1
//   k2 >= (lambda+1)/2:  k2 -> k2 - lambda - 1,  k1 -> k1 - 1
// (the second uses lambda^2 = -lambda - 1 mod r).  k is reduced in place.
__device__ __forceinline__ void fr_glv_balanced(uint32_t* m1, uint32_t* m2, bool& s1, bool& s2, uint32_t* k)
{
    while (fr_geq(k, FR_R)) fr_sub_r(k);
    fr_glv_split(m1, m2, k);
    s1 = false;
    s2 = false;
    if (ge4(m1, GLV_HALF)) {
        sub4(m1, FR_LAMBDA, m1);
        s1 = true;
        inc4(m2);
    }
    if (ge4(m2, GLV_HALF)) {
        sub4(m2, GLV_LAMBDA1, m2);
        s2 = true;
        if (s1) {
            inc4(m1);
        } else if ((m1[0] | m1[1] | m1[2] | m1[3]) == 0) {
            m1[0] = 1;
            s1 = true;
        } else {
            dec4(m1);
        }
    }
}

}  // namespace catmsm
