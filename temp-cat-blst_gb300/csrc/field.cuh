// BLS12-381 base field Fp on sm_103a: 12 x 32-bit limbs, Montgomery form with
// R = 2^384.  Because 12 x 32 = 6 x 64, the Montgomery representation (and the
// little-endian byte image) is identical to the reference's 6 x u64 blst_fp
// (bindings/blst_types.h:84, scalar/fields/Fp.h:35-40), so device buffers hold
// caller bytes unchanged.
//
// Multiplication is CIOS Montgomery (Koc, Acar, Kaliski 1996) written with PTX
// carry chains (mad.lo.cc / madc.hi.cc).  Each limb step keeps two independent
// accumulators: E collects the even-limb products (a[2k]*b_i, p[2k]*m) whose
// low/high words fall on even/odd weights without overlap, and O collects the
// odd-limb products shifted by one word.  One add chain merges them while
// dividing by 2^32.  Two chains in flight per step give the scheduler ILP.
//
// Values are kept lazily reduced in [0, 2p): 4p < 2^384 / 2, so a product of
// two values below 2p leaves CIOS below 1.41p and the final conditional
// subtraction is skipped.  add/sub reduce modulo 2p.  fp_canon() maps to
// [0, p) for output; fp_is_zero() tests congruence to zero.
#pragma once
#include <cstdint>

namespace catmsm {

struct fp { uint32_t v[12]; };

// p, 2p, R mod p (Montgomery one), R^2 mod p, -p^-1 mod 2^32
#define CATMSM_P0  0xffffaaabu
#define CATMSM_P1  0xb9feffffu
#define CATMSM_P2  0xb153ffffu
#define CATMSM_P3  0x1eabfffeu
#define CATMSM_P4  0xf6b0f624u
#define CATMSM_P5  0x6730d2a0u
#define CATMSM_P6  0xf38512bfu
#define CATMSM_P7  0x64774b84u
#define CATMSM_P8  0x434bacd7u
#define CATMSM_P9  0x4b1ba7b6u
#define CATMSM_P10 0x397fe69au
#define CATMSM_P11 0x1a0111eau
#define CATMSM_N0  0xfffcfffdu

__device__ __constant__ static const uint32_t FP_P[12] = {
    0xffffaaabu, 0xb9feffffu, 0xb153ffffu, 0x1eabfffeu, 0xf6b0f624u, 0x6730d2a0u,
    0xf38512bfu, 0x64774b84u, 0x434bacd7u, 0x4b1ba7b6u, 0x397fe69au, 0x1a0111eau};
__device__ __constant__ static const uint32_t FP_ONE[12] = {
    0x0002fffdu, 0x76090000u, 0xc40c0002u, 0xebf4000bu, 0x53c758bau, 0x5f489857u,
    0x70525745u, 0x77ce5853u, 0xa256ec6du, 0x5c071a97u, 0xfa80e493u, 0x15f65ec3u};

__device__ __forceinline__ void fp_zero(fp& r)
{
#pragma unroll
    for (int i = 0; i < 12; i++) r.v[i] = 0;
}

__device__ __forceinline__ void fp_set_one(fp& r)
{
#pragma unroll
    for (int i = 0; i < 12; i++) r.v[i] = FP_ONE[i];
}

// r = a * b * 2^-384 mod p; inputs in [0, 2p), output in [0, 2p).
__device__ __forceinline__ void fp_mul_impl(fp& r, const fp& a, const fp& b)
{
    uint32_t t[12];
    uint32_t e[13], o[13];
#pragma unroll
    for (int i = 0; i < 12; i++) {
        const uint32_t bi = b.v[i];
        if (i == 0) {
#pragma unroll
            for (int k = 0; k < 6; k++) {
                e[2 * k] = a.v[2 * k] * bi;
                e[2 * k + 1] = __umulhi(a.v[2 * k], bi);
            }
            e[12] = 0;
        } else {
#pragma unroll
            for (int k = 0; k < 12; k++) e[k] = t[k];
            asm("mad.lo.cc.u32  %0, %13, %19, %0;\n\t"
                "madc.hi.cc.u32 %1, %13, %19, %1;\n\t"
                "madc.lo.cc.u32 %2, %14, %19, %2;\n\t"
                "madc.hi.cc.u32 %3, %14, %19, %3;\n\t"
                "madc.lo.cc.u32 %4, %15, %19, %4;\n\t"
                "madc.hi.cc.u32 %5, %15, %19, %5;\n\t"
                "madc.lo.cc.u32 %6, %16, %19, %6;\n\t"
                "madc.hi.cc.u32 %7, %16, %19, %7;\n\t"
                "madc.lo.cc.u32 %8, %17, %19, %8;\n\t"
                "madc.hi.cc.u32 %9, %17, %19, %9;\n\t"
                "madc.lo.cc.u32 %10, %18, %19, %10;\n\t"
                "madc.hi.cc.u32 %11, %18, %19, %11;\n\t"
                "addc.u32       %12, 0, 0;"
                : "+r"(e[0]), "+r"(e[1]), "+r"(e[2]), "+r"(e[3]), "+r"(e[4]), "+r"(e[5]),
                  "+r"(e[6]), "+r"(e[7]), "+r"(e[8]), "+r"(e[9]), "+r"(e[10]), "+r"(e[11]),
                  "=r"(e[12])
                : "r"(a.v[0]), "r"(a.v[2]), "r"(a.v[4]), "r"(a.v[6]), "r"(a.v[8]), "r"(a.v[10]),
                  "r"(bi));
        }
#pragma unroll
        for (int k = 0; k < 6; k++) {
            o[2 * k] = a.v[2 * k + 1] * bi;
            o[2 * k + 1] = __umulhi(a.v[2 * k + 1], bi);
        }
        const uint32_t m = e[0] * CATMSM_N0;
        asm("mad.lo.cc.u32  %0, %13, %14, %0;\n\t"
            "madc.hi.cc.u32 %1, %13, %14, %1;\n\t"
            "madc.lo.cc.u32 %2, %13, %15, %2;\n\t"
            "madc.hi.cc.u32 %3, %13, %15, %3;\n\t"
            "madc.lo.cc.u32 %4, %13, %16, %4;\n\t"
            "madc.hi.cc.u32 %5, %13, %16, %5;\n\t"
            "madc.lo.cc.u32 %6, %13, %17, %6;\n\t"
            "madc.hi.cc.u32 %7, %13, %17, %7;\n\t"
            "madc.lo.cc.u32 %8, %13, %18, %8;\n\t"
            "madc.hi.cc.u32 %9, %13, %18, %9;\n\t"
            "madc.lo.cc.u32 %10, %13, %19, %10;\n\t"
            "madc.hi.cc.u32 %11, %13, %19, %11;\n\t"
            "addc.u32       %12, %12, 0;"
            : "+r"(e[0]), "+r"(e[1]), "+r"(e[2]), "+r"(e[3]), "+r"(e[4]), "+r"(e[5]),
              "+r"(e[6]), "+r"(e[7]), "+r"(e[8]), "+r"(e[9]), "+r"(e[10]), "+r"(e[11]),
              "+r"(e[12])
            : "r"(m), "n"(CATMSM_P0), "n"(CATMSM_P2), "n"(CATMSM_P4), "n"(CATMSM_P6),
              "n"(CATMSM_P8), "n"(CATMSM_P10));
        asm("mad.lo.cc.u32  %0, %13, %14, %0;\n\t"
            "madc.hi.cc.u32 %1, %13, %14, %1;\n\t"
            "madc.lo.cc.u32 %2, %13, %15, %2;\n\t"
            "madc.hi.cc.u32 %3, %13, %15, %3;\n\t"
            "madc.lo.cc.u32 %4, %13, %16, %4;\n\t"
            "madc.hi.cc.u32 %5, %13, %16, %5;\n\t"
            "madc.lo.cc.u32 %6, %13, %17, %6;\n\t"
            "madc.hi.cc.u32 %7, %13, %17, %7;\n\t"
            "madc.lo.cc.u32 %8, %13, %18, %8;\n\t"
            "madc.hi.cc.u32 %9, %13, %18, %9;\n\t"
            "madc.lo.cc.u32 %10, %13, %19, %10;\n\t"
            "madc.hi.cc.u32 %11, %13, %19, %11;\n\t"
            "addc.u32       %12, 0, 0;"
            : "+r"(o[0]), "+r"(o[1]), "+r"(o[2]), "+r"(o[3]), "+r"(o[4]), "+r"(o[5]),
              "+r"(o[6]), "+r"(o[7]), "+r"(o[8]), "+r"(o[9]), "+r"(o[10]), "+r"(o[11]),
              "=r"(o[12])
            : "r"(m), "n"(CATMSM_P1), "n"(CATMSM_P3), "n"(CATMSM_P5), "n"(CATMSM_P7),
              "n"(CATMSM_P9), "n"(CATMSM_P11));
        // t = (E + O*2^32) / 2^32: weight-k word is E[k+1] + O[k]
        asm("add.cc.u32  %0, %0, %12;\n\t"
            "addc.cc.u32 %1, %1, %13;\n\t"
            "addc.cc.u32 %2, %2, %14;\n\t"
            "addc.cc.u32 %3, %3, %15;\n\t"
            "addc.cc.u32 %4, %4, %16;\n\t"
            "addc.cc.u32 %5, %5, %17;\n\t"
            "addc.cc.u32 %6, %6, %18;\n\t"
            "addc.cc.u32 %7, %7, %19;\n\t"
            "addc.cc.u32 %8, %8, %20;\n\t"
            "addc.cc.u32 %9, %9, %21;\n\t"
            "addc.cc.u32 %10, %10, %22;\n\t"
            "addc.u32    %11, %11, %23;"
            : "+r"(o[0]), "+r"(o[1]), "+r"(o[2]), "+r"(o[3]), "+r"(o[4]), "+r"(o[5]),
              "+r"(o[6]), "+r"(o[7]), "+r"(o[8]), "+r"(o[9]), "+r"(o[10]), "+r"(o[11])
            : "r"(e[1]), "r"(e[2]), "r"(e[3]), "r"(e[4]), "r"(e[5]), "r"(e[6]),
              "r"(e[7]), "r"(e[8]), "r"(e[9]), "r"(e[10]), "r"(e[11]), "r"(e[12]));
#pragma unroll
        for (int k = 0; k < 12; k++) t[k] = o[k];
    }
#pragma unroll
    for (int k = 0; k < 12; k++) r.v[k] = t[k];
}

// The multiplication is one out-of-line function per translation unit, called
// with its operands and result in registers.  Inlined, a group operation is
// ~10 copies of ~750 instructions and the accumulation loop outgrows the
// instruction cache (ncu: ~2 cycles of no_instruction stall per issue); out of
// line the hot loop is one body plus call sites.  Measured on GB300: the 2^20
// MSM 9.1 -> 8.0 ms, a 2^14 G1 FFT 39 -> 26 ms.
static __device__ __noinline__ fp fp_mul_call(const fp a, const fp b)
{
    fp r;
    fp_mul_impl(r, a, b);
    return r;
}

__device__ __forceinline__ void fp_mul(fp& r, const fp& a, const fp& b) { r = fp_mul_call(a, b); }

// r = a^2 * 2^-384 mod p; input in [0, 2p), output in [0, 2p).  The CIOS
// schedule of fp_mul_impl with the symmetry of a square: step i adds
// a_i * V_i, V_i = a_i 2^(32i) + 2 sum_{j>i} a_j 2^(32j) (a < 2p keeps the top word
// below 2^30, so doubling stays in 12 words), i.e. 12 - i limb products
// instead of 12: 156 product IMAD instead of 288.  Products of even and odd
// positions go to the independent E and O accumulators as in fp_mul_impl, and
// the Montgomery step is the same.  Each step adds at most 4p 2^32, so the
// running value stays below 6p < 2^384 and the result below 2p.  The body is
// the output of gen/gen_fp_sqr.py (in this package), checked by a CPU test.
__device__ __forceinline__ void fp_sqr_impl(fp& r, const fp& a)
{
    uint32_t t[12], e[13], o[13], d[12];
#pragma unroll
    for (int j = 1; j < 12; j++) d[j] = __funnelshift_l(a.v[j - 1], a.v[j], 1);   // (2a)_j
    {   // step 0
        const uint32_t bi = a.v[0];
#pragma unroll
        for (int k = 0; k < 13; k++) e[k] = 0;
        e[0] = a.v[0] * bi;
        e[1] = __umulhi(a.v[0], bi);
        e[2] = d[2] * bi;
        e[3] = __umulhi(d[2], bi);
        e[4] = d[4] * bi;
        e[5] = __umulhi(d[4], bi);
        e[6] = d[6] * bi;
        e[7] = __umulhi(d[6], bi);
        e[8] = d[8] * bi;
        e[9] = __umulhi(d[8], bi);
        e[10] = d[10] * bi;
        e[11] = __umulhi(d[10], bi);
#pragma unroll
        for (int k = 0; k < 13; k++) o[k] = 0;
        o[0] = (a.v[1] << 1) * bi;
        o[1] = __umulhi((a.v[1] << 1), bi);
        o[2] = d[3] * bi;
        o[3] = __umulhi(d[3], bi);
        o[4] = d[5] * bi;
        o[5] = __umulhi(d[5], bi);
        o[6] = d[7] * bi;
        o[7] = __umulhi(d[7], bi);
        o[8] = d[9] * bi;
        o[9] = __umulhi(d[9], bi);
        o[10] = d[11] * bi;
        o[11] = __umulhi(d[11], bi);
        const uint32_t m = e[0] * CATMSM_N0;
        asm("mad.lo.cc.u32  %0, %13, %14, %0;\n\t"
            "madc.hi.cc.u32 %1, %13, %14, %1;\n\t"
            "madc.lo.cc.u32 %2, %13, %15, %2;\n\t"
            "madc.hi.cc.u32 %3, %13, %15, %3;\n\t"
            "madc.lo.cc.u32 %4, %13, %16, %4;\n\t"
            "madc.hi.cc.u32 %5, %13, %16, %5;\n\t"
            "madc.lo.cc.u32 %6, %13, %17, %6;\n\t"
            "madc.hi.cc.u32 %7, %13, %17, %7;\n\t"
            "madc.lo.cc.u32 %8, %13, %18, %8;\n\t"
            "madc.hi.cc.u32 %9, %13, %18, %9;\n\t"
            "madc.lo.cc.u32 %10, %13, %19, %10;\n\t"
            "madc.hi.cc.u32 %11, %13, %19, %11;\n\t"
            "addc.u32       %12, %12, 0;"
            : "+r"(e[0]), "+r"(e[1]), "+r"(e[2]), "+r"(e[3]), "+r"(e[4]), "+r"(e[5]),
              "+r"(e[6]), "+r"(e[7]), "+r"(e[8]), "+r"(e[9]), "+r"(e[10]), "+r"(e[11]),
              "+r"(e[12])
            : "r"(m), "n"(CATMSM_P0), "n"(CATMSM_P2), "n"(CATMSM_P4), "n"(CATMSM_P6),
              "n"(CATMSM_P8), "n"(CATMSM_P10));
        asm("mad.lo.cc.u32  %0, %13, %14, %0;\n\t"
            "madc.hi.cc.u32 %1, %13, %14, %1;\n\t"
            "madc.lo.cc.u32 %2, %13, %15, %2;\n\t"
            "madc.hi.cc.u32 %3, %13, %15, %3;\n\t"
            "madc.lo.cc.u32 %4, %13, %16, %4;\n\t"
            "madc.hi.cc.u32 %5, %13, %16, %5;\n\t"
            "madc.lo.cc.u32 %6, %13, %17, %6;\n\t"
            "madc.hi.cc.u32 %7, %13, %17, %7;\n\t"
            "madc.lo.cc.u32 %8, %13, %18, %8;\n\t"
            "madc.hi.cc.u32 %9, %13, %18, %9;\n\t"
            "madc.lo.cc.u32 %10, %13, %19, %10;\n\t"
            "madc.hi.cc.u32 %11, %13, %19, %11;\n\t"
            "addc.u32       %12, 0, 0;"
            : "+r"(o[0]), "+r"(o[1]), "+r"(o[2]), "+r"(o[3]), "+r"(o[4]), "+r"(o[5]),
              "+r"(o[6]), "+r"(o[7]), "+r"(o[8]), "+r"(o[9]), "+r"(o[10]), "+r"(o[11]),
              "=r"(o[12])
            : "r"(m), "n"(CATMSM_P1), "n"(CATMSM_P3), "n"(CATMSM_P5), "n"(CATMSM_P7),
              "n"(CATMSM_P9), "n"(CATMSM_P11));
        asm("add.cc.u32  %0, %0, %12;\n\t"
            "addc.cc.u32 %1, %1, %13;\n\t"
            "addc.cc.u32 %2, %2, %14;\n\t"
            "addc.cc.u32 %3, %3, %15;\n\t"
            "addc.cc.u32 %4, %4, %16;\n\t"
            "addc.cc.u32 %5, %5, %17;\n\t"
            "addc.cc.u32 %6, %6, %18;\n\t"
            "addc.cc.u32 %7, %7, %19;\n\t"
            "addc.cc.u32 %8, %8, %20;\n\t"
            "addc.cc.u32 %9, %9, %21;\n\t"
            "addc.cc.u32 %10, %10, %22;\n\t"
            "addc.u32    %11, %11, %23;"
            : "+r"(o[0]), "+r"(o[1]), "+r"(o[2]), "+r"(o[3]), "+r"(o[4]), "+r"(o[5]),
              "+r"(o[6]), "+r"(o[7]), "+r"(o[8]), "+r"(o[9]), "+r"(o[10]), "+r"(o[11])
            : "r"(e[1]), "r"(e[2]), "r"(e[3]), "r"(e[4]), "r"(e[5]), "r"(e[6]),
              "r"(e[7]), "r"(e[8]), "r"(e[9]), "r"(e[10]), "r"(e[11]), "r"(e[12]));
#pragma unroll
        for (int k = 0; k < 12; k++) t[k] = o[k];
    }
    {   // step 1
        const uint32_t bi = a.v[1];
#pragma unroll
        for (int k = 0; k < 12; k++) e[k] = t[k];
        asm("mad.lo.cc.u32  %0, %11, %16, %0;\n\t"
            "madc.hi.cc.u32 %1, %11, %16, %1;\n\t"
            "madc.lo.cc.u32 %2, %12, %16, %2;\n\t"
            "madc.hi.cc.u32 %3, %12, %16, %3;\n\t"
            "madc.lo.cc.u32 %4, %13, %16, %4;\n\t"
            "madc.hi.cc.u32 %5, %13, %16, %5;\n\t"
            "madc.lo.cc.u32 %6, %14, %16, %6;\n\t"
            "madc.hi.cc.u32 %7, %14, %16, %7;\n\t"
            "madc.lo.cc.u32 %8, %15, %16, %8;\n\t"
            "madc.hi.cc.u32 %9, %15, %16, %9;\n\t"
            "addc.u32       %10, 0, 0;"
            : "+r"(e[2]), "+r"(e[3]), "+r"(e[4]), "+r"(e[5]), "+r"(e[6]), "+r"(e[7]), "+r"(e[8]), "+r"(e[9]), "+r"(e[10]), "+r"(e[11]), "=r"(e[12])
            : "r"((a.v[2] << 1)), "r"(d[4]), "r"(d[6]), "r"(d[8]), "r"(d[10]), "r"(bi));
#pragma unroll
        for (int k = 0; k < 13; k++) o[k] = 0;
        o[0] = a.v[1] * bi;
        o[1] = __umulhi(a.v[1], bi);
        o[2] = d[3] * bi;
        o[3] = __umulhi(d[3], bi);
        o[4] = d[5] * bi;
        o[5] = __umulhi(d[5], bi);
        o[6] = d[7] * bi;
        o[7] = __umulhi(d[7], bi);
        o[8] = d[9] * bi;
        o[9] = __umulhi(d[9], bi);
        o[10] = d[11] * bi;
        o[11] = __umulhi(d[11], bi);
        const uint32_t m = e[0] * CATMSM_N0;
        asm("mad.lo.cc.u32  %0, %13, %14, %0;\n\t"
            "madc.hi.cc.u32 %1, %13, %14, %1;\n\t"
            "madc.lo.cc.u32 %2, %13, %15, %2;\n\t"
            "madc.hi.cc.u32 %3, %13, %15, %3;\n\t"
            "madc.lo.cc.u32 %4, %13, %16, %4;\n\t"
            "madc.hi.cc.u32 %5, %13, %16, %5;\n\t"
            "madc.lo.cc.u32 %6, %13, %17, %6;\n\t"
            "madc.hi.cc.u32 %7, %13, %17, %7;\n\t"
            "madc.lo.cc.u32 %8, %13, %18, %8;\n\t"
            "madc.hi.cc.u32 %9, %13, %18, %9;\n\t"
            "madc.lo.cc.u32 %10, %13, %19, %10;\n\t"
            "madc.hi.cc.u32 %11, %13, %19, %11;\n\t"
            "addc.u32       %12, %12, 0;"
            : "+r"(e[0]), "+r"(e[1]), "+r"(e[2]), "+r"(e[3]), "+r"(e[4]), "+r"(e[5]),
              "+r"(e[6]), "+r"(e[7]), "+r"(e[8]), "+r"(e[9]), "+r"(e[10]), "+r"(e[11]),
              "+r"(e[12])
            : "r"(m), "n"(CATMSM_P0), "n"(CATMSM_P2), "n"(CATMSM_P4), "n"(CATMSM_P6),
              "n"(CATMSM_P8), "n"(CATMSM_P10));
        asm("mad.lo.cc.u32  %0, %13, %14, %0;\n\t"
            "madc.hi.cc.u32 %1, %13, %14, %1;\n\t"
            "madc.lo.cc.u32 %2, %13, %15, %2;\n\t"
            "madc.hi.cc.u32 %3, %13, %15, %3;\n\t"
            "madc.lo.cc.u32 %4, %13, %16, %4;\n\t"
            "madc.hi.cc.u32 %5, %13, %16, %5;\n\t"
            "madc.lo.cc.u32 %6, %13, %17, %6;\n\t"
            "madc.hi.cc.u32 %7, %13, %17, %7;\n\t"
            "madc.lo.cc.u32 %8, %13, %18, %8;\n\t"
            "madc.hi.cc.u32 %9, %13, %18, %9;\n\t"
            "madc.lo.cc.u32 %10, %13, %19, %10;\n\t"
            "madc.hi.cc.u32 %11, %13, %19, %11;\n\t"
            "addc.u32       %12, 0, 0;"
            : "+r"(o[0]), "+r"(o[1]), "+r"(o[2]), "+r"(o[3]), "+r"(o[4]), "+r"(o[5]),
              "+r"(o[6]), "+r"(o[7]), "+r"(o[8]), "+r"(o[9]), "+r"(o[10]), "+r"(o[11]),
              "=r"(o[12])
            : "r"(m), "n"(CATMSM_P1), "n"(CATMSM_P3), "n"(CATMSM_P5), "n"(CATMSM_P7),
              "n"(CATMSM_P9), "n"(CATMSM_P11));
        asm("add.cc.u32  %0, %0, %12;\n\t"
            "addc.cc.u32 %1, %1, %13;\n\t"
            "addc.cc.u32 %2, %2, %14;\n\t"
            "addc.cc.u32 %3, %3, %15;\n\t"
            "addc.cc.u32 %4, %4, %16;\n\t"
            "addc.cc.u32 %5, %5, %17;\n\t"
            "addc.cc.u32 %6, %6, %18;\n\t"
            "addc.cc.u32 %7, %7, %19;\n\t"
            "addc.cc.u32 %8, %8, %20;\n\t"
            "addc.cc.u32 %9, %9, %21;\n\t"
            "addc.cc.u32 %10, %10, %22;\n\t"
            "addc.u32    %11, %11, %23;"
            : "+r"(o[0]), "+r"(o[1]), "+r"(o[2]), "+r"(o[3]), "+r"(o[4]), "+r"(o[5]),
              "+r"(o[6]), "+r"(o[7]), "+r"(o[8]), "+r"(o[9]), "+r"(o[10]), "+r"(o[11])
            : "r"(e[1]), "r"(e[2]), "r"(e[3]), "r"(e[4]), "r"(e[5]), "r"(e[6]),
              "r"(e[7]), "r"(e[8]), "r"(e[9]), "r"(e[10]), "r"(e[11]), "r"(e[12]));
#pragma unroll
        for (int k = 0; k < 12; k++) t[k] = o[k];
    }
    {   // step 2
        const uint32_t bi = a.v[2];
#pragma unroll
        for (int k = 0; k < 12; k++) e[k] = t[k];
        asm("mad.lo.cc.u32  %0, %11, %16, %0;\n\t"
            "madc.hi.cc.u32 %1, %11, %16, %1;\n\t"
            "madc.lo.cc.u32 %2, %12, %16, %2;\n\t"
            "madc.hi.cc.u32 %3, %12, %16, %3;\n\t"
            "madc.lo.cc.u32 %4, %13, %16, %4;\n\t"
            "madc.hi.cc.u32 %5, %13, %16, %5;\n\t"
            "madc.lo.cc.u32 %6, %14, %16, %6;\n\t"
            "madc.hi.cc.u32 %7, %14, %16, %7;\n\t"
            "madc.lo.cc.u32 %8, %15, %16, %8;\n\t"
            "madc.hi.cc.u32 %9, %15, %16, %9;\n\t"
            "addc.u32       %10, 0, 0;"
            : "+r"(e[2]), "+r"(e[3]), "+r"(e[4]), "+r"(e[5]), "+r"(e[6]), "+r"(e[7]), "+r"(e[8]), "+r"(e[9]), "+r"(e[10]), "+r"(e[11]), "=r"(e[12])
            : "r"(a.v[2]), "r"(d[4]), "r"(d[6]), "r"(d[8]), "r"(d[10]), "r"(bi));
#pragma unroll
        for (int k = 0; k < 13; k++) o[k] = 0;
        o[2] = (a.v[3] << 1) * bi;
        o[3] = __umulhi((a.v[3] << 1), bi);
        o[4] = d[5] * bi;
        o[5] = __umulhi(d[5], bi);
        o[6] = d[7] * bi;
        o[7] = __umulhi(d[7], bi);
        o[8] = d[9] * bi;
        o[9] = __umulhi(d[9], bi);
        o[10] = d[11] * bi;
        o[11] = __umulhi(d[11], bi);
        const uint32_t m = e[0] * CATMSM_N0;
        asm("mad.lo.cc.u32  %0, %13, %14, %0;\n\t"
            "madc.hi.cc.u32 %1, %13, %14, %1;\n\t"
            "madc.lo.cc.u32 %2, %13, %15, %2;\n\t"
            "madc.hi.cc.u32 %3, %13, %15, %3;\n\t"
            "madc.lo.cc.u32 %4, %13, %16, %4;\n\t"
            "madc.hi.cc.u32 %5, %13, %16, %5;\n\t"
            "madc.lo.cc.u32 %6, %13, %17, %6;\n\t"
            "madc.hi.cc.u32 %7, %13, %17, %7;\n\t"
            "madc.lo.cc.u32 %8, %13, %18, %8;\n\t"
            "madc.hi.cc.u32 %9, %13, %18, %9;\n\t"
            "madc.lo.cc.u32 %10, %13, %19, %10;\n\t"
            "madc.hi.cc.u32 %11, %13, %19, %11;\n\t"
            "addc.u32       %12, %12, 0;"
            : "+r"(e[0]), "+r"(e[1]), "+r"(e[2]), "+r"(e[3]), "+r"(e[4]), "+r"(e[5]),
              "+r"(e[6]), "+r"(e[7]), "+r"(e[8]), "+r"(e[9]), "+r"(e[10]), "+r"(e[11]),
              "+r"(e[12])
            : "r"(m), "n"(CATMSM_P0), "n"(CATMSM_P2), "n"(CATMSM_P4), "n"(CATMSM_P6),
              "n"(CATMSM_P8), "n"(CATMSM_P10));
        asm("mad.lo.cc.u32  %0, %13, %14, %0;\n\t"
            "madc.hi.cc.u32 %1, %13, %14, %1;\n\t"
            "madc.lo.cc.u32 %2, %13, %15, %2;\n\t"
            "madc.hi.cc.u32 %3, %13, %15, %3;\n\t"
            "madc.lo.cc.u32 %4, %13, %16, %4;\n\t"
            "madc.hi.cc.u32 %5, %13, %16, %5;\n\t"
            "madc.lo.cc.u32 %6, %13, %17, %6;\n\t"
            "madc.hi.cc.u32 %7, %13, %17, %7;\n\t"
            "madc.lo.cc.u32 %8, %13, %18, %8;\n\t"
            "madc.hi.cc.u32 %9, %13, %18, %9;\n\t"
            "madc.lo.cc.u32 %10, %13, %19, %10;\n\t"
            "madc.hi.cc.u32 %11, %13, %19, %11;\n\t"
            "addc.u32       %12, 0, 0;"
            : "+r"(o[0]), "+r"(o[1]), "+r"(o[2]), "+r"(o[3]), "+r"(o[4]), "+r"(o[5]),
              "+r"(o[6]), "+r"(o[7]), "+r"(o[8]), "+r"(o[9]), "+r"(o[10]), "+r"(o[11]),
              "=r"(o[12])
            : "r"(m), "n"(CATMSM_P1), "n"(CATMSM_P3), "n"(CATMSM_P5), "n"(CATMSM_P7),
              "n"(CATMSM_P9), "n"(CATMSM_P11));
        asm("add.cc.u32  %0, %0, %12;\n\t"
            "addc.cc.u32 %1, %1, %13;\n\t"
            "addc.cc.u32 %2, %2, %14;\n\t"
            "addc.cc.u32 %3, %3, %15;\n\t"
            "addc.cc.u32 %4, %4, %16;\n\t"
            "addc.cc.u32 %5, %5, %17;\n\t"
            "addc.cc.u32 %6, %6, %18;\n\t"
            "addc.cc.u32 %7, %7, %19;\n\t"
            "addc.cc.u32 %8, %8, %20;\n\t"
            "addc.cc.u32 %9, %9, %21;\n\t"
            "addc.cc.u32 %10, %10, %22;\n\t"
            "addc.u32    %11, %11, %23;"
            : "+r"(o[0]), "+r"(o[1]), "+r"(o[2]), "+r"(o[3]), "+r"(o[4]), "+r"(o[5]),
              "+r"(o[6]), "+r"(o[7]), "+r"(o[8]), "+r"(o[9]), "+r"(o[10]), "+r"(o[11])
            : "r"(e[1]), "r"(e[2]), "r"(e[3]), "r"(e[4]), "r"(e[5]), "r"(e[6]),
              "r"(e[7]), "r"(e[8]), "r"(e[9]), "r"(e[10]), "r"(e[11]), "r"(e[12]));
#pragma unroll
        for (int k = 0; k < 12; k++) t[k] = o[k];
    }
    {   // step 3
        const uint32_t bi = a.v[3];
#pragma unroll
        for (int k = 0; k < 12; k++) e[k] = t[k];
        asm("mad.lo.cc.u32  %0, %9, %13, %0;\n\t"
            "madc.hi.cc.u32 %1, %9, %13, %1;\n\t"
            "madc.lo.cc.u32 %2, %10, %13, %2;\n\t"
            "madc.hi.cc.u32 %3, %10, %13, %3;\n\t"
            "madc.lo.cc.u32 %4, %11, %13, %4;\n\t"
            "madc.hi.cc.u32 %5, %11, %13, %5;\n\t"
            "madc.lo.cc.u32 %6, %12, %13, %6;\n\t"
            "madc.hi.cc.u32 %7, %12, %13, %7;\n\t"
            "addc.u32       %8, 0, 0;"
            : "+r"(e[4]), "+r"(e[5]), "+r"(e[6]), "+r"(e[7]), "+r"(e[8]), "+r"(e[9]), "+r"(e[10]), "+r"(e[11]), "=r"(e[12])
            : "r"((a.v[4] << 1)), "r"(d[6]), "r"(d[8]), "r"(d[10]), "r"(bi));
#pragma unroll
        for (int k = 0; k < 13; k++) o[k] = 0;
        o[2] = a.v[3] * bi;
        o[3] = __umulhi(a.v[3], bi);
        o[4] = d[5] * bi;
        o[5] = __umulhi(d[5], bi);
        o[6] = d[7] * bi;
        o[7] = __umulhi(d[7], bi);
        o[8] = d[9] * bi;
        o[9] = __umulhi(d[9], bi);
        o[10] = d[11] * bi;
        o[11] = __umulhi(d[11], bi);
        const uint32_t m = e[0] * CATMSM_N0;
        asm("mad.lo.cc.u32  %0, %13, %14, %0;\n\t"
            "madc.hi.cc.u32 %1, %13, %14, %1;\n\t"
            "madc.lo.cc.u32 %2, %13, %15, %2;\n\t"
            "madc.hi.cc.u32 %3, %13, %15, %3;\n\t"
            "madc.lo.cc.u32 %4, %13, %16, %4;\n\t"
            "madc.hi.cc.u32 %5, %13, %16, %5;\n\t"
            "madc.lo.cc.u32 %6, %13, %17, %6;\n\t"
            "madc.hi.cc.u32 %7, %13, %17, %7;\n\t"
            "madc.lo.cc.u32 %8, %13, %18, %8;\n\t"
            "madc.hi.cc.u32 %9, %13, %18, %9;\n\t"
            "madc.lo.cc.u32 %10, %13, %19, %10;\n\t"
            "madc.hi.cc.u32 %11, %13, %19, %11;\n\t"
            "addc.u32       %12, %12, 0;"
            : "+r"(e[0]), "+r"(e[1]), "+r"(e[2]), "+r"(e[3]), "+r"(e[4]), "+r"(e[5]),
              "+r"(e[6]), "+r"(e[7]), "+r"(e[8]), "+r"(e[9]), "+r"(e[10]), "+r"(e[11]),
              "+r"(e[12])
            : "r"(m), "n"(CATMSM_P0), "n"(CATMSM_P2), "n"(CATMSM_P4), "n"(CATMSM_P6),
              "n"(CATMSM_P8), "n"(CATMSM_P10));
        asm("mad.lo.cc.u32  %0, %13, %14, %0;\n\t"
            "madc.hi.cc.u32 %1, %13, %14, %1;\n\t"
            "madc.lo.cc.u32 %2, %13, %15, %2;\n\t"
            "madc.hi.cc.u32 %3, %13, %15, %3;\n\t"
            "madc.lo.cc.u32 %4, %13, %16, %4;\n\t"
            "madc.hi.cc.u32 %5, %13, %16, %5;\n\t"
            "madc.lo.cc.u32 %6, %13, %17, %6;\n\t"
            "madc.hi.cc.u32 %7, %13, %17, %7;\n\t"
            "madc.lo.cc.u32 %8, %13, %18, %8;\n\t"
            "madc.hi.cc.u32 %9, %13, %18, %9;\n\t"
            "madc.lo.cc.u32 %10, %13, %19, %10;\n\t"
            "madc.hi.cc.u32 %11, %13, %19, %11;\n\t"
            "addc.u32       %12, 0, 0;"
            : "+r"(o[0]), "+r"(o[1]), "+r"(o[2]), "+r"(o[3]), "+r"(o[4]), "+r"(o[5]),
              "+r"(o[6]), "+r"(o[7]), "+r"(o[8]), "+r"(o[9]), "+r"(o[10]), "+r"(o[11]),
              "=r"(o[12])
            : "r"(m), "n"(CATMSM_P1), "n"(CATMSM_P3), "n"(CATMSM_P5), "n"(CATMSM_P7),
              "n"(CATMSM_P9), "n"(CATMSM_P11));
        asm("add.cc.u32  %0, %0, %12;\n\t"
            "addc.cc.u32 %1, %1, %13;\n\t"
            "addc.cc.u32 %2, %2, %14;\n\t"
            "addc.cc.u32 %3, %3, %15;\n\t"
            "addc.cc.u32 %4, %4, %16;\n\t"
            "addc.cc.u32 %5, %5, %17;\n\t"
            "addc.cc.u32 %6, %6, %18;\n\t"
            "addc.cc.u32 %7, %7, %19;\n\t"
            "addc.cc.u32 %8, %8, %20;\n\t"
            "addc.cc.u32 %9, %9, %21;\n\t"
            "addc.cc.u32 %10, %10, %22;\n\t"
            "addc.u32    %11, %11, %23;"
            : "+r"(o[0]), "+r"(o[1]), "+r"(o[2]), "+r"(o[3]), "+r"(o[4]), "+r"(o[5]),
              "+r"(o[6]), "+r"(o[7]), "+r"(o[8]), "+r"(o[9]), "+r"(o[10]), "+r"(o[11])
            : "r"(e[1]), "r"(e[2]), "r"(e[3]), "r"(e[4]), "r"(e[5]), "r"(e[6]),
              "r"(e[7]), "r"(e[8]), "r"(e[9]), "r"(e[10]), "r"(e[11]), "r"(e[12]));
#pragma unroll
        for (int k = 0; k < 12; k++) t[k] = o[k];
    }
    {   // step 4
        const uint32_t bi = a.v[4];
#pragma unroll
        for (int k = 0; k < 12; k++) e[k] = t[k];
        asm("mad.lo.cc.u32  %0, %9, %13, %0;\n\t"
            "madc.hi.cc.u32 %1, %9, %13, %1;\n\t"
            "madc.lo.cc.u32 %2, %10, %13, %2;\n\t"
            "madc.hi.cc.u32 %3, %10, %13, %3;\n\t"
            "madc.lo.cc.u32 %4, %11, %13, %4;\n\t"
            "madc.hi.cc.u32 %5, %11, %13, %5;\n\t"
            "madc.lo.cc.u32 %6, %12, %13, %6;\n\t"
            "madc.hi.cc.u32 %7, %12, %13, %7;\n\t"
            "addc.u32       %8, 0, 0;"
            : "+r"(e[4]), "+r"(e[5]), "+r"(e[6]), "+r"(e[7]), "+r"(e[8]), "+r"(e[9]), "+r"(e[10]), "+r"(e[11]), "=r"(e[12])
            : "r"(a.v[4]), "r"(d[6]), "r"(d[8]), "r"(d[10]), "r"(bi));
#pragma unroll
        for (int k = 0; k < 13; k++) o[k] = 0;
        o[4] = (a.v[5] << 1) * bi;
        o[5] = __umulhi((a.v[5] << 1), bi);
        o[6] = d[7] * bi;
        o[7] = __umulhi(d[7], bi);
        o[8] = d[9] * bi;
        o[9] = __umulhi(d[9], bi);
        o[10] = d[11] * bi;
        o[11] = __umulhi(d[11], bi);
        const uint32_t m = e[0] * CATMSM_N0;
        asm("mad.lo.cc.u32  %0, %13, %14, %0;\n\t"
            "madc.hi.cc.u32 %1, %13, %14, %1;\n\t"
            "madc.lo.cc.u32 %2, %13, %15, %2;\n\t"
            "madc.hi.cc.u32 %3, %13, %15, %3;\n\t"
            "madc.lo.cc.u32 %4, %13, %16, %4;\n\t"
            "madc.hi.cc.u32 %5, %13, %16, %5;\n\t"
            "madc.lo.cc.u32 %6, %13, %17, %6;\n\t"
            "madc.hi.cc.u32 %7, %13, %17, %7;\n\t"
            "madc.lo.cc.u32 %8, %13, %18, %8;\n\t"
            "madc.hi.cc.u32 %9, %13, %18, %9;\n\t"
            "madc.lo.cc.u32 %10, %13, %19, %10;\n\t"
            "madc.hi.cc.u32 %11, %13, %19, %11;\n\t"
            "addc.u32       %12, %12, 0;"
            : "+r"(e[0]), "+r"(e[1]), "+r"(e[2]), "+r"(e[3]), "+r"(e[4]), "+r"(e[5]),
              "+r"(e[6]), "+r"(e[7]), "+r"(e[8]), "+r"(e[9]), "+r"(e[10]), "+r"(e[11]),
              "+r"(e[12])
            : "r"(m), "n"(CATMSM_P0), "n"(CATMSM_P2), "n"(CATMSM_P4), "n"(CATMSM_P6),
              "n"(CATMSM_P8), "n"(CATMSM_P10));
        asm("mad.lo.cc.u32  %0, %13, %14, %0;\n\t"
            "madc.hi.cc.u32 %1, %13, %14, %1;\n\t"
            "madc.lo.cc.u32 %2, %13, %15, %2;\n\t"
            "madc.hi.cc.u32 %3, %13, %15, %3;\n\t"
            "madc.lo.cc.u32 %4, %13, %16, %4;\n\t"
            "madc.hi.cc.u32 %5, %13, %16, %5;\n\t"
            "madc.lo.cc.u32 %6, %13, %17, %6;\n\t"
            "madc.hi.cc.u32 %7, %13, %17, %7;\n\t"
            "madc.lo.cc.u32 %8, %13, %18, %8;\n\t"
            "madc.hi.cc.u32 %9, %13, %18, %9;\n\t"
            "madc.lo.cc.u32 %10, %13, %19, %10;\n\t"
            "madc.hi.cc.u32 %11, %13, %19, %11;\n\t"
            "addc.u32       %12, 0, 0;"
            : "+r"(o[0]), "+r"(o[1]), "+r"(o[2]), "+r"(o[3]), "+r"(o[4]), "+r"(o[5]),
              "+r"(o[6]), "+r"(o[7]), "+r"(o[8]), "+r"(o[9]), "+r"(o[10]), "+r"(o[11]),
              "=r"(o[12])
            : "r"(m), "n"(CATMSM_P1), "n"(CATMSM_P3), "n"(CATMSM_P5), "n"(CATMSM_P7),
              "n"(CATMSM_P9), "n"(CATMSM_P11));
        asm("add.cc.u32  %0, %0, %12;\n\t"
            "addc.cc.u32 %1, %1, %13;\n\t"
            "addc.cc.u32 %2, %2, %14;\n\t"
            "addc.cc.u32 %3, %3, %15;\n\t"
            "addc.cc.u32 %4, %4, %16;\n\t"
            "addc.cc.u32 %5, %5, %17;\n\t"
            "addc.cc.u32 %6, %6, %18;\n\t"
            "addc.cc.u32 %7, %7, %19;\n\t"
            "addc.cc.u32 %8, %8, %20;\n\t"
            "addc.cc.u32 %9, %9, %21;\n\t"
            "addc.cc.u32 %10, %10, %22;\n\t"
            "addc.u32    %11, %11, %23;"
            : "+r"(o[0]), "+r"(o[1]), "+r"(o[2]), "+r"(o[3]), "+r"(o[4]), "+r"(o[5]),
              "+r"(o[6]), "+r"(o[7]), "+r"(o[8]), "+r"(o[9]), "+r"(o[10]), "+r"(o[11])
            : "r"(e[1]), "r"(e[2]), "r"(e[3]), "r"(e[4]), "r"(e[5]), "r"(e[6]),
              "r"(e[7]), "r"(e[8]), "r"(e[9]), "r"(e[10]), "r"(e[11]), "r"(e[12]));
#pragma unroll
        for (int k = 0; k < 12; k++) t[k] = o[k];
    }
    {   // step 5
        const uint32_t bi = a.v[5];
#pragma unroll
        for (int k = 0; k < 12; k++) e[k] = t[k];
        asm("mad.lo.cc.u32  %0, %7, %10, %0;\n\t"
            "madc.hi.cc.u32 %1, %7, %10, %1;\n\t"
            "madc.lo.cc.u32 %2, %8, %10, %2;\n\t"
            "madc.hi.cc.u32 %3, %8, %10, %3;\n\t"
            "madc.lo.cc.u32 %4, %9, %10, %4;\n\t"
            "madc.hi.cc.u32 %5, %9, %10, %5;\n\t"
            "addc.u32       %6, 0, 0;"
            : "+r"(e[6]), "+r"(e[7]), "+r"(e[8]), "+r"(e[9]), "+r"(e[10]), "+r"(e[11]), "=r"(e[12])
            : "r"((a.v[6] << 1)), "r"(d[8]), "r"(d[10]), "r"(bi));
#pragma unroll
        for (int k = 0; k < 13; k++) o[k] = 0;
        o[4] = a.v[5] * bi;
        o[5] = __umulhi(a.v[5], bi);
        o[6] = d[7] * bi;
        o[7] = __umulhi(d[7], bi);
        o[8] = d[9] * bi;
        o[9] = __umulhi(d[9], bi);
        o[10] = d[11] * bi;
        o[11] = __umulhi(d[11], bi);
        const uint32_t m = e[0] * CATMSM_N0;
        asm("mad.lo.cc.u32  %0, %13, %14, %0;\n\t"
            "madc.hi.cc.u32 %1, %13, %14, %1;\n\t"
            "madc.lo.cc.u32 %2, %13, %15, %2;\n\t"
            "madc.hi.cc.u32 %3, %13, %15, %3;\n\t"
            "madc.lo.cc.u32 %4, %13, %16, %4;\n\t"
            "madc.hi.cc.u32 %5, %13, %16, %5;\n\t"
            "madc.lo.cc.u32 %6, %13, %17, %6;\n\t"
            "madc.hi.cc.u32 %7, %13, %17, %7;\n\t"
            "madc.lo.cc.u32 %8, %13, %18, %8;\n\t"
            "madc.hi.cc.u32 %9, %13, %18, %9;\n\t"
            "madc.lo.cc.u32 %10, %13, %19, %10;\n\t"
            "madc.hi.cc.u32 %11, %13, %19, %11;\n\t"
            "addc.u32       %12, %12, 0;"
            : "+r"(e[0]), "+r"(e[1]), "+r"(e[2]), "+r"(e[3]), "+r"(e[4]), "+r"(e[5]),
              "+r"(e[6]), "+r"(e[7]), "+r"(e[8]), "+r"(e[9]), "+r"(e[10]), "+r"(e[11]),
              "+r"(e[12])
            : "r"(m), "n"(CATMSM_P0), "n"(CATMSM_P2), "n"(CATMSM_P4), "n"(CATMSM_P6),
              "n"(CATMSM_P8), "n"(CATMSM_P10));
        asm("mad.lo.cc.u32  %0, %13, %14, %0;\n\t"
            "madc.hi.cc.u32 %1, %13, %14, %1;\n\t"
            "madc.lo.cc.u32 %2, %13, %15, %2;\n\t"
            "madc.hi.cc.u32 %3, %13, %15, %3;\n\t"
            "madc.lo.cc.u32 %4, %13, %16, %4;\n\t"
            "madc.hi.cc.u32 %5, %13, %16, %5;\n\t"
            "madc.lo.cc.u32 %6, %13, %17, %6;\n\t"
            "madc.hi.cc.u32 %7, %13, %17, %7;\n\t"
            "madc.lo.cc.u32 %8, %13, %18, %8;\n\t"
            "madc.hi.cc.u32 %9, %13, %18, %9;\n\t"
            "madc.lo.cc.u32 %10, %13, %19, %10;\n\t"
            "madc.hi.cc.u32 %11, %13, %19, %11;\n\t"
            "addc.u32       %12, 0, 0;"
            : "+r"(o[0]), "+r"(o[1]), "+r"(o[2]), "+r"(o[3]), "+r"(o[4]), "+r"(o[5]),
              "+r"(o[6]), "+r"(o[7]), "+r"(o[8]), "+r"(o[9]), "+r"(o[10]), "+r"(o[11]),
              "=r"(o[12])
            : "r"(m), "n"(CATMSM_P1), "n"(CATMSM_P3), "n"(CATMSM_P5), "n"(CATMSM_P7),
              "n"(CATMSM_P9), "n"(CATMSM_P11));
        asm("add.cc.u32  %0, %0, %12;\n\t"
            "addc.cc.u32 %1, %1, %13;\n\t"
            "addc.cc.u32 %2, %2, %14;\n\t"
            "addc.cc.u32 %3, %3, %15;\n\t"
            "addc.cc.u32 %4, %4, %16;\n\t"
            "addc.cc.u32 %5, %5, %17;\n\t"
            "addc.cc.u32 %6, %6, %18;\n\t"
            "addc.cc.u32 %7, %7, %19;\n\t"
            "addc.cc.u32 %8, %8, %20;\n\t"
            "addc.cc.u32 %9, %9, %21;\n\t"
            "addc.cc.u32 %10, %10, %22;\n\t"
            "addc.u32    %11, %11, %23;"
            : "+r"(o[0]), "+r"(o[1]), "+r"(o[2]), "+r"(o[3]), "+r"(o[4]), "+r"(o[5]),
              "+r"(o[6]), "+r"(o[7]), "+r"(o[8]), "+r"(o[9]), "+r"(o[10]), "+r"(o[11])
            : "r"(e[1]), "r"(e[2]), "r"(e[3]), "r"(e[4]), "r"(e[5]), "r"(e[6]),
              "r"(e[7]), "r"(e[8]), "r"(e[9]), "r"(e[10]), "r"(e[11]), "r"(e[12]));
#pragma unroll
        for (int k = 0; k < 12; k++) t[k] = o[k];
    }
    {   // step 6
        const uint32_t bi = a.v[6];
#pragma unroll
        for (int k = 0; k < 12; k++) e[k] = t[k];
        asm("mad.lo.cc.u32  %0, %7, %10, %0;\n\t"
            "madc.hi.cc.u32 %1, %7, %10, %1;\n\t"
            "madc.lo.cc.u32 %2, %8, %10, %2;\n\t"
            "madc.hi.cc.u32 %3, %8, %10, %3;\n\t"
            "madc.lo.cc.u32 %4, %9, %10, %4;\n\t"
            "madc.hi.cc.u32 %5, %9, %10, %5;\n\t"
            "addc.u32       %6, 0, 0;"
            : "+r"(e[6]), "+r"(e[7]), "+r"(e[8]), "+r"(e[9]), "+r"(e[10]), "+r"(e[11]), "=r"(e[12])
            : "r"(a.v[6]), "r"(d[8]), "r"(d[10]), "r"(bi));
#pragma unroll
        for (int k = 0; k < 13; k++) o[k] = 0;
        o[6] = (a.v[7] << 1) * bi;
        o[7] = __umulhi((a.v[7] << 1), bi);
        o[8] = d[9] * bi;
        o[9] = __umulhi(d[9], bi);
        o[10] = d[11] * bi;
        o[11] = __umulhi(d[11], bi);
        const uint32_t m = e[0] * CATMSM_N0;
        asm("mad.lo.cc.u32  %0, %13, %14, %0;\n\t"
            "madc.hi.cc.u32 %1, %13, %14, %1;\n\t"
            "madc.lo.cc.u32 %2, %13, %15, %2;\n\t"
            "madc.hi.cc.u32 %3, %13, %15, %3;\n\t"
            "madc.lo.cc.u32 %4, %13, %16, %4;\n\t"
            "madc.hi.cc.u32 %5, %13, %16, %5;\n\t"
            "madc.lo.cc.u32 %6, %13, %17, %6;\n\t"
            "madc.hi.cc.u32 %7, %13, %17, %7;\n\t"
            "madc.lo.cc.u32 %8, %13, %18, %8;\n\t"
            "madc.hi.cc.u32 %9, %13, %18, %9;\n\t"
            "madc.lo.cc.u32 %10, %13, %19, %10;\n\t"
            "madc.hi.cc.u32 %11, %13, %19, %11;\n\t"
            "addc.u32       %12, %12, 0;"
            : "+r"(e[0]), "+r"(e[1]), "+r"(e[2]), "+r"(e[3]), "+r"(e[4]), "+r"(e[5]),
              "+r"(e[6]), "+r"(e[7]), "+r"(e[8]), "+r"(e[9]), "+r"(e[10]), "+r"(e[11]),
              "+r"(e[12])
            : "r"(m), "n"(CATMSM_P0), "n"(CATMSM_P2), "n"(CATMSM_P4), "n"(CATMSM_P6),
              "n"(CATMSM_P8), "n"(CATMSM_P10));
        asm("mad.lo.cc.u32  %0, %13, %14, %0;\n\t"
            "madc.hi.cc.u32 %1, %13, %14, %1;\n\t"
            "madc.lo.cc.u32 %2, %13, %15, %2;\n\t"
            "madc.hi.cc.u32 %3, %13, %15, %3;\n\t"
            "madc.lo.cc.u32 %4, %13, %16, %4;\n\t"
            "madc.hi.cc.u32 %5, %13, %16, %5;\n\t"
            "madc.lo.cc.u32 %6, %13, %17, %6;\n\t"
            "madc.hi.cc.u32 %7, %13, %17, %7;\n\t"
            "madc.lo.cc.u32 %8, %13, %18, %8;\n\t"
            "madc.hi.cc.u32 %9, %13, %18, %9;\n\t"
            "madc.lo.cc.u32 %10, %13, %19, %10;\n\t"
            "madc.hi.cc.u32 %11, %13, %19, %11;\n\t"
            "addc.u32       %12, 0, 0;"
            : "+r"(o[0]), "+r"(o[1]), "+r"(o[2]), "+r"(o[3]), "+r"(o[4]), "+r"(o[5]),
              "+r"(o[6]), "+r"(o[7]), "+r"(o[8]), "+r"(o[9]), "+r"(o[10]), "+r"(o[11]),
              "=r"(o[12])
            : "r"(m), "n"(CATMSM_P1), "n"(CATMSM_P3), "n"(CATMSM_P5), "n"(CATMSM_P7),
              "n"(CATMSM_P9), "n"(CATMSM_P11));
        asm("add.cc.u32  %0, %0, %12;\n\t"
            "addc.cc.u32 %1, %1, %13;\n\t"
            "addc.cc.u32 %2, %2, %14;\n\t"
            "addc.cc.u32 %3, %3, %15;\n\t"
            "addc.cc.u32 %4, %4, %16;\n\t"
            "addc.cc.u32 %5, %5, %17;\n\t"
            "addc.cc.u32 %6, %6, %18;\n\t"
            "addc.cc.u32 %7, %7, %19;\n\t"
            "addc.cc.u32 %8, %8, %20;\n\t"
            "addc.cc.u32 %9, %9, %21;\n\t"
            "addc.cc.u32 %10, %10, %22;\n\t"
            "addc.u32    %11, %11, %23;"
            : "+r"(o[0]), "+r"(o[1]), "+r"(o[2]), "+r"(o[3]), "+r"(o[4]), "+r"(o[5]),
              "+r"(o[6]), "+r"(o[7]), "+r"(o[8]), "+r"(o[9]), "+r"(o[10]), "+r"(o[11])
            : "r"(e[1]), "r"(e[2]), "r"(e[3]), "r"(e[4]), "r"(e[5]), "r"(e[6]),
              "r"(e[7]), "r"(e[8]), "r"(e[9]), "r"(e[10]), "r"(e[11]), "r"(e[12]));
#pragma unroll
        for (int k = 0; k < 12; k++) t[k] = o[k];
    }
    {   // step 7
        const uint32_t bi = a.v[7];
#pragma unroll
        for (int k = 0; k < 12; k++) e[k] = t[k];
        asm("mad.lo.cc.u32  %0, %5, %7, %0;\n\t"
            "madc.hi.cc.u32 %1, %5, %7, %1;\n\t"
            "madc.lo.cc.u32 %2, %6, %7, %2;\n\t"
            "madc.hi.cc.u32 %3, %6, %7, %3;\n\t"
            "addc.u32       %4, 0, 0;"
            : "+r"(e[8]), "+r"(e[9]), "+r"(e[10]), "+r"(e[11]), "=r"(e[12])
            : "r"((a.v[8] << 1)), "r"(d[10]), "r"(bi));
#pragma unroll
        for (int k = 0; k < 13; k++) o[k] = 0;
        o[6] = a.v[7] * bi;
        o[7] = __umulhi(a.v[7], bi);
        o[8] = d[9] * bi;
        o[9] = __umulhi(d[9], bi);
        o[10] = d[11] * bi;
        o[11] = __umulhi(d[11], bi);
        const uint32_t m = e[0] * CATMSM_N0;
        asm("mad.lo.cc.u32  %0, %13, %14, %0;\n\t"
            "madc.hi.cc.u32 %1, %13, %14, %1;\n\t"
            "madc.lo.cc.u32 %2, %13, %15, %2;\n\t"
            "madc.hi.cc.u32 %3, %13, %15, %3;\n\t"
            "madc.lo.cc.u32 %4, %13, %16, %4;\n\t"
            "madc.hi.cc.u32 %5, %13, %16, %5;\n\t"
            "madc.lo.cc.u32 %6, %13, %17, %6;\n\t"
            "madc.hi.cc.u32 %7, %13, %17, %7;\n\t"
            "madc.lo.cc.u32 %8, %13, %18, %8;\n\t"
            "madc.hi.cc.u32 %9, %13, %18, %9;\n\t"
            "madc.lo.cc.u32 %10, %13, %19, %10;\n\t"
            "madc.hi.cc.u32 %11, %13, %19, %11;\n\t"
            "addc.u32       %12, %12, 0;"
            : "+r"(e[0]), "+r"(e[1]), "+r"(e[2]), "+r"(e[3]), "+r"(e[4]), "+r"(e[5]),
              "+r"(e[6]), "+r"(e[7]), "+r"(e[8]), "+r"(e[9]), "+r"(e[10]), "+r"(e[11]),
              "+r"(e[12])
            : "r"(m), "n"(CATMSM_P0), "n"(CATMSM_P2), "n"(CATMSM_P4), "n"(CATMSM_P6),
              "n"(CATMSM_P8), "n"(CATMSM_P10));
        asm("mad.lo.cc.u32  %0, %13, %14, %0;\n\t"
            "madc.hi.cc.u32 %1, %13, %14, %1;\n\t"
            "madc.lo.cc.u32 %2, %13, %15, %2;\n\t"
            "madc.hi.cc.u32 %3, %13, %15, %3;\n\t"
            "madc.lo.cc.u32 %4, %13, %16, %4;\n\t"
            "madc.hi.cc.u32 %5, %13, %16, %5;\n\t"
            "madc.lo.cc.u32 %6, %13, %17, %6;\n\t"
            "madc.hi.cc.u32 %7, %13, %17, %7;\n\t"
            "madc.lo.cc.u32 %8, %13, %18, %8;\n\t"
            "madc.hi.cc.u32 %9, %13, %18, %9;\n\t"
            "madc.lo.cc.u32 %10, %13, %19, %10;\n\t"
            "madc.hi.cc.u32 %11, %13, %19, %11;\n\t"
            "addc.u32       %12, 0, 0;"
            : "+r"(o[0]), "+r"(o[1]), "+r"(o[2]), "+r"(o[3]), "+r"(o[4]), "+r"(o[5]),
              "+r"(o[6]), "+r"(o[7]), "+r"(o[8]), "+r"(o[9]), "+r"(o[10]), "+r"(o[11]),
              "=r"(o[12])
            : "r"(m), "n"(CATMSM_P1), "n"(CATMSM_P3), "n"(CATMSM_P5), "n"(CATMSM_P7),
              "n"(CATMSM_P9), "n"(CATMSM_P11));
        asm("add.cc.u32  %0, %0, %12;\n\t"
            "addc.cc.u32 %1, %1, %13;\n\t"
            "addc.cc.u32 %2, %2, %14;\n\t"
            "addc.cc.u32 %3, %3, %15;\n\t"
            "addc.cc.u32 %4, %4, %16;\n\t"
            "addc.cc.u32 %5, %5, %17;\n\t"
            "addc.cc.u32 %6, %6, %18;\n\t"
            "addc.cc.u32 %7, %7, %19;\n\t"
            "addc.cc.u32 %8, %8, %20;\n\t"
            "addc.cc.u32 %9, %9, %21;\n\t"
            "addc.cc.u32 %10, %10, %22;\n\t"
            "addc.u32    %11, %11, %23;"
            : "+r"(o[0]), "+r"(o[1]), "+r"(o[2]), "+r"(o[3]), "+r"(o[4]), "+r"(o[5]),
              "+r"(o[6]), "+r"(o[7]), "+r"(o[8]), "+r"(o[9]), "+r"(o[10]), "+r"(o[11])
            : "r"(e[1]), "r"(e[2]), "r"(e[3]), "r"(e[4]), "r"(e[5]), "r"(e[6]),
              "r"(e[7]), "r"(e[8]), "r"(e[9]), "r"(e[10]), "r"(e[11]), "r"(e[12]));
#pragma unroll
        for (int k = 0; k < 12; k++) t[k] = o[k];
    }
    {   // step 8
        const uint32_t bi = a.v[8];
#pragma unroll
        for (int k = 0; k < 12; k++) e[k] = t[k];
        asm("mad.lo.cc.u32  %0, %5, %7, %0;\n\t"
            "madc.hi.cc.u32 %1, %5, %7, %1;\n\t"
            "madc.lo.cc.u32 %2, %6, %7, %2;\n\t"
            "madc.hi.cc.u32 %3, %6, %7, %3;\n\t"
            "addc.u32       %4, 0, 0;"
            : "+r"(e[8]), "+r"(e[9]), "+r"(e[10]), "+r"(e[11]), "=r"(e[12])
            : "r"(a.v[8]), "r"(d[10]), "r"(bi));
#pragma unroll
        for (int k = 0; k < 13; k++) o[k] = 0;
        o[8] = (a.v[9] << 1) * bi;
        o[9] = __umulhi((a.v[9] << 1), bi);
        o[10] = d[11] * bi;
        o[11] = __umulhi(d[11], bi);
        const uint32_t m = e[0] * CATMSM_N0;
        asm("mad.lo.cc.u32  %0, %13, %14, %0;\n\t"
            "madc.hi.cc.u32 %1, %13, %14, %1;\n\t"
            "madc.lo.cc.u32 %2, %13, %15, %2;\n\t"
            "madc.hi.cc.u32 %3, %13, %15, %3;\n\t"
            "madc.lo.cc.u32 %4, %13, %16, %4;\n\t"
            "madc.hi.cc.u32 %5, %13, %16, %5;\n\t"
            "madc.lo.cc.u32 %6, %13, %17, %6;\n\t"
            "madc.hi.cc.u32 %7, %13, %17, %7;\n\t"
            "madc.lo.cc.u32 %8, %13, %18, %8;\n\t"
            "madc.hi.cc.u32 %9, %13, %18, %9;\n\t"
            "madc.lo.cc.u32 %10, %13, %19, %10;\n\t"
            "madc.hi.cc.u32 %11, %13, %19, %11;\n\t"
            "addc.u32       %12, %12, 0;"
            : "+r"(e[0]), "+r"(e[1]), "+r"(e[2]), "+r"(e[3]), "+r"(e[4]), "+r"(e[5]),
              "+r"(e[6]), "+r"(e[7]), "+r"(e[8]), "+r"(e[9]), "+r"(e[10]), "+r"(e[11]),
              "+r"(e[12])
            : "r"(m), "n"(CATMSM_P0), "n"(CATMSM_P2), "n"(CATMSM_P4), "n"(CATMSM_P6),
              "n"(CATMSM_P8), "n"(CATMSM_P10));
        asm("mad.lo.cc.u32  %0, %13, %14, %0;\n\t"
            "madc.hi.cc.u32 %1, %13, %14, %1;\n\t"
            "madc.lo.cc.u32 %2, %13, %15, %2;\n\t"
            "madc.hi.cc.u32 %3, %13, %15, %3;\n\t"
            "madc.lo.cc.u32 %4, %13, %16, %4;\n\t"
            "madc.hi.cc.u32 %5, %13, %16, %5;\n\t"
            "madc.lo.cc.u32 %6, %13, %17, %6;\n\t"
            "madc.hi.cc.u32 %7, %13, %17, %7;\n\t"
            "madc.lo.cc.u32 %8, %13, %18, %8;\n\t"
            "madc.hi.cc.u32 %9, %13, %18, %9;\n\t"
            "madc.lo.cc.u32 %10, %13, %19, %10;\n\t"
            "madc.hi.cc.u32 %11, %13, %19, %11;\n\t"
            "addc.u32       %12, 0, 0;"
            : "+r"(o[0]), "+r"(o[1]), "+r"(o[2]), "+r"(o[3]), "+r"(o[4]), "+r"(o[5]),
              "+r"(o[6]), "+r"(o[7]), "+r"(o[8]), "+r"(o[9]), "+r"(o[10]), "+r"(o[11]),
              "=r"(o[12])
            : "r"(m), "n"(CATMSM_P1), "n"(CATMSM_P3), "n"(CATMSM_P5), "n"(CATMSM_P7),
              "n"(CATMSM_P9), "n"(CATMSM_P11));
        asm("add.cc.u32  %0, %0, %12;\n\t"
            "addc.cc.u32 %1, %1, %13;\n\t"
            "addc.cc.u32 %2, %2, %14;\n\t"
            "addc.cc.u32 %3, %3, %15;\n\t"
            "addc.cc.u32 %4, %4, %16;\n\t"
            "addc.cc.u32 %5, %5, %17;\n\t"
            "addc.cc.u32 %6, %6, %18;\n\t"
            "addc.cc.u32 %7, %7, %19;\n\t"
            "addc.cc.u32 %8, %8, %20;\n\t"
            "addc.cc.u32 %9, %9, %21;\n\t"
            "addc.cc.u32 %10, %10, %22;\n\t"
            "addc.u32    %11, %11, %23;"
            : "+r"(o[0]), "+r"(o[1]), "+r"(o[2]), "+r"(o[3]), "+r"(o[4]), "+r"(o[5]),
              "+r"(o[6]), "+r"(o[7]), "+r"(o[8]), "+r"(o[9]), "+r"(o[10]), "+r"(o[11])
            : "r"(e[1]), "r"(e[2]), "r"(e[3]), "r"(e[4]), "r"(e[5]), "r"(e[6]),
              "r"(e[7]), "r"(e[8]), "r"(e[9]), "r"(e[10]), "r"(e[11]), "r"(e[12]));
#pragma unroll
        for (int k = 0; k < 12; k++) t[k] = o[k];
    }
    {   // step 9
        const uint32_t bi = a.v[9];
#pragma unroll
        for (int k = 0; k < 12; k++) e[k] = t[k];
        asm("mad.lo.cc.u32  %0, %3, %4, %0;\n\t"
            "madc.hi.cc.u32 %1, %3, %4, %1;\n\t"
            "addc.u32       %2, 0, 0;"
            : "+r"(e[10]), "+r"(e[11]), "=r"(e[12])
            : "r"((a.v[10] << 1)), "r"(bi));
#pragma unroll
        for (int k = 0; k < 13; k++) o[k] = 0;
        o[8] = a.v[9] * bi;
        o[9] = __umulhi(a.v[9], bi);
        o[10] = d[11] * bi;
        o[11] = __umulhi(d[11], bi);
        const uint32_t m = e[0] * CATMSM_N0;
        asm("mad.lo.cc.u32  %0, %13, %14, %0;\n\t"
            "madc.hi.cc.u32 %1, %13, %14, %1;\n\t"
            "madc.lo.cc.u32 %2, %13, %15, %2;\n\t"
            "madc.hi.cc.u32 %3, %13, %15, %3;\n\t"
            "madc.lo.cc.u32 %4, %13, %16, %4;\n\t"
            "madc.hi.cc.u32 %5, %13, %16, %5;\n\t"
            "madc.lo.cc.u32 %6, %13, %17, %6;\n\t"
            "madc.hi.cc.u32 %7, %13, %17, %7;\n\t"
            "madc.lo.cc.u32 %8, %13, %18, %8;\n\t"
            "madc.hi.cc.u32 %9, %13, %18, %9;\n\t"
            "madc.lo.cc.u32 %10, %13, %19, %10;\n\t"
            "madc.hi.cc.u32 %11, %13, %19, %11;\n\t"
            "addc.u32       %12, %12, 0;"
            : "+r"(e[0]), "+r"(e[1]), "+r"(e[2]), "+r"(e[3]), "+r"(e[4]), "+r"(e[5]),
              "+r"(e[6]), "+r"(e[7]), "+r"(e[8]), "+r"(e[9]), "+r"(e[10]), "+r"(e[11]),
              "+r"(e[12])
            : "r"(m), "n"(CATMSM_P0), "n"(CATMSM_P2), "n"(CATMSM_P4), "n"(CATMSM_P6),
              "n"(CATMSM_P8), "n"(CATMSM_P10));
        asm("mad.lo.cc.u32  %0, %13, %14, %0;\n\t"
            "madc.hi.cc.u32 %1, %13, %14, %1;\n\t"
            "madc.lo.cc.u32 %2, %13, %15, %2;\n\t"
            "madc.hi.cc.u32 %3, %13, %15, %3;\n\t"
            "madc.lo.cc.u32 %4, %13, %16, %4;\n\t"
            "madc.hi.cc.u32 %5, %13, %16, %5;\n\t"
            "madc.lo.cc.u32 %6, %13, %17, %6;\n\t"
            "madc.hi.cc.u32 %7, %13, %17, %7;\n\t"
            "madc.lo.cc.u32 %8, %13, %18, %8;\n\t"
            "madc.hi.cc.u32 %9, %13, %18, %9;\n\t"
            "madc.lo.cc.u32 %10, %13, %19, %10;\n\t"
            "madc.hi.cc.u32 %11, %13, %19, %11;\n\t"
            "addc.u32       %12, 0, 0;"
            : "+r"(o[0]), "+r"(o[1]), "+r"(o[2]), "+r"(o[3]), "+r"(o[4]), "+r"(o[5]),
              "+r"(o[6]), "+r"(o[7]), "+r"(o[8]), "+r"(o[9]), "+r"(o[10]), "+r"(o[11]),
              "=r"(o[12])
            : "r"(m), "n"(CATMSM_P1), "n"(CATMSM_P3), "n"(CATMSM_P5), "n"(CATMSM_P7),
              "n"(CATMSM_P9), "n"(CATMSM_P11));
        asm("add.cc.u32  %0, %0, %12;\n\t"
            "addc.cc.u32 %1, %1, %13;\n\t"
            "addc.cc.u32 %2, %2, %14;\n\t"
            "addc.cc.u32 %3, %3, %15;\n\t"
            "addc.cc.u32 %4, %4, %16;\n\t"
            "addc.cc.u32 %5, %5, %17;\n\t"
            "addc.cc.u32 %6, %6, %18;\n\t"
            "addc.cc.u32 %7, %7, %19;\n\t"
            "addc.cc.u32 %8, %8, %20;\n\t"
            "addc.cc.u32 %9, %9, %21;\n\t"
            "addc.cc.u32 %10, %10, %22;\n\t"
            "addc.u32    %11, %11, %23;"
            : "+r"(o[0]), "+r"(o[1]), "+r"(o[2]), "+r"(o[3]), "+r"(o[4]), "+r"(o[5]),
              "+r"(o[6]), "+r"(o[7]), "+r"(o[8]), "+r"(o[9]), "+r"(o[10]), "+r"(o[11])
            : "r"(e[1]), "r"(e[2]), "r"(e[3]), "r"(e[4]), "r"(e[5]), "r"(e[6]),
              "r"(e[7]), "r"(e[8]), "r"(e[9]), "r"(e[10]), "r"(e[11]), "r"(e[12]));
#pragma unroll
        for (int k = 0; k < 12; k++) t[k] = o[k];
    }
    {   // step 10
        const uint32_t bi = a.v[10];
#pragma unroll
        for (int k = 0; k < 12; k++) e[k] = t[k];
        asm("mad.lo.cc.u32  %0, %3, %4, %0;\n\t"
            "madc.hi.cc.u32 %1, %3, %4, %1;\n\t"
            "addc.u32       %2, 0, 0;"
            : "+r"(e[10]), "+r"(e[11]), "=r"(e[12])
            : "r"(a.v[10]), "r"(bi));
#pragma unroll
        for (int k = 0; k < 13; k++) o[k] = 0;
        o[10] = (a.v[11] << 1) * bi;
        o[11] = __umulhi((a.v[11] << 1), bi);
        const uint32_t m = e[0] * CATMSM_N0;
        asm("mad.lo.cc.u32  %0, %13, %14, %0;\n\t"
            "madc.hi.cc.u32 %1, %13, %14, %1;\n\t"
            "madc.lo.cc.u32 %2, %13, %15, %2;\n\t"
            "madc.hi.cc.u32 %3, %13, %15, %3;\n\t"
            "madc.lo.cc.u32 %4, %13, %16, %4;\n\t"
            "madc.hi.cc.u32 %5, %13, %16, %5;\n\t"
            "madc.lo.cc.u32 %6, %13, %17, %6;\n\t"
            "madc.hi.cc.u32 %7, %13, %17, %7;\n\t"
            "madc.lo.cc.u32 %8, %13, %18, %8;\n\t"
            "madc.hi.cc.u32 %9, %13, %18, %9;\n\t"
            "madc.lo.cc.u32 %10, %13, %19, %10;\n\t"
            "madc.hi.cc.u32 %11, %13, %19, %11;\n\t"
            "addc.u32       %12, %12, 0;"
            : "+r"(e[0]), "+r"(e[1]), "+r"(e[2]), "+r"(e[3]), "+r"(e[4]), "+r"(e[5]),
              "+r"(e[6]), "+r"(e[7]), "+r"(e[8]), "+r"(e[9]), "+r"(e[10]), "+r"(e[11]),
              "+r"(e[12])
            : "r"(m), "n"(CATMSM_P0), "n"(CATMSM_P2), "n"(CATMSM_P4), "n"(CATMSM_P6),
              "n"(CATMSM_P8), "n"(CATMSM_P10));
        asm("mad.lo.cc.u32  %0, %13, %14, %0;\n\t"
            "madc.hi.cc.u32 %1, %13, %14, %1;\n\t"
            "madc.lo.cc.u32 %2, %13, %15, %2;\n\t"
            "madc.hi.cc.u32 %3, %13, %15, %3;\n\t"
            "madc.lo.cc.u32 %4, %13, %16, %4;\n\t"
            "madc.hi.cc.u32 %5, %13, %16, %5;\n\t"
            "madc.lo.cc.u32 %6, %13, %17, %6;\n\t"
            "madc.hi.cc.u32 %7, %13, %17, %7;\n\t"
            "madc.lo.cc.u32 %8, %13, %18, %8;\n\t"
            "madc.hi.cc.u32 %9, %13, %18, %9;\n\t"
            "madc.lo.cc.u32 %10, %13, %19, %10;\n\t"
            "madc.hi.cc.u32 %11, %13, %19, %11;\n\t"
            "addc.u32       %12, 0, 0;"
            : "+r"(o[0]), "+r"(o[1]), "+r"(o[2]), "+r"(o[3]), "+r"(o[4]), "+r"(o[5]),
              "+r"(o[6]), "+r"(o[7]), "+r"(o[8]), "+r"(o[9]), "+r"(o[10]), "+r"(o[11]),
              "=r"(o[12])
            : "r"(m), "n"(CATMSM_P1), "n"(CATMSM_P3), "n"(CATMSM_P5), "n"(CATMSM_P7),
              "n"(CATMSM_P9), "n"(CATMSM_P11));
        asm("add.cc.u32  %0, %0, %12;\n\t"
            "addc.cc.u32 %1, %1, %13;\n\t"
            "addc.cc.u32 %2, %2, %14;\n\t"
            "addc.cc.u32 %3, %3, %15;\n\t"
            "addc.cc.u32 %4, %4, %16;\n\t"
            "addc.cc.u32 %5, %5, %17;\n\t"
            "addc.cc.u32 %6, %6, %18;\n\t"
            "addc.cc.u32 %7, %7, %19;\n\t"
            "addc.cc.u32 %8, %8, %20;\n\t"
            "addc.cc.u32 %9, %9, %21;\n\t"
            "addc.cc.u32 %10, %10, %22;\n\t"
            "addc.u32    %11, %11, %23;"
            : "+r"(o[0]), "+r"(o[1]), "+r"(o[2]), "+r"(o[3]), "+r"(o[4]), "+r"(o[5]),
              "+r"(o[6]), "+r"(o[7]), "+r"(o[8]), "+r"(o[9]), "+r"(o[10]), "+r"(o[11])
            : "r"(e[1]), "r"(e[2]), "r"(e[3]), "r"(e[4]), "r"(e[5]), "r"(e[6]),
              "r"(e[7]), "r"(e[8]), "r"(e[9]), "r"(e[10]), "r"(e[11]), "r"(e[12]));
#pragma unroll
        for (int k = 0; k < 12; k++) t[k] = o[k];
    }
    {   // step 11
        const uint32_t bi = a.v[11];
#pragma unroll
        for (int k = 0; k < 12; k++) e[k] = t[k];
        e[12] = 0;
#pragma unroll
        for (int k = 0; k < 13; k++) o[k] = 0;
        o[10] = a.v[11] * bi;
        o[11] = __umulhi(a.v[11], bi);
        const uint32_t m = e[0] * CATMSM_N0;
        asm("mad.lo.cc.u32  %0, %13, %14, %0;\n\t"
            "madc.hi.cc.u32 %1, %13, %14, %1;\n\t"
            "madc.lo.cc.u32 %2, %13, %15, %2;\n\t"
            "madc.hi.cc.u32 %3, %13, %15, %3;\n\t"
            "madc.lo.cc.u32 %4, %13, %16, %4;\n\t"
            "madc.hi.cc.u32 %5, %13, %16, %5;\n\t"
            "madc.lo.cc.u32 %6, %13, %17, %6;\n\t"
            "madc.hi.cc.u32 %7, %13, %17, %7;\n\t"
            "madc.lo.cc.u32 %8, %13, %18, %8;\n\t"
            "madc.hi.cc.u32 %9, %13, %18, %9;\n\t"
            "madc.lo.cc.u32 %10, %13, %19, %10;\n\t"
            "madc.hi.cc.u32 %11, %13, %19, %11;\n\t"
            "addc.u32       %12, %12, 0;"
            : "+r"(e[0]), "+r"(e[1]), "+r"(e[2]), "+r"(e[3]), "+r"(e[4]), "+r"(e[5]),
              "+r"(e[6]), "+r"(e[7]), "+r"(e[8]), "+r"(e[9]), "+r"(e[10]), "+r"(e[11]),
              "+r"(e[12])
            : "r"(m), "n"(CATMSM_P0), "n"(CATMSM_P2), "n"(CATMSM_P4), "n"(CATMSM_P6),
              "n"(CATMSM_P8), "n"(CATMSM_P10));
        asm("mad.lo.cc.u32  %0, %13, %14, %0;\n\t"
            "madc.hi.cc.u32 %1, %13, %14, %1;\n\t"
            "madc.lo.cc.u32 %2, %13, %15, %2;\n\t"
            "madc.hi.cc.u32 %3, %13, %15, %3;\n\t"
            "madc.lo.cc.u32 %4, %13, %16, %4;\n\t"
            "madc.hi.cc.u32 %5, %13, %16, %5;\n\t"
            "madc.lo.cc.u32 %6, %13, %17, %6;\n\t"
            "madc.hi.cc.u32 %7, %13, %17, %7;\n\t"
            "madc.lo.cc.u32 %8, %13, %18, %8;\n\t"
            "madc.hi.cc.u32 %9, %13, %18, %9;\n\t"
            "madc.lo.cc.u32 %10, %13, %19, %10;\n\t"
            "madc.hi.cc.u32 %11, %13, %19, %11;\n\t"
            "addc.u32       %12, 0, 0;"
            : "+r"(o[0]), "+r"(o[1]), "+r"(o[2]), "+r"(o[3]), "+r"(o[4]), "+r"(o[5]),
              "+r"(o[6]), "+r"(o[7]), "+r"(o[8]), "+r"(o[9]), "+r"(o[10]), "+r"(o[11]),
              "=r"(o[12])
            : "r"(m), "n"(CATMSM_P1), "n"(CATMSM_P3), "n"(CATMSM_P5), "n"(CATMSM_P7),
              "n"(CATMSM_P9), "n"(CATMSM_P11));
        asm("add.cc.u32  %0, %0, %12;\n\t"
            "addc.cc.u32 %1, %1, %13;\n\t"
            "addc.cc.u32 %2, %2, %14;\n\t"
            "addc.cc.u32 %3, %3, %15;\n\t"
            "addc.cc.u32 %4, %4, %16;\n\t"
            "addc.cc.u32 %5, %5, %17;\n\t"
            "addc.cc.u32 %6, %6, %18;\n\t"
            "addc.cc.u32 %7, %7, %19;\n\t"
            "addc.cc.u32 %8, %8, %20;\n\t"
            "addc.cc.u32 %9, %9, %21;\n\t"
            "addc.cc.u32 %10, %10, %22;\n\t"
            "addc.u32    %11, %11, %23;"
            : "+r"(o[0]), "+r"(o[1]), "+r"(o[2]), "+r"(o[3]), "+r"(o[4]), "+r"(o[5]),
              "+r"(o[6]), "+r"(o[7]), "+r"(o[8]), "+r"(o[9]), "+r"(o[10]), "+r"(o[11])
            : "r"(e[1]), "r"(e[2]), "r"(e[3]), "r"(e[4]), "r"(e[5]), "r"(e[6]),
              "r"(e[7]), "r"(e[8]), "r"(e[9]), "r"(e[10]), "r"(e[11]), "r"(e[12]));
#pragma unroll
        for (int k = 0; k < 12; k++) t[k] = o[k];
    }
#pragma unroll
    for (int k = 0; k < 12; k++) r.v[k] = t[k];
}

static __device__ __noinline__ fp fp_sqr_call(const fp a)
{
    fp r;
    fp_sqr_impl(r, a);
    return r;
}

__device__ __forceinline__ void fp_sqr(fp& r, const fp& a) { r = fp_sqr_call(a); }

// r = (a * b + c * d) * 2^-384 mod p; inputs in [0, 2p), output in [0, 2p).
// The CIOS schedule of fp_mul_impl with both products added in each step
// before its single Montgomery reduction (876 IMAD against 2 x 588).  Each
// step adds at most 4p 2^32, so the running value stays below 6p < 2^384,
// and a b + c d < 8p^2 < p 2^384 leaves the result below 1.82p.
__device__ __forceinline__ void fp_mul2_impl(fp& r, const fp& a, const fp& b, const fp& c, const fp& d)
{
    uint32_t t[12], e[13], o[13];
#pragma unroll
    for (int i = 0; i < 12; i++) {
        const uint32_t bi = b.v[i], di = d.v[i];
        if (i == 0) {
#pragma unroll
            for (int k = 0; k < 6; k++) {
                e[2 * k] = a.v[2 * k] * bi;
                e[2 * k + 1] = __umulhi(a.v[2 * k], bi);
            }
            e[12] = 0;
        } else {
#pragma unroll
            for (int k = 0; k < 12; k++) e[k] = t[k];
            asm("mad.lo.cc.u32  %0, %13, %14, %0;\n\t"
                "madc.hi.cc.u32 %1, %13, %14, %1;\n\t"
                "madc.lo.cc.u32 %2, %13, %15, %2;\n\t"
                "madc.hi.cc.u32 %3, %13, %15, %3;\n\t"
                "madc.lo.cc.u32 %4, %13, %16, %4;\n\t"
                "madc.hi.cc.u32 %5, %13, %16, %5;\n\t"
                "madc.lo.cc.u32 %6, %13, %17, %6;\n\t"
                "madc.hi.cc.u32 %7, %13, %17, %7;\n\t"
                "madc.lo.cc.u32 %8, %13, %18, %8;\n\t"
                "madc.hi.cc.u32 %9, %13, %18, %9;\n\t"
                "madc.lo.cc.u32 %10, %13, %19, %10;\n\t"
                "madc.hi.cc.u32 %11, %13, %19, %11;\n\t"
                "addc.u32       %12, 0, 0;"
                : "+r"(e[0]), "+r"(e[1]), "+r"(e[2]), "+r"(e[3]), "+r"(e[4]), "+r"(e[5]), "+r"(e[6]), "+r"(e[7]), "+r"(e[8]), "+r"(e[9]), "+r"(e[10]), "+r"(e[11]), "=r"(e[12])
                : "r"(bi), "r"(a.v[0]), "r"(a.v[2]), "r"(a.v[4]), "r"(a.v[6]), "r"(a.v[8]), "r"(a.v[10]));
        }
        asm("mad.lo.cc.u32  %0, %13, %14, %0;\n\t"
            "madc.hi.cc.u32 %1, %13, %14, %1;\n\t"
            "madc.lo.cc.u32 %2, %13, %15, %2;\n\t"
            "madc.hi.cc.u32 %3, %13, %15, %3;\n\t"
            "madc.lo.cc.u32 %4, %13, %16, %4;\n\t"
            "madc.hi.cc.u32 %5, %13, %16, %5;\n\t"
            "madc.lo.cc.u32 %6, %13, %17, %6;\n\t"
            "madc.hi.cc.u32 %7, %13, %17, %7;\n\t"
            "madc.lo.cc.u32 %8, %13, %18, %8;\n\t"
            "madc.hi.cc.u32 %9, %13, %18, %9;\n\t"
            "madc.lo.cc.u32 %10, %13, %19, %10;\n\t"
            "madc.hi.cc.u32 %11, %13, %19, %11;\n\t"
            "addc.u32       %12, %12, 0;"
            : "+r"(e[0]), "+r"(e[1]), "+r"(e[2]), "+r"(e[3]), "+r"(e[4]), "+r"(e[5]), "+r"(e[6]), "+r"(e[7]), "+r"(e[8]), "+r"(e[9]), "+r"(e[10]), "+r"(e[11]), "+r"(e[12])
            : "r"(di), "r"(c.v[0]), "r"(c.v[2]), "r"(c.v[4]), "r"(c.v[6]), "r"(c.v[8]), "r"(c.v[10]));
#pragma unroll
        for (int k = 0; k < 6; k++) {
            o[2 * k] = a.v[2 * k + 1] * bi;
            o[2 * k + 1] = __umulhi(a.v[2 * k + 1], bi);
        }
        asm("mad.lo.cc.u32  %0, %13, %14, %0;\n\t"
            "madc.hi.cc.u32 %1, %13, %14, %1;\n\t"
            "madc.lo.cc.u32 %2, %13, %15, %2;\n\t"
            "madc.hi.cc.u32 %3, %13, %15, %3;\n\t"
            "madc.lo.cc.u32 %4, %13, %16, %4;\n\t"
            "madc.hi.cc.u32 %5, %13, %16, %5;\n\t"
            "madc.lo.cc.u32 %6, %13, %17, %6;\n\t"
            "madc.hi.cc.u32 %7, %13, %17, %7;\n\t"
            "madc.lo.cc.u32 %8, %13, %18, %8;\n\t"
            "madc.hi.cc.u32 %9, %13, %18, %9;\n\t"
            "madc.lo.cc.u32 %10, %13, %19, %10;\n\t"
            "madc.hi.cc.u32 %11, %13, %19, %11;\n\t"
            "addc.u32       %12, 0, 0;"
            : "+r"(o[0]), "+r"(o[1]), "+r"(o[2]), "+r"(o[3]), "+r"(o[4]), "+r"(o[5]), "+r"(o[6]), "+r"(o[7]), "+r"(o[8]), "+r"(o[9]), "+r"(o[10]), "+r"(o[11]), "=r"(o[12])
            : "r"(di), "r"(c.v[1]), "r"(c.v[3]), "r"(c.v[5]), "r"(c.v[7]), "r"(c.v[9]), "r"(c.v[11]));
        const uint32_t m = e[0] * CATMSM_N0;
        asm("mad.lo.cc.u32  %0, %13, %14, %0;\n\t"
            "madc.hi.cc.u32 %1, %13, %14, %1;\n\t"
            "madc.lo.cc.u32 %2, %13, %15, %2;\n\t"
            "madc.hi.cc.u32 %3, %13, %15, %3;\n\t"
            "madc.lo.cc.u32 %4, %13, %16, %4;\n\t"
            "madc.hi.cc.u32 %5, %13, %16, %5;\n\t"
            "madc.lo.cc.u32 %6, %13, %17, %6;\n\t"
            "madc.hi.cc.u32 %7, %13, %17, %7;\n\t"
            "madc.lo.cc.u32 %8, %13, %18, %8;\n\t"
            "madc.hi.cc.u32 %9, %13, %18, %9;\n\t"
            "madc.lo.cc.u32 %10, %13, %19, %10;\n\t"
            "madc.hi.cc.u32 %11, %13, %19, %11;\n\t"
            "addc.u32       %12, %12, 0;"
            : "+r"(e[0]), "+r"(e[1]), "+r"(e[2]), "+r"(e[3]), "+r"(e[4]), "+r"(e[5]), "+r"(e[6]), "+r"(e[7]), "+r"(e[8]), "+r"(e[9]), "+r"(e[10]), "+r"(e[11]), "+r"(e[12])
            : "r"(m), "n"(CATMSM_P0), "n"(CATMSM_P2), "n"(CATMSM_P4), "n"(CATMSM_P6), "n"(CATMSM_P8), "n"(CATMSM_P10));
        asm("mad.lo.cc.u32  %0, %13, %14, %0;\n\t"
            "madc.hi.cc.u32 %1, %13, %14, %1;\n\t"
            "madc.lo.cc.u32 %2, %13, %15, %2;\n\t"
            "madc.hi.cc.u32 %3, %13, %15, %3;\n\t"
            "madc.lo.cc.u32 %4, %13, %16, %4;\n\t"
            "madc.hi.cc.u32 %5, %13, %16, %5;\n\t"
            "madc.lo.cc.u32 %6, %13, %17, %6;\n\t"
            "madc.hi.cc.u32 %7, %13, %17, %7;\n\t"
            "madc.lo.cc.u32 %8, %13, %18, %8;\n\t"
            "madc.hi.cc.u32 %9, %13, %18, %9;\n\t"
            "madc.lo.cc.u32 %10, %13, %19, %10;\n\t"
            "madc.hi.cc.u32 %11, %13, %19, %11;\n\t"
            "addc.u32       %12, %12, 0;"
            : "+r"(o[0]), "+r"(o[1]), "+r"(o[2]), "+r"(o[3]), "+r"(o[4]), "+r"(o[5]), "+r"(o[6]), "+r"(o[7]), "+r"(o[8]), "+r"(o[9]), "+r"(o[10]), "+r"(o[11]), "+r"(o[12])
            : "r"(m), "n"(CATMSM_P1), "n"(CATMSM_P3), "n"(CATMSM_P5), "n"(CATMSM_P7), "n"(CATMSM_P9), "n"(CATMSM_P11));
        // t = (E + O*2^32) / 2^32 (the weight-13 word is zero by the bound)
        asm("add.cc.u32  %0, %0, %12;\n\t"
            "addc.cc.u32 %1, %1, %13;\n\t"
            "addc.cc.u32 %2, %2, %14;\n\t"
            "addc.cc.u32 %3, %3, %15;\n\t"
            "addc.cc.u32 %4, %4, %16;\n\t"
            "addc.cc.u32 %5, %5, %17;\n\t"
            "addc.cc.u32 %6, %6, %18;\n\t"
            "addc.cc.u32 %7, %7, %19;\n\t"
            "addc.cc.u32 %8, %8, %20;\n\t"
            "addc.cc.u32 %9, %9, %21;\n\t"
            "addc.cc.u32 %10, %10, %22;\n\t"
            "addc.u32    %11, %11, %23;"
            : "+r"(o[0]), "+r"(o[1]), "+r"(o[2]), "+r"(o[3]), "+r"(o[4]), "+r"(o[5]),
              "+r"(o[6]), "+r"(o[7]), "+r"(o[8]), "+r"(o[9]), "+r"(o[10]), "+r"(o[11])
            : "r"(e[1]), "r"(e[2]), "r"(e[3]), "r"(e[4]), "r"(e[5]), "r"(e[6]),
              "r"(e[7]), "r"(e[8]), "r"(e[9]), "r"(e[10]), "r"(e[11]), "r"(e[12]));
#pragma unroll
        for (int k = 0; k < 12; k++) t[k] = o[k];
    }
#pragma unroll
    for (int k = 0; k < 12; k++) r.v[k] = t[k];
}

static __device__ __noinline__ fp fp_mul2_call(const fp a, const fp b, const fp c, const fp d)
{
    fp r;
    fp_mul2_impl(r, a, b, c, d);
    return r;
}

// r = a * b + c * d (Montgomery), one reduction
__device__ __forceinline__ void fp_mul2(fp& r, const fp& a, const fp& b, const fp& c, const fp& d)
{
    r = fp_mul2_call(a, b, c, d);
}

// r = a + b mod 2p (inputs < 2p)
__device__ __forceinline__ void fp_add(fp& r, const fp& a, const fp& b)
{
    uint32_t s[12], d[12], borrow;
    asm("add.cc.u32  %0, %12, %24;\n\t"
        "addc.cc.u32 %1, %13, %25;\n\t"
        "addc.cc.u32 %2, %14, %26;\n\t"
        "addc.cc.u32 %3, %15, %27;\n\t"
        "addc.cc.u32 %4, %16, %28;\n\t"
        "addc.cc.u32 %5, %17, %29;\n\t"
        "addc.cc.u32 %6, %18, %30;\n\t"
        "addc.cc.u32 %7, %19, %31;\n\t"
        "addc.cc.u32 %8, %20, %32;\n\t"
        "addc.cc.u32 %9, %21, %33;\n\t"
        "addc.cc.u32 %10, %22, %34;\n\t"
        "addc.u32    %11, %23, %35;"
        : "=r"(s[0]), "=r"(s[1]), "=r"(s[2]), "=r"(s[3]), "=r"(s[4]), "=r"(s[5]),
          "=r"(s[6]), "=r"(s[7]), "=r"(s[8]), "=r"(s[9]), "=r"(s[10]), "=r"(s[11])
        : "r"(a.v[0]), "r"(a.v[1]), "r"(a.v[2]), "r"(a.v[3]), "r"(a.v[4]), "r"(a.v[5]),
          "r"(a.v[6]), "r"(a.v[7]), "r"(a.v[8]), "r"(a.v[9]), "r"(a.v[10]), "r"(a.v[11]),
          "r"(b.v[0]), "r"(b.v[1]), "r"(b.v[2]), "r"(b.v[3]), "r"(b.v[4]), "r"(b.v[5]),
          "r"(b.v[6]), "r"(b.v[7]), "r"(b.v[8]), "r"(b.v[9]), "r"(b.v[10]), "r"(b.v[11]));
    asm("sub.cc.u32  %0, %13, 0xffff5556;\n\t"
        "subc.cc.u32 %1, %14, 0x73fdffff;\n\t"
        "subc.cc.u32 %2, %15, 0x62a7ffff;\n\t"
        "subc.cc.u32 %3, %16, 0x3d57fffd;\n\t"
        "subc.cc.u32 %4, %17, 0xed61ec48;\n\t"
        "subc.cc.u32 %5, %18, 0xce61a541;\n\t"
        "subc.cc.u32 %6, %19, 0xe70a257e;\n\t"
        "subc.cc.u32 %7, %20, 0xc8ee9709;\n\t"
        "subc.cc.u32 %8, %21, 0x869759ae;\n\t"
        "subc.cc.u32 %9, %22, 0x96374f6c;\n\t"
        "subc.cc.u32 %10, %23, 0x72ffcd34;\n\t"
        "subc.cc.u32 %11, %24, 0x340223d4;\n\t"
        "subc.u32    %12, 0, 0;"
        : "=r"(d[0]), "=r"(d[1]), "=r"(d[2]), "=r"(d[3]), "=r"(d[4]), "=r"(d[5]),
          "=r"(d[6]), "=r"(d[7]), "=r"(d[8]), "=r"(d[9]), "=r"(d[10]), "=r"(d[11]),
          "=r"(borrow)
        : "r"(s[0]), "r"(s[1]), "r"(s[2]), "r"(s[3]), "r"(s[4]), "r"(s[5]),
          "r"(s[6]), "r"(s[7]), "r"(s[8]), "r"(s[9]), "r"(s[10]), "r"(s[11]));
    // borrow == 0xffffffff iff s < 2p
#pragma unroll
    for (int k = 0; k < 12; k++) r.v[k] = borrow ? s[k] : d[k];
}

// r = a - b mod 2p (inputs < 2p)
__device__ __forceinline__ void fp_sub(fp& r, const fp& a, const fp& b)
{
    uint32_t d[12], s[12], borrow;
    asm("sub.cc.u32  %0, %13, %25;\n\t"
        "subc.cc.u32 %1, %14, %26;\n\t"
        "subc.cc.u32 %2, %15, %27;\n\t"
        "subc.cc.u32 %3, %16, %28;\n\t"
        "subc.cc.u32 %4, %17, %29;\n\t"
        "subc.cc.u32 %5, %18, %30;\n\t"
        "subc.cc.u32 %6, %19, %31;\n\t"
        "subc.cc.u32 %7, %20, %32;\n\t"
        "subc.cc.u32 %8, %21, %33;\n\t"
        "subc.cc.u32 %9, %22, %34;\n\t"
        "subc.cc.u32 %10, %23, %35;\n\t"
        "subc.cc.u32 %11, %24, %36;\n\t"
        "subc.u32    %12, 0, 0;"
        : "=r"(d[0]), "=r"(d[1]), "=r"(d[2]), "=r"(d[3]), "=r"(d[4]), "=r"(d[5]),
          "=r"(d[6]), "=r"(d[7]), "=r"(d[8]), "=r"(d[9]), "=r"(d[10]), "=r"(d[11]),
          "=r"(borrow)
        : "r"(a.v[0]), "r"(a.v[1]), "r"(a.v[2]), "r"(a.v[3]), "r"(a.v[4]), "r"(a.v[5]),
          "r"(a.v[6]), "r"(a.v[7]), "r"(a.v[8]), "r"(a.v[9]), "r"(a.v[10]), "r"(a.v[11]),
          "r"(b.v[0]), "r"(b.v[1]), "r"(b.v[2]), "r"(b.v[3]), "r"(b.v[4]), "r"(b.v[5]),
          "r"(b.v[6]), "r"(b.v[7]), "r"(b.v[8]), "r"(b.v[9]), "r"(b.v[10]), "r"(b.v[11]));
    asm("add.cc.u32  %0, %12, 0xffff5556;\n\t"
        "addc.cc.u32 %1, %13, 0x73fdffff;\n\t"
        "addc.cc.u32 %2, %14, 0x62a7ffff;\n\t"
        "addc.cc.u32 %3, %15, 0x3d57fffd;\n\t"
        "addc.cc.u32 %4, %16, 0xed61ec48;\n\t"
        "addc.cc.u32 %5, %17, 0xce61a541;\n\t"
        "addc.cc.u32 %6, %18, 0xe70a257e;\n\t"
        "addc.cc.u32 %7, %19, 0xc8ee9709;\n\t"
        "addc.cc.u32 %8, %20, 0x869759ae;\n\t"
        "addc.cc.u32 %9, %21, 0x96374f6c;\n\t"
        "addc.cc.u32 %10, %22, 0x72ffcd34;\n\t"
        "addc.u32    %11, %23, 0x340223d4;"
        : "=r"(s[0]), "=r"(s[1]), "=r"(s[2]), "=r"(s[3]), "=r"(s[4]), "=r"(s[5]),
          "=r"(s[6]), "=r"(s[7]), "=r"(s[8]), "=r"(s[9]), "=r"(s[10]), "=r"(s[11])
        : "r"(d[0]), "r"(d[1]), "r"(d[2]), "r"(d[3]), "r"(d[4]), "r"(d[5]),
          "r"(d[6]), "r"(d[7]), "r"(d[8]), "r"(d[9]), "r"(d[10]), "r"(d[11]));
#pragma unroll
    for (int k = 0; k < 12; k++) r.v[k] = borrow ? s[k] : d[k];
}

__device__ __forceinline__ void fp_neg(fp& r, const fp& a)
{
    fp z;
    fp_zero(z);
    fp_sub(r, z, a);
}

// Map [0, 2p) to [0, p).
__device__ __forceinline__ void fp_canon(fp& r, const fp& a)
{
    uint32_t d[12], borrow;
    asm("sub.cc.u32  %0, %13, 0xffffaaab;\n\t"
        "subc.cc.u32 %1, %14, 0xb9feffff;\n\t"
        "subc.cc.u32 %2, %15, 0xb153ffff;\n\t"
        "subc.cc.u32 %3, %16, 0x1eabfffe;\n\t"
        "subc.cc.u32 %4, %17, 0xf6b0f624;\n\t"
        "subc.cc.u32 %5, %18, 0x6730d2a0;\n\t"
        "subc.cc.u32 %6, %19, 0xf38512bf;\n\t"
        "subc.cc.u32 %7, %20, 0x64774b84;\n\t"
        "subc.cc.u32 %8, %21, 0x434bacd7;\n\t"
        "subc.cc.u32 %9, %22, 0x4b1ba7b6;\n\t"
        "subc.cc.u32 %10, %23, 0x397fe69a;\n\t"
        "subc.cc.u32 %11, %24, 0x1a0111ea;\n\t"
        "subc.u32    %12, 0, 0;"
        : "=r"(d[0]), "=r"(d[1]), "=r"(d[2]), "=r"(d[3]), "=r"(d[4]), "=r"(d[5]),
          "=r"(d[6]), "=r"(d[7]), "=r"(d[8]), "=r"(d[9]), "=r"(d[10]), "=r"(d[11]),
          "=r"(borrow)
        : "r"(a.v[0]), "r"(a.v[1]), "r"(a.v[2]), "r"(a.v[3]), "r"(a.v[4]), "r"(a.v[5]),
          "r"(a.v[6]), "r"(a.v[7]), "r"(a.v[8]), "r"(a.v[9]), "r"(a.v[10]), "r"(a.v[11]));
#pragma unroll
    for (int k = 0; k < 12; k++) r.v[k] = borrow ? a.v[k] : d[k];
}

// a == 0 mod p, for a in [0, 2p): a == 0 or a == p
__device__ __forceinline__ bool fp_is_zero(const fp& a)
{
    uint32_t z = 0, q = 0;
#pragma unroll
    for (int k = 0; k < 12; k++) {
        z |= a.v[k];
        q |= a.v[k] ^ FP_P[k];
    }
    return z == 0 || q == 0;
}

// exact (bitwise) zero test, for encodings where zero means "absent"
__device__ __forceinline__ bool fp_is_zero_raw(const fp& a)
{
    uint32_t z = 0;
#pragma unroll
    for (int k = 0; k < 12; k++) z |= a.v[k];
    return z == 0;
}

__device__ __forceinline__ void fp_dbl(fp& r, const fp& a) { fp_add(r, a, a); }

// r = a^e for a public exponent given as 12 little-endian words
__device__ __forceinline__ void fp_pow(fp& r, const fp& a, const uint32_t* e)
{
    fp acc;
    fp_set_one(acc);
    for (int i = 383; i >= 0; i--) {
        fp_sqr(acc, acc);
        if ((e[i >> 5] >> (i & 31)) & 1) fp_mul(acc, acc, a);
    }
    r = acc;
}

// r = a^(p-2) = a^-1 (Fermat); zero maps to zero
__device__ __forceinline__ void fp_inv(fp& r, const fp& a)
{
    uint32_t e[12];
#pragma unroll
    for (int k = 0; k < 12; k++) e[k] = FP_P[k];
    e[0] -= 2;
    fp_pow(r, a, e);
}

}  // namespace catmsm
