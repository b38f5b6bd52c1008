// Batched point decoding and validation on sm_103a.
//
// Each element follows the reference's single-point semantics exactly:
//   uncompress   blst_p1_uncompress  (blst/c_api.cpp:1633 -> scalar/curve/
//                point.cpp:909-1001): compressed flag required; infinity only
//                as 0xc0 followed by zeros; top 3 bits of x cleared, x < p,
//                y = sqrt(x^3 + 4) (p = 3 mod 4: a^((p+1)/4)), sign flag picks
//                y or -y by "y > (p-1)/2"; x == 0 is the order-2-coset point
//                (0, +/-2) -> POINT_NOT_IN_GROUP.
//   deserialize  blst_p1_deserialize (c_api.cpp:1643 -> point.cpp:1007-1103):
//                no flags -> big-endian x, y < p, on the curve, x != 0;
//                compressed flag -> uncompress; infinity flag alone with zeros
//                -> infinity; anything else -> BAD_ENCODING.
//   in_g1        blst_p1_affine_in_g1 (c_api.cpp:1257 -> point.cpp:1182-1244):
//                on the curve and phi^2(P) == -z^2 P (Scott's endomorphism
//                test, eprint 2021/1130, proof El Housni et al. 2022/352
//                Prop. 4), z = -0xd201000000010000; infinity is a member.
// Failed elements keep the caller's output bytes.  A decode can optionally be
// followed by the membership test (POINT_NOT_IN_GROUP on failure).
#include "common.cuh"
#include "curve.cuh"
#include "catmsm_internal.h"
#include "catmsm_gpu.h"

namespace catmsm {

enum { kOk = 0, kBadEncoding = 1, kNotOnCurve = 2, kNotInGroup = 3 };

__device__ __constant__ static const uint32_t FP_R2[12] = {
    0x1c341746u, 0xf4df1f34u, 0x09d104f1u, 0x0a76e6a6u, 0x4c95b6d5u, 0x8de5476cu,
    0x939d83c0u, 0x67eb88a9u, 0xb519952du, 0x9a793e85u, 0x92cae3aau, 0x11988fe5u};
__device__ __constant__ static const uint32_t FP_FOUR[12] = {   // 4 (Montgomery)
    0x000cfff3u, 0xaa270000u, 0xfc34000au, 0x53cc0032u, 0x6b0a807fu, 0x478fe97au,
    0xe6ba24d7u, 0xb1d37ebeu, 0xbf78ab2fu, 0x8ec9733bu, 0x3d83de7eu, 0x09d64551u};
__device__ __constant__ static const uint32_t FP_SQRT_E[12] = { // (p + 1) / 4
    0xffffeaabu, 0xee7fbfffu, 0xac54ffffu, 0x07aaffffu, 0x3dac3d89u, 0xd9cc34a8u,
    0x3ce144afu, 0xd91dd2e1u, 0x90d2eb35u, 0x92c6e9edu, 0x8e5ff9a6u, 0x0680447au};
__device__ __constant__ static const uint32_t FP_HALF[12] = {   // (p - 1) / 2
    0xffffd555u, 0xdcff7fffu, 0x58a9ffffu, 0x0f55ffffu, 0x7b587b12u, 0xb3986950u,
    0x79c2895fu, 0xb23ba5c2u, 0x21a5d66bu, 0x258dd3dbu, 0x1cbff34du, 0x0d0088f5u};
__device__ __constant__ static const uint32_t FP_BETA2[12] = {  // beta^2 (Montgomery)
    0x798a64e8u, 0x30f1361bu, 0x7ece5a2au, 0xf3b8ddabu, 0xc61577f7u, 0x16a8ca3au,
    0x74fd029bu, 0xc26a2ff8u, 0x60701c6eu, 0x3636b766u, 0x241b6160u, 0x051ba4abu};

__device__ __forceinline__ void fp_from_be(fp& r, const uint8_t* b)
{
#pragma unroll
    for (int k = 0; k < 12; k++) {
        const uint8_t* q = b + 44 - 4 * k;
        r.v[k] = ((uint32_t)q[0] << 24) | ((uint32_t)q[1] << 16) | ((uint32_t)q[2] << 8) | q[3];
    }
}

// a < b as 384-bit integers
__device__ __forceinline__ bool lt384(const fp& a, const uint32_t* b)
{
    for (int k = 11; k >= 0; k--)
        if (a.v[k] != b[k]) return a.v[k] < b[k];
    return false;
}

__device__ __forceinline__ bool eq_canon(const fp& a, const fp& b)
{
    fp x, y;
    fp_canon(x, a);
    fp_canon(y, b);
    uint32_t d = 0;
#pragma unroll
    for (int k = 0; k < 12; k++) d |= x.v[k] ^ y.v[k];
    return d == 0;
}

__device__ __forceinline__ void load_const(fp& r, const uint32_t* c)
{
#pragma unroll
    for (int k = 0; k < 12; k++) r.v[k] = c[k];
}

// y^2 == x^3 + 4 (Montgomery inputs)
__device__ __forceinline__ bool on_curve_xy(const fp& x, const fp& y)
{
    fp yy, xxx, four;
    fp_sqr(yy, y);
    fp_sqr(xxx, x);
    fp_mul(xxx, xxx, x);
    load_const(four, FP_FOUR);
    fp_add(xxx, xxx, four);
    return eq_canon(yy, xxx);
}

// canonical integer of a Montgomery value > (p - 1) / 2
__device__ __forceinline__ bool is_large(const fp& y)
{
    fp one, t;
    fp_zero(one);
    one.v[0] = 1;
    fp_mul(t, y, one);
    fp_canon(t, t);
    for (int k = 11; k >= 0; k--)
        if (t.v[k] != FP_HALF[k]) return t.v[k] > FP_HALF[k];
    return false;
}

__device__ int uncompress48(affine& out, const uint8_t* in)
{
    const uint8_t in0 = in[0];
    if ((in0 & 0x80) == 0) return kBadEncoding;
    if (in0 & 0x40) {
        uint32_t z = in0 & 0x3f;
        for (int i = 1; i < 48; i++) z |= in[i];
        if (z) return kBadEncoding;
        fp_zero(out.x);
        fp_zero(out.y);
        return kOk;
    }
    fp x;
    fp_from_be(x, in);
    x.v[11] &= 0x1fffffffu;                       // top 3 bits carry flags
    if (!lt384(x, FP_P)) return kBadEncoding;
    fp r2;
    load_const(r2, FP_R2);
    fp_mul(x, x, r2);
    fp a, four, y;
    fp_sqr(a, x);
    fp_mul(a, a, x);
    load_const(four, FP_FOUR);
    fp_add(a, a, four);
    fp_pow(y, a, FP_SQRT_E);
    fp yy;
    fp_sqr(yy, y);
    if (!eq_canon(yy, a)) return kNotOnCurve;
    const bool want = (in0 & 0x20) != 0;
    if (is_large(y) != want) fp_neg(y, y);
    fp_canon(x, x);
    fp_canon(y, y);
    if (fp_is_zero_raw(x)) return kNotInGroup;
    out.x = x;
    out.y = y;
    return kOk;
}

__device__ int deserialize96(affine& out, const uint8_t* in)
{
    const uint8_t in0 = in[0];
    if ((in0 & 0xe0) == 0) {
        fp x, y;
        fp_from_be(x, in);
        fp_from_be(y, in + 48);
        if (!lt384(x, FP_P) || !lt384(y, FP_P)) return kBadEncoding;
        fp r2;
        load_const(r2, FP_R2);
        fp_mul(x, x, r2);
        fp_mul(y, y, r2);
        fp_canon(x, x);
        fp_canon(y, y);
        const bool inf = fp_is_zero_raw(x) && fp_is_zero_raw(y);
        if (!inf && !on_curve_xy(x, y)) return kNotOnCurve;
        if (fp_is_zero_raw(x)) return kNotInGroup;
        out.x = x;
        out.y = y;
        return kOk;
    }
    if (in0 & 0x80) return uncompress48(out, in);
    if (in0 & 0x40) {
        uint32_t z = in0 & 0x3f;
        for (int i = 1; i < 96; i++) z |= in[i];
        if (z) return kBadEncoding;
        fp_zero(out.x);
        fp_zero(out.y);
        return kOk;
    }
    return kBadEncoding;
}

// out = |z| * p with |z| = 0xd201000000010000 (the reference's addition chain)
__device__ __forceinline__ void times_abs_z(jac& out, const jac& p)
{
    out = p;
    jac_dbl(out);                                           // 0x2
    jac_add(out, p); jac_dbl(out); jac_dbl(out);            // 0xc
    jac_add(out, p); for (int i = 0; i < 3; i++) jac_dbl(out);   // 0x68
    jac_add(out, p); for (int i = 0; i < 9; i++) jac_dbl(out);   // 0xd200
    jac_add(out, p); for (int i = 0; i < 32; i++) jac_dbl(out);  // 0xd20100000000
    jac_add(out, p); for (int i = 0; i < 16; i++) jac_dbl(out);  // 0xd201000000010000
}

__device__ bool in_g1(const affine& a)
{
    const bool inf = fp_is_zero_raw(a.x) && fp_is_zero_raw(a.y);
    if (inf) return true;
    if (!on_curve_xy(a.x, a.y)) return false;
    jac P, t0, t1;
    P.x = a.x;
    P.y = a.y;
    fp_set_one(P.z);
    times_abs_z(t0, P);
    times_abs_z(t1, t0);                                    // z^2 P
    jac_neg(t1);                                            // -z^2 P
    if (jac_is_inf(t1)) return false;                       // phi^2(P) is finite
    // phi^2(P) = (beta^2 x, y) vs t1 = (X, Y, Z): X == beta^2 x Z^2, Y == y Z^3
    fp b2, zz, zzz, t;
    load_const(b2, FP_BETA2);
    fp_sqr(zz, t1.z);
    fp_mul(zzz, zz, t1.z);
    fp_mul(t, a.x, b2);
    fp_mul(t, t, zz);
    if (!eq_canon(t, t1.x)) return false;
    fp_mul(t, a.y, zzz);
    return eq_canon(t, t1.y);
}

// mode 0: uncompress (48-byte elements), 1: deserialize (96), 2: in_g1 only
// (96-byte affine Montgomery points in `out`)
__global__ void __launch_bounds__(128) k_decode(const uint8_t* __restrict__ in, uint32_t n, int mode,
                                                int check_group, affine* __restrict__ out,
                                                int32_t* __restrict__ errs)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    affine a;
    int err = kOk;
    if (mode == 2) {
        a = out[i];
        errs[i] = in_g1(a) ? 1 : 0;
        return;
    }
    err = mode == 0 ? uncompress48(a, in + 48 * (size_t)i) : deserialize96(a, in + 96 * (size_t)i);
    if (err == kOk && check_group && !in_g1(a)) err = kNotInGroup;
    if (err == kOk) out[i] = a;
    errs[i] = err;
}

static int decode_run(const uint8_t* in, size_t elem, int mode, size_t n, blst_p1_affine* out, int* errs,
                      int check_group)
{
    if (n == 0) return 0;
    if (!out || !errs || (mode != 2 && !in) || n > 0x7fffffffu) return (int)cudaErrorInvalidValue;
    Ctx* ctx = get_ctx();
    if (!ctx) return (int)cudaErrorInitializationError;
    cudaStream_t st = ctx->stream;
    uint8_t* din = mode == 2 ? nullptr : (uint8_t*)ctx->msm.scalars.get(n * elem);
    affine* dout = (affine*)ctx->msm.points.get(n * sizeof(affine));
    int32_t* derr = (int32_t*)ctx->msm.digits.get(n * 4);
    if ((mode != 2 && !din) || !dout || !derr) return (int)cudaErrorMemoryAllocation;
    cudaError_t err = cudaSuccess;
    if (mode != 2) err = cudaMemcpyAsync(din, in, n * elem, cudaMemcpyHostToDevice, st);
    if (err == cudaSuccess) err = cudaMemcpyAsync(dout, out, n * sizeof(affine), cudaMemcpyHostToDevice, st);
    if (err == cudaSuccess) {
        k_decode<<<div_up(n, 128), 128, 0, st>>>(din, (uint32_t)n, mode, check_group, dout, derr);
        g_stats.launches++;
        err = cudaGetLastError();
    }
    if (err == cudaSuccess && mode != 2)
        err = cudaMemcpyAsync(out, dout, n * sizeof(affine), cudaMemcpyDeviceToHost, st);
    if (err == cudaSuccess) err = cudaMemcpyAsync(errs, derr, n * 4, cudaMemcpyDeviceToHost, st);
    if (err == cudaSuccess) err = cudaStreamSynchronize(st);
    return (int)err;
}

}  // namespace catmsm

using namespace catmsm;

extern "C" {

int catmsm_p1s_uncompress(blst_p1_affine* out, const blst_byte* in48, size_t n, int* errs, int check_group)
{
    return decode_run(in48, 48, 0, n, out, errs, check_group);
}

int catmsm_p1s_deserialize(blst_p1_affine* out, const blst_byte* in96, size_t n, int* errs, int check_group)
{
    return decode_run(in96, 96, 1, n, out, errs, check_group);
}

int catmsm_p1s_affine_in_g1(const blst_p1_affine* points, size_t n, int* results)
{
    return decode_run(nullptr, 96, 2, n, const_cast<blst_p1_affine*>(points), results, 0);
}

}  // extern "C"
