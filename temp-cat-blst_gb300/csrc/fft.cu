// BLS12-381 G1 group-valued FFT on sm_103a.
//
// Drop-in for blst_p1_fft / blst_p1_fft_with_domain /
// blst_p1_ifft_unscaled_with_domain (reference fft_c_api.cpp:51-103,
// fft/ctFft.h:32-124, fft/context.h:182-215).  The transform is the same
// radix-2 decimation-in-time schedule with the same root indexing
// (root j * n/len, or n - j * n/len when the inverse reads forward roots), so
// outputs equal the reference's for any root table the caller supplies.
//
// Device layout: n Jacobian points (blst_p1 bytes, 144 B) in HBM.
//   k_roots_prepare  per root index: Montgomery Fr -> canonical -> GLV halves
//                    (k = k1 + lambda k2), stored as 8 words.
//   k_bitrev         out-of-place bit-reversal permutation.
//   k_fft_stage      one launch per stage; threads map first onto the
//                    non-trivial butterflies (j >= 1, one GLV wNAF-5 scalar
//                    multiplication each), then onto the j == 0 butterflies,
//                    so a warp rarely mixes the two.
//   k_fft_scale      inverse 1/n scale: one GLV multiplication per element.
// Each butterfly is ~1.7k Fp multiplications (~1M IMAD) against 576 bytes of
// traffic, so the stages are IMAD-bound and read/write straight from HBM/L2;
// staging tiles in shared memory would save nothing measurable.
#include "common.cuh"
#include "curve.cuh"
#include "fr.cuh"
#include "catmsm_internal.h"

namespace catmsm {

__device__ __forceinline__ void load_jac(jac& p, const jac* src)
{
    const uint4* q = reinterpret_cast<const uint4*>(src);
    uint32_t* d = reinterpret_cast<uint32_t*>(&p);
#pragma unroll
    for (int k = 0; k < 9; k++) {
        uint4 v = q[k];
        d[4 * k] = v.x; d[4 * k + 1] = v.y; d[4 * k + 2] = v.z; d[4 * k + 3] = v.w;
    }
}

__device__ __forceinline__ void store_jac(jac* dst, const jac& p)
{
    uint4* q = reinterpret_cast<uint4*>(dst);
    const uint32_t* s = reinterpret_cast<const uint32_t*>(&p);
#pragma unroll
    for (int k = 0; k < 9; k++) q[k] = make_uint4(s[4 * k], s[4 * k + 1], s[4 * k + 2], s[4 * k + 3]);
}

// roots_mont: n Montgomery Fr (caller table); out: n x {k1[4], k2[4]}
__global__ void k_roots_prepare(const uint32_t* __restrict__ roots_mont, uint32_t n, uint32_t* __restrict__ out)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    uint32_t m[8], c[8];
    for (int k = 0; k < 8; k++) m[k] = roots_mont[8 * i + k];
    fr_from_mont(c, m);
    fr_glv_split(out + 8 * i, out + 8 * i + 4, c);
}

// powers of a Montgomery root: out[i] = w^i (Montgomery)
__global__ void k_root_powers(const uint32_t* __restrict__ w, uint32_t n, uint32_t* __restrict__ out)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    uint32_t b[8], o[8];
    for (int k = 0; k < 8; k++) b[k] = w[k];
    fr_pow_u32(o, b, i);
    for (int k = 0; k < 8; k++) out[8 * i + k] = o[k];
}

__global__ void k_bitrev(const jac* __restrict__ in, jac* __restrict__ out, uint32_t n, uint32_t logn)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t r = logn ? (__brev(i) >> (32 - logn)) : 0;
    jac p;
    load_jac(p, in + i);
    store_jac(out + r, p);
}

__global__ void __launch_bounds__(128) k_fft_stage(jac* __restrict__ a, uint32_t n, uint32_t len,
                                                   const uint32_t* __restrict__ glv, int inv_from_fwd)
{
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t half = len >> 1;
    const uint32_t groups = n / len;
    const uint32_t nontriv = groups * (half - 1);
    uint32_t g, j;
    if (t < nontriv) {
        g = t / (half - 1);
        j = 1 + t % (half - 1);
    } else if (t < nontriv + groups) {
        g = t - nontriv;
        j = 0;
    } else {
        return;
    }
    const uint32_t i0 = g * len + j, i1 = i0 + half;
    jac u, v;
    load_jac(u, a + i0);
    load_jac(v, a + i1);
    if (j) {
        uint32_t idx = j * (n / len);
        if (inv_from_fwd) idx = n - idx;
        jac_mult_glv(v, v, glv + 8 * idx, glv + 8 * idx + 4);
    }
    jac s = u;
    jac_add(s, v);
    jac_neg(v);
    jac_add(u, v);
    store_jac(a + i0, s);
    store_jac(a + i1, u);
}

__global__ void __launch_bounds__(128) k_fft_scale(jac* __restrict__ a, uint32_t n, const uint32_t* __restrict__ glv)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    jac v;
    load_jac(v, a + i);
    jac_mult_glv(v, v, glv, glv + 4);
    store_jac(a + i, v);
}

// Canonicalise coordinates to [0, p) so the output bytes are reduced
// Montgomery values like the reference's.
__global__ void k_canon(jac* __restrict__ a, uint32_t n)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    jac v;
    load_jac(v, a + i);
    if (jac_is_inf(v)) {
        jac_set_inf(v);
    } else {
        fp_canon(v.x, v.x);
        fp_canon(v.y, v.y);
        fp_canon(v.z, v.z);
    }
    store_jac(a + i, v);
}

// d_values: n Jacobian points; d_roots_mont: n Montgomery roots (the table
// the butterflies index); d_scale_mont: optional Montgomery scale factor.
// The result lands back in d_values.
cudaError_t fft_run(Ctx* ctx, void* d_values, size_t n, const uint32_t* d_roots_mont, bool inv_from_fwd,
                    const uint32_t* d_scale_mont)
{
    cudaStream_t st = ctx->stream;
    FftWork& W = ctx->fft;
    jac* vals = (jac*)d_values;
    jac* tmp = (jac*)W.scratch.get(n * sizeof(jac));
    uint32_t* glv = (uint32_t*)W.glv.get((n + 1) * 32);
    if (!tmp || !glv) return cudaErrorMemoryAllocation;
    uint32_t logn = 0;
    while (((size_t)1 << logn) < n) logn++;
    k_roots_prepare<<<div_up(n, 256), 256, 0, st>>>(d_roots_mont, (uint32_t)n, glv);
    if (d_scale_mont) k_roots_prepare<<<1, 32, 0, st>>>(d_scale_mont, 1, glv + 8 * n);
    k_bitrev<<<div_up(n, 256), 256, 0, st>>>(vals, tmp, (uint32_t)n, logn);
    g_stats.launches += 2 + (d_scale_mont ? 1 : 0);
    for (size_t len = 2; len <= n; len <<= 1) {
        const size_t half = len / 2, groups = n / len;
        const size_t threads = groups * (half - 1) + groups;
        k_fft_stage<<<div_up(threads, 128), 128, 0, st>>>(tmp, (uint32_t)n, (uint32_t)len, glv, inv_from_fwd ? 1 : 0);
        g_stats.launches++;
    }
    if (d_scale_mont) {
        k_fft_scale<<<div_up(n, 128), 128, 0, st>>>(tmp, (uint32_t)n, glv + 8 * n);
        g_stats.launches++;
    }
    k_canon<<<div_up(n, 256), 256, 0, st>>>(tmp, (uint32_t)n);
    g_stats.launches++;
    CATMSM_CHECK(cudaGetLastError());
    CATMSM_CHECK(cudaMemcpyAsync(vals, tmp, n * sizeof(jac), cudaMemcpyDeviceToDevice, st));
    return cudaSuccess;
}

cudaError_t fft_root_powers(Ctx* ctx, const uint32_t* d_w_mont, size_t n, uint32_t* d_out)
{
    k_root_powers<<<div_up(n, 256), 256, 0, ctx->stream>>>(d_w_mont, (uint32_t)n, d_out);
    g_stats.launches++;
    return cudaGetLastError();
}

}  // namespace catmsm
