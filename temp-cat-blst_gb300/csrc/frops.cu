// Scalar-field (Fr) entry points on sm_103a:
//  * blst_p1s_mult_pippenger_fr (reference blst/c_api.cpp:1420-1435 ->
//    c_api_pippenger_fr :532-585), blst_p1s_mult_fr (:1502-1520 ->
//    c_api_msm_fr :809-850) and blst_p1s_mult_batch_affine_fr (:1522-1545 ->
//    c_api_batch_affine_fr :641-690): Montgomery-form blst_fr scalars are
//    converted to canonical integers on the device (Fr::to_scaler, i.e.
//    from_mont), then the G1 MSM pipeline runs with nbits = 255.  The three
//    differ only in their scratch contracts, which are kept exactly (the
//    reference's batch-affine algorithm and window are a CPU schedule; the
//    result is the same group element);
//  * blst_fr_fft / blst_fr_fft_with_domain (reference blst/fft_c_api.cpp:
//    109-182): radix-2 DIT over Fr with the reference's schedule and root
//    indexing (ctFft.h:50-94; FrCoeffCtx plus/minus/mult = Fr add/sub/mul).
//    Transforms of up to 2048 values run all stages in one block in shared
//    memory; larger ones take one launch per stage (an Fr butterfly is one
//    Montgomery multiplication against 64 bytes moved, so the stages are
//    HBM-bound).
#include "common.cuh"
#include "fr.cuh"
#include "catmsm_internal.h"
#include "host_fr.hpp"
#include "catmsm_gpu.h"

#include <algorithm>
#include <climits>
#include <cstring>

namespace catmsm {

__global__ void k_fr_to_canonical(uint32_t* __restrict__ s, uint32_t n)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    uint32_t m[8], c[8];
    for (int k = 0; k < 8; k++) m[k] = s[8 * i + k];
    fr_from_mont(c, m);
    for (int k = 0; k < 8; k++) s[8 * i + k] = c[k];
}

struct fr8 { uint32_t v[8]; };

__device__ __forceinline__ fr8 ld8(const uint32_t* p)
{
    const uint4 a = reinterpret_cast<const uint4*>(p)[0], b = reinterpret_cast<const uint4*>(p)[1];
    fr8 r = {{a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w}};
    return r;
}

__device__ __forceinline__ void st8(uint32_t* p, const fr8& x)
{
    reinterpret_cast<uint4*>(p)[0] = make_uint4(x.v[0], x.v[1], x.v[2], x.v[3]);
    reinterpret_cast<uint4*>(p)[1] = make_uint4(x.v[4], x.v[5], x.v[6], x.v[7]);
}

// one butterfly: (u, v) -> (u + w v, u - w v)
__device__ __forceinline__ void fr_bfly(fr8& u, fr8& v, const uint32_t* w)
{
    fr8 t;
    fr_mul(t.v, v.v, w);
    fr8 s;
    fr_add(s.v, u.v, t.v);
    fr_sub(v.v, u.v, t.v);
    u = s;
}

constexpr uint32_t kFrSmall = 2048;

// whole transform in one block (n <= 2048): bit-reversed load, all stages in
// shared memory, optional scale, store
__global__ void __launch_bounds__(1024) k_fr_fft_small(uint32_t* __restrict__ a, uint32_t n, uint32_t logn,
                                                       const uint32_t* __restrict__ roots, int inv_from_fwd,
                                                       const uint32_t* __restrict__ scale)
{
    __shared__ __align__(16) uint32_t sh[kFrSmall * 8];
    for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) {
        const uint32_t r = logn ? (__brev(i) >> (32 - logn)) : 0;
        st8(sh + 8 * r, ld8(a + 8 * i));
    }
    __syncthreads();
    for (uint32_t len = 2; len <= n; len <<= 1) {
        const uint32_t half = len >> 1;
        for (uint32_t b = threadIdx.x; b < n / 2; b += blockDim.x) {
            const uint32_t g = b / half, j = b % half;
            const uint32_t i0 = g * len + j, i1 = i0 + half;
            fr8 u = ld8(sh + 8 * i0), v = ld8(sh + 8 * i1);
            if (j) {
                uint32_t idx = j * (n / len);
                if (inv_from_fwd) idx = n - idx;
                fr_bfly(u, v, roots + 8 * idx);
            } else {
                fr8 s;
                fr_add(s.v, u.v, v.v);
                fr_sub(v.v, u.v, v.v);
                u = s;
            }
            st8(sh + 8 * i0, u);
            st8(sh + 8 * i1, v);
        }
        __syncthreads();
    }
    for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) {
        fr8 x = ld8(sh + 8 * i);
        if (scale) fr_mul(x.v, x.v, scale);
        st8(a + 8 * i, x);
    }
}

__global__ void k_fr_bitrev(const uint32_t* __restrict__ in, uint32_t* __restrict__ out, uint32_t n, uint32_t logn)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t r = __brev(i) >> (32 - logn);
    st8(out + 8 * (size_t)r, ld8(in + 8 * (size_t)i));
}

__global__ void k_fr_stage(uint32_t* __restrict__ a, uint32_t n, uint32_t len, const uint32_t* __restrict__ roots,
                           int inv_from_fwd)
{
    const uint32_t b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= n / 2) return;
    const uint32_t half = len >> 1, g = b / half, j = b % half;
    const uint32_t i0 = g * len + j, i1 = i0 + half;
    fr8 u = ld8(a + 8 * (size_t)i0), v = ld8(a + 8 * (size_t)i1);
    if (j) {
        uint32_t idx = j * (n / len);
        if (inv_from_fwd) idx = n - idx;
        fr_bfly(u, v, roots + 8 * (size_t)idx);
    } else {
        fr8 s;
        fr_add(s.v, u.v, v.v);
        fr_sub(v.v, u.v, v.v);
        u = s;
    }
    st8(a + 8 * (size_t)i0, u);
    st8(a + 8 * (size_t)i1, v);
}

__global__ void k_fr_scale(uint32_t* __restrict__ a, uint32_t n, const uint32_t* __restrict__ scale)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    fr8 x = ld8(a + 8 * (size_t)i);
    fr_mul(x.v, x.v, scale);
    st8(a + 8 * (size_t)i, x);
}

// in place on d_vals (n Montgomery Fr); tmp: n more
static cudaError_t fr_fft_run(cudaStream_t st, uint32_t* d_vals, uint32_t* tmp, size_t n, const uint32_t* d_roots,
                              bool inv_from_fwd, const uint32_t* d_scale)
{
    uint32_t logn = 0;
    while (((size_t)1 << logn) < n) logn++;
    if (n <= kFrSmall) {
        k_fr_fft_small<<<1, 1024, 0, st>>>(d_vals, (uint32_t)n, logn, d_roots, inv_from_fwd ? 1 : 0, d_scale);
        g_stats.launches++;
        return cudaGetLastError();
    }
    k_fr_bitrev<<<div_up(n, 256), 256, 0, st>>>(d_vals, tmp, (uint32_t)n, logn);
    for (size_t len = 2; len <= n; len <<= 1)
        k_fr_stage<<<div_up(n / 2, 256), 256, 0, st>>>(tmp, (uint32_t)n, (uint32_t)len, d_roots, inv_from_fwd ? 1 : 0);
    if (d_scale) k_fr_scale<<<div_up(n, 256), 256, 0, st>>>(tmp, (uint32_t)n, d_scale);
    g_stats.launches += 2 + logn;
    CATMSM_CHECK(cudaGetLastError());
    return cudaMemcpyAsync(d_vals, tmp, n * 32, cudaMemcpyDeviceToDevice, st);
}

static bool valid_size(size_t n) { return n != 0 && (n & (n - 1)) == 0 && n <= (size_t)INT_MAX; }

static unsigned log2_of(size_t n)
{
    unsigned k = 0;
    while (((size_t)1 << k) < n) k++;
    return k;
}

// domain == nullptr: one-shot roots (powers of the primitive root or of its
// inverse, scale 1/n for the inverse); else the caller's prepared domain
static bool fr_fft_entry(blst_fr* values, size_t n, const blst_fr* domain, bool inverse)
{
    using namespace catmsm_host;
    Ctx* ctx = get_ctx();
    if (!ctx) return false;
    cudaStream_t st = ctx->stream;
    uint32_t* dv = (uint32_t*)ctx->fft.values.get(2 * n * 32);
    uint32_t* dr = (uint32_t*)ctx->fft.roots.get((n + 2) * 32);
    hfr* hw = (hfr*)ctx->h_out.get(2 * sizeof(hfr));
    void* hstage = ctx->h_values.get(n * 32);
    if (!dv || !dr || !hw || !hstage) return false;
    cudaError_t err = cudaSuccess;
    const uint32_t* scale = nullptr;
    if (domain) {
        err = cudaMemcpyAsync(dr, domain, (n + 1) * 32, cudaMemcpyHostToDevice, st);
        if (inverse) scale = dr + 8 * n;
    } else {
        hfr w = fr_root_of_unity(log2_of(n));
        if (inverse) w = fr_inv(w);
        hw[0] = w;
        hw[1] = fr_inv(fr_from_u64(n));
        err = cudaMemcpyAsync(dr + 8 * n, hw, 2 * sizeof(hfr), cudaMemcpyHostToDevice, st);
        if (err == cudaSuccess) err = fft_root_powers(ctx, dr + 8 * n, n, dr);
        if (err == cudaSuccess && inverse) scale = dr + 8 * n + 8;
    }
    if (err == cudaSuccess) err = cudaMemcpyAsync(dv, values, n * 32, cudaMemcpyHostToDevice, st);
    if (err == cudaSuccess) err = fr_fft_run(st, dv, dv + 8 * n, n, dr, domain != nullptr && inverse, scale);
    if (err == cudaSuccess) err = cudaMemcpyAsync(hstage, dv, n * 32, cudaMemcpyDeviceToHost, st);
    if (err == cudaSuccess) err = cudaStreamSynchronize(st);
    if (err != cudaSuccess) return false;
    host_copy(values, hstage, n * 32);
    return true;
}

// reference c_api_pippenger_fr_scratch_sizeof (c_api.cpp:271-296)
static size_t pippenger_fr_scratch(size_t n)
{
    if (n == 0) return 0;
    if (n > SIZE_MAX / 32) return 0;
    const size_t scalar_bytes = n * 32;
    if (n == 1) return scalar_bytes;
    size_t w = 0;
    for (size_t m = n; m >>= 1;) w++;
    if (w > 12) w -= 3;
    else if (w > 8) w -= 2;
    else if (w > 4) w -= 1;
    else w = w ? 2 : 1;
    if (w > 24) w = 24;
    const size_t buckets = (size_t)1 << (w - 1);
    if (buckets > (SIZE_MAX - scalar_bytes) / 192) return 0;
    return scalar_bytes + buckets * 192;
}

// reference c_api_batch_affine_fr_scratch_sizeof (c_api.cpp:593-639) with
// msm_mult_batch_affine_scratch_sizeof (multi_scalar_batch_affine.cpp:149-170,
// :468-471): 32 n canonical-scalar bytes plus, for n > 1, 2^(w-1) 256-byte
// bucket pairs and 108 bytes per batch slot; B in {128, 384}, w in [1, 24],
// n < 2^32.
static size_t batch_affine_fr_scratch(size_t n, size_t w, size_t B)
{
    if (n == 0 || n > 0xffffffffull) return 0;
    if ((B != 128 && B != 384) || w < 1 || w > 24) return 0;
    const size_t alg = ((size_t)256 << (w - 1)) + 108 * B;
    if (n > SIZE_MAX / 32) return 0;
    const size_t scalar_bytes = n * 32;
    if (n == 1) return scalar_bytes;
    if (alg > SIZE_MAX - scalar_bytes) return 0;
    return scalar_bytes + alg;
}

// reference c_api_msm_fr_plan (c_api.cpp:723-756): the window and batch size
// the reference's policy MSM picks (window 0 = Pippenger).
static void msm_fr_plan(size_t n, size_t* w, size_t* B)
{
    *w = 0;
    *B = 0;
    if (n < ((size_t)1 << 12) || n > ((size_t)1 << 18)) return;
    if (n <= ((size_t)1 << 12)) *w = 10;
    else if (n <= ((size_t)1 << 14)) *w = 11;
    else if (n <= ((size_t)1 << 15)) *w = 12;
    else if (n <= ((size_t)1 << 16)) *w = 13;
    else if (n <= ((size_t)1 << 17)) *w = 14;
    else *w = 15;
    *B = n >= ((size_t)1 << 18) ? 384 : 128;
}

// reference c_api_msm_fr_scratch_sizeof (c_api.cpp:758-807): a capacity
// query, the larger of the Pippenger and the planned batch-affine sizes (and
// of the largest measured batch plan above 2^18 points).
static size_t mult_fr_scratch(size_t n)
{
    if (n == 0) return 0;
    size_t req = pippenger_fr_scratch(n);
    if (req == 0) return 0;
    size_t w, B;
    msm_fr_plan(n, &w, &B);
    if (w) {
        const size_t b = batch_affine_fr_scratch(n, w, B);
        if (b == 0) return 0;
        req = std::max(req, b);
    }
    const size_t measured = (size_t)1 << 18;
    if (n > measured) {
        msm_fr_plan(measured, &w, &B);
        const size_t b = batch_affine_fr_scratch(measured, w, B);
        if (b == 0) return 0;
        req = std::max(req, b);
    }
    return req;
}

// Montgomery-form scalars -> canonical integers on the device, then the MSM
// pipeline over 255-bit scalars; ret untouched unless it succeeds.
static bool fr_msm_run(blst_p1* ret, const blst_p1_affine points[], const blst_fr scalars[], size_t npoints)
{
    if (npoints > 0x7fffffffu) return false;
    Ctx* ctx = get_ctx();
    if (!ctx) return false;
    void* dp = ctx->msm.points.get(npoints * sizeof(blst_p1_affine));
    uint32_t* ds = (uint32_t*)ctx->msm.scalars.get(npoints * 32 + 16);
    if (!dp || !ds) return false;
    cudaStream_t st = ctx->stream;
    cudaError_t err = cudaMemcpyAsync(ds, scalars, npoints * 32, cudaMemcpyHostToDevice, st);
    cudaEvent_t ready = nullptr;
    if (err == cudaSuccess) err = copy_points_async(ctx, dp, points, npoints * sizeof(blst_p1_affine), &ready);
    if (err == cudaSuccess) {
        k_fr_to_canonical<<<div_up(npoints, 256), 256, 0, st>>>(ds, (uint32_t)npoints);
        g_stats.launches++;
        err = cudaGetLastError();
    }
    uint64_t out[18];
    if (err == cudaSuccess) err = msm_device(ctx, dp, (const uint8_t*)ds, 32, npoints, 255, 0, out, ready);
    if (ready) cudaStreamSynchronize(ctx->copy_stream);   // the caller's points are not read after return
    if (err != cudaSuccess) return false;
    std::memcpy(ret, out, sizeof(*ret));
    return true;
}

}  // namespace catmsm

using namespace catmsm;

extern "C" {

size_t blst_p1s_mult_pippenger_fr_scratch_sizeof(size_t npoints) { return pippenger_fr_scratch(npoints); }

bool blst_p1s_mult_pippenger_fr(blst_p1* ret, const blst_p1_affine points[], const blst_fr scalars[],
                                size_t npoints, blst_limb_t* scratch, size_t scratch_size)
{
    try {
        if (!ret) return false;
        if (npoints == 0) {
            std::memset(ret, 0, sizeof(*ret));
            return true;
        }
        const size_t required = pippenger_fr_scratch(npoints);
        if (required == 0 || !points || !scalars || !scratch || scratch_size < required) return false;
        return fr_msm_run(ret, points, scalars, npoints);
    } catch (...) {
        return false;
    }
}

size_t blst_p1s_mult_fr_scratch_sizeof(size_t max_points) { return mult_fr_scratch(max_points); }

bool blst_p1s_mult_fr(blst_p1* ret, const blst_p1_affine points[], const blst_fr scalars[], size_t npoints,
                      blst_limb_t* scratch, size_t scratch_size)
{
    try {
        if (!ret) return false;
        if (npoints == 0) {
            std::memset(ret, 0, sizeof(*ret));
            return true;
        }
        const size_t required = mult_fr_scratch(npoints);
        if (required == 0 || !points || !scalars || !scratch || scratch_size < required) return false;
        return fr_msm_run(ret, points, scalars, npoints);
    } catch (...) {
        return false;
    }
}

size_t blst_p1s_mult_batch_affine_fr_scratch_sizeof(size_t npoints, size_t window, size_t batch_size)
{
    return batch_affine_fr_scratch(npoints, window, batch_size);
}

bool blst_p1s_mult_batch_affine_fr(blst_p1* ret, const blst_p1_affine points[], const blst_fr scalars[],
                                   size_t npoints, blst_limb_t* scratch, size_t scratch_size, size_t window,
                                   size_t batch_size)
{
    try {
        if (!ret) return false;
        if (npoints == 0) {
            std::memset(ret, 0, sizeof(*ret));
            return true;
        }
        const size_t required = batch_affine_fr_scratch(npoints, window, batch_size);
        if (required == 0 || !points || !scalars || !scratch || scratch_size < required) return false;
        return fr_msm_run(ret, points, scalars, npoints);
    } catch (...) {
        return false;
    }
}

bool blst_fr_fft(blst_fr* values, size_t n, bool inverse)
{
    try {
        if (!values || !valid_size(n)) return false;
        return fr_fft_entry(values, n, nullptr, inverse);
    } catch (...) {
        return false;
    }
}

bool blst_fr_fft_with_domain(blst_fr* values, size_t n, const blst_fr* domain, size_t domain_len, bool inverse)
{
    try {
        if (!values || !domain || !valid_size(n) || domain_len != n + 2) return false;
        catmsm_host::hfr tag = catmsm_host::fr_from_u64(n);
        if (std::memcmp(&domain[n + 1], tag.l, 32) != 0) return false;
        return fr_fft_entry(values, n, domain, inverse);
    } catch (...) {
        return false;
    }
}

}  // extern "C"
