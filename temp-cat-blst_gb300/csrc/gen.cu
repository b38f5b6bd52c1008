// Device helpers outside the reference boundary:
//  * seeded synthetic input support: P_i = k_i * G for 32-byte scalars k_i via
//    a fixed-base byte comb (32 rows of the 255 nonzero multiples b * 2^(8j) G,
//    built once per device), normalised to affine (canonical Montgomery bytes,
//    identical to any other correct computation of k_i * G);
//  * an element-wise Fp multiply used by the field-level parity tests.
#include "common.cuh"
#include "curve.cuh"
#include "catmsm_internal.h"

#include <mutex>

namespace catmsm {

// G1 generator (Montgomery form)
__device__ __constant__ static const uint32_t G1X[12] = {
    0xfd530c16u, 0x5cb38790u, 0x9976fff5u, 0x7817fc67u, 0x143ba1c1u, 0x154f95c7u,
    0xf3d0e747u, 0xf0ae6acdu, 0x21dbf440u, 0xedce6eccu, 0x9e0bfb75u, 0x12017741u};
__device__ __constant__ static const uint32_t G1Y[12] = {
    0x0ce72271u, 0xbaac93d5u, 0x7918fd8eu, 0x8c22631au, 0x570725ceu, 0xdd595f13u,
    0x50405194u, 0x51ac5829u, 0xad0059c0u, 0x0e1c8c3fu, 0x5008a26au, 0x0bbc3efcu};

// table[j*256 + b] = b * 2^(8j) * G (affine), b = 0 -> infinity
__global__ void __launch_bounds__(128) k_comb_table(affine* __restrict__ table)
{
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= 32 * 256) return;
    const uint32_t j = t >> 8, b = t & 255;
    affine out;
    if (b == 0) {
        fp_zero(out.x);
        fp_zero(out.y);
    } else {
        // scalar = b << (8j): double-and-add from the top bit
        fp gx, gy;
#pragma unroll
        for (int k = 0; k < 12; k++) { gx.v[k] = G1X[k]; gy.v[k] = G1Y[k]; }
        xyzz acc;
        xyzz_set_inf(acc);
        for (int bit = 7; bit >= 0; bit--) {
            xyzz_dbl(acc);
            if ((b >> bit) & 1) xyzz_madd(acc, gx, gy);
        }
        for (uint32_t d = 0; d < 8 * j; d++) xyzz_dbl(acc);
        xyzz_to_affine(out, acc);
    }
    table[t] = out;
}

__global__ void __launch_bounds__(128) k_points_from_scalars(const uint8_t* __restrict__ k32, uint32_t n,
                                                             const affine* __restrict__ table,
                                                             affine* __restrict__ out)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint8_t* k = k32 + 32 * (size_t)i;
    xyzz acc;
    xyzz_set_inf(acc);
    for (int j = 0; j < 32; j++) {
        const uint32_t b = k[j];
        if (b) {
            const affine& e = table[j * 256 + b];
            xyzz_madd(acc, e.x, e.y);
        }
    }
    affine a;
    xyzz_to_affine(a, acc);
    out[i] = a;
}

cudaError_t points_from_scalars_device(Ctx* ctx, const uint8_t* d_k32, size_t n, void* d_out)
{
    static std::mutex mu;
    static affine* tables[64] = {nullptr};
    int dev = 0;
    CATMSM_CHECK(cudaGetDevice(&dev));
    affine* table;
    {
        std::lock_guard<std::mutex> lk(mu);
        if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
        if (!tables[dev]) {
            affine* tb = nullptr;
            CATMSM_CHECK(cudaMalloc(&tb, 32 * 256 * sizeof(affine)));
            k_comb_table<<<32 * 256 / 128, 128, 0, ctx->stream>>>(tb);
            g_stats.launches++;
            CATMSM_CHECK(cudaGetLastError());
            CATMSM_CHECK(cudaStreamSynchronize(ctx->stream));
            tables[dev] = tb;
        }
        table = tables[dev];
    }
    if (n == 0) return cudaSuccess;
    k_points_from_scalars<<<div_up(n, 128), 128, 0, ctx->stream>>>(d_k32, (uint32_t)n, table, (affine*)d_out);
    g_stats.launches++;
    return cudaGetLastError();
}

__global__ void k_fp_mul_test(const fp* __restrict__ a, const fp* __restrict__ b, fp* __restrict__ o, uint32_t n,
                              int square)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    fp x = a[i], y = b[i], r;
    if (square) fp_sqr(r, x);
    else fp_mul(r, x, y);
    fp_canon(r, r);
    o[i] = r;
}

cudaError_t fp_mul_test_device(Ctx* ctx, const uint64_t* d_a, const uint64_t* d_b, uint64_t* d_out, size_t n,
                               bool square)
{
    k_fp_mul_test<<<div_up(n, 128), 128, 0, ctx->stream>>>((const fp*)d_a, (const fp*)d_b, (fp*)d_out,
                                                           (uint32_t)n, square ? 1 : 0);
    g_stats.launches++;
    return cudaGetLastError();
}

}  // namespace catmsm
