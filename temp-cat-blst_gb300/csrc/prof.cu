// Measurement support: the integer-pipe roofline denominator and the MSM's
// per-stage CUDA-event profile.
//
// k_imad_peak issues independent 32-bit IMAD chains (16 per thread, enough
// to hide the dependent-issue latency) across a grid of 8 x 152 blocks x 256
// threads, so every SM sub-partition's integer multiply-add pipe stays busy.
// Achieved IMADs per second is the device's integer multiply-add throughput
// under the clocks of the moment; the MSM's field arithmetic is measured
// against it (576 IMAD per 381-bit Montgomery multiplication).
#include "common.cuh"
#include "catmsm_internal.h"
#include "catmsm_gpu.h"

namespace catmsm {

constexpr int kImadChains = 16;
constexpr int kImadIters = 4096;

__global__ void __launch_bounds__(256) k_imad_peak(uint32_t* out, uint32_t seed)
{
    uint32_t a[kImadChains];
#pragma unroll
    for (int c = 0; c < kImadChains; c++) a[c] = seed + threadIdx.x * 31u + c;
    const uint32_t m = seed | 1u;
    for (int it = 0; it < kImadIters; it++) {
#pragma unroll
        for (int c = 0; c < kImadChains; c++) asm volatile("mad.lo.u32 %0, %0, %1, %2;" : "+r"(a[c]) : "r"(m), "r"(c + 1));
    }
    uint32_t x = 0;
#pragma unroll
    for (int c = 0; c < kImadChains; c++) x ^= a[c];
    if (x == 0x12345678u) out[blockIdx.x] = x;   // keeps the chains live
}

// Same with mad.wide.u32 (32x32+64 -> 64): each instruction yields both
// product halves, counted as two IMAD-equivalents.
__global__ void __launch_bounds__(256) k_imad_wide_peak(uint32_t* out, uint32_t seed)
{
    uint64_t a[kImadChains];
#pragma unroll
    for (int c = 0; c < kImadChains; c++) a[c] = seed + threadIdx.x * 31u + c;
    const uint32_t m = seed | 1u;
    for (int it = 0; it < kImadIters; it++) {
#pragma unroll
        for (int c = 0; c < kImadChains; c++)
            asm volatile("mad.wide.u32 %0, %1, %2, %0;" : "+l"(a[c]) : "r"((uint32_t)a[c]), "r"(m));
    }
    uint64_t x = 0;
#pragma unroll
    for (int c = 0; c < kImadChains; c++) x ^= a[c];
    if (x == 0x12345678u) out[blockIdx.x] = (uint32_t)x;
}

}  // namespace catmsm

using namespace catmsm;

extern "C" {

static double imad_run(bool wide)
{
    Ctx* ctx = get_ctx();
    if (!ctx) return -1.0;
    int sms = device_sms();
    int dev = 0;
    if (cudaGetDevice(&dev) == cudaSuccess) cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int blocks = 8 * sms, threads = 256;
    uint32_t* d = (uint32_t*)ctx->msm.misc.get((size_t)blocks * 4);
    if (!d) return -1.0;
    cudaEvent_t a, b;
    if (cudaEventCreate(&a) != cudaSuccess || cudaEventCreate(&b) != cudaSuccess) return -1.0;
    double best = 0.0;
    for (int rep = 0; rep < 6; rep++) {
        cudaEventRecord(a, ctx->stream);
        if (wide) k_imad_wide_peak<<<blocks, threads, 0, ctx->stream>>>(d, 12345u + rep);
        else k_imad_peak<<<blocks, threads, 0, ctx->stream>>>(d, 12345u + rep);
        cudaEventRecord(b, ctx->stream);
        if (cudaEventSynchronize(b) != cudaSuccess) { best = -1.0; break; }
        float ms = 0.f;
        cudaEventElapsedTime(&ms, a, b);
        const double imads = (double)blocks * threads * kImadIters * kImadChains * (wide ? 2 : 1);
        const double t = imads / (ms * 1e-3) / 1e12;
        if (rep > 0 && t > best) best = t;   // first launch is warm-up
    }
    g_stats.launches += 6;
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    return best;
}

// Measured tera-IMAD per second: the better of the mad.lo and mad.wide forms
// (in 32-bit IMAD-equivalents, best of 5 launches each), negative on failure.
double catmsm_imad_peak(void)
{
    const double lo = imad_run(false), wide = imad_run(true);
    return lo > wide ? lo : wide;
}

double catmsm_imad_peak_form(int wide) { return imad_run(wide != 0); }

void catmsm_profile(int enable)
{
    Ctx* ctx = get_ctx();
    if (ctx) ctx->prof.enabled = enable != 0;
}

void catmsm_profile_reset(void)
{
    Ctx* ctx = get_ctx();
    if (!ctx) return;
    for (int i = 0; i < kMsmStages; i++) ctx->prof.ms[i] = 0.0;
    ctx->prof.calls = 0;
    ctx->prof.entries = 0;
}

double catmsm_profile_entries(void)
{
    Ctx* ctx = get_ctx();
    return ctx ? ctx->prof.entries : 0.0;
}

int catmsm_profile_read(double* ms, int max, long* calls)
{
    Ctx* ctx = get_ctx();
    if (!ctx) return 0;
    const int k = max < kMsmStages ? max : kMsmStages;
    for (int i = 0; i < k; i++) ms[i] = ctx->prof.ms[i];
    if (calls) *calls = ctx->prof.calls;
    return kMsmStages;
}

}  // extern "C"
