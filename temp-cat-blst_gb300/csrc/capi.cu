// C-ABI boundary: the category-blst entry points for the G1 MSM and the G1
// FFT (declared in include/catmsm_gpu.h with the reference file:line each one
// replaces), plus the device-resident extensions.  Every entry point runs on
// the calling thread's own stream and workspaces, is synchronous, and fails
// closed exactly like the reference: the MSM writes infinity, the FFT returns
// false with the caller's values untouched.
#include "common.cuh"
#include "catmsm_internal.h"
#include "host_curve.hpp"
#include "host_fr.hpp"
#include "catmsm_gpu.h"

#include <climits>
#include <cstring>
#include <new>
#include <vector>

#include <sys/syscall.h>
#include <unistd.h>

namespace catmsm {

// Everything a context holds, after its queued work: a worker thread of a
// short-lived server (or any caller thread) must not leave its workspaces
// allocated when it exits.
static void ctx_destroy(Ctx* c)
{
    if (cudaSetDevice(c->device) == cudaSuccess) {
        if (c->stream) cudaStreamSynchronize(c->stream);
        if (c->copy_stream) cudaStreamSynchronize(c->copy_stream);
        if (c->aff_stream) cudaStreamSynchronize(c->aff_stream);
        c->msm.release();
        c->fft.release();
        for (PinnedBuf* b : {&c->h_points, &c->h_scalars, &c->h_out, &c->h_values, &c->h_meta}) b->release();
        for (cudaEvent_t e : c->prof.ev)
            if (e) cudaEventDestroy(e);
        for (cudaEvent_t e : {c->points_ready, c->aff_fork, c->aff_join})
            if (e) cudaEventDestroy(e);
        for (cudaStream_t st : {c->stream, c->copy_stream, c->aff_stream})
            if (st) cudaStreamDestroy(st);
    }
    delete c;
}

// The calling thread's contexts, one per device, released at thread exit.
// The main thread's exit is the process's: its contexts are left to the
// driver's teardown, so no CUDA call runs while the runtime unloads.
struct ThreadCtxs {
    Ctx* per_dev[64] = {nullptr};
    ~ThreadCtxs()
    {
        if ((pid_t)syscall(SYS_gettid) == getpid()) return;
        int prev = -1;
        const bool had = cudaGetDevice(&prev) == cudaSuccess;
        for (Ctx*& c : per_dev)
            if (c) {
                ctx_destroy(c);
                c = nullptr;
            }
        if (had) cudaSetDevice(prev);
    }
};

Ctx* get_ctx()
{
    static thread_local ThreadCtxs ctxs;
    Ctx** per_dev = ctxs.per_dev;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return nullptr;
    if (!per_dev[dev]) {
        Ctx* c = new (std::nothrow) Ctx();
        if (!c) return nullptr;
        c->device = dev;
        if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) {
            delete c;
            return nullptr;
        }
        if (msm_setup_device() != cudaSuccess) {
            cudaStreamDestroy(c->stream);
            delete c;
            return nullptr;
        }
        per_dev[dev] = c;
    }
    return per_dev[dev];
}

// Reference window heuristic (multi_scalar.h:329-348), used only for the
// scratch-size contract.
static size_t ref_window(size_t n)
{
    size_t w;
    for (w = 0; n >>= 1; w++) {}
    if (w > 12) w -= 3;
    else if (w > 8) w -= 2;
    else if (w > 4) w -= 1;
    else return w ? 2 : 1;
    return w < 24 ? w : 24;
}

static bool valid_fft_size(size_t n) { return n != 0 && (n & (n - 1)) == 0 && n <= (size_t)INT_MAX; }

static unsigned log2_exact(size_t n)
{
    unsigned k = 0;
    while (((size_t)1 << k) < n) k++;
    return k;
}

static void write_inf(blst_p1* ret) { std::memset(ret, 0, sizeof(*ret)); }

// H2D of n points on the context's copy stream (created on first use),
// ordered after the work already queued on the pipeline stream; *ready is
// recorded after the copy.
cudaError_t copy_points_async(Ctx* ctx, void* dst, const void* src, size_t bytes, cudaEvent_t* ready)
{
    if (!ctx->copy_stream) {
        CATMSM_CHECK(cudaStreamCreateWithFlags(&ctx->copy_stream, cudaStreamNonBlocking));
        CATMSM_CHECK(cudaEventCreateWithFlags(&ctx->points_ready, cudaEventDisableTiming));
    }
    // the copy overwrites the points buffer: wait for earlier users of it
    CATMSM_CHECK(cudaEventRecord(ctx->points_ready, ctx->stream));
    CATMSM_CHECK(cudaStreamWaitEvent(ctx->copy_stream, ctx->points_ready, 0));
    CATMSM_CHECK(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, ctx->copy_stream));
    const cudaError_t err = cudaEventRecord(ctx->points_ready, ctx->copy_stream);
    if (err != cudaSuccess) {
        cudaStreamSynchronize(ctx->copy_stream);   // nothing may read the caller's buffer after return
        return err;
    }
    *ready = ctx->points_ready;
    return cudaSuccess;
}

static void msm_entry(blst_p1* ret, const blst_p1_affine* const points[], size_t npoints,
                      const blst_byte* const scalars[], size_t nbits, blst_limb_t* scratch, bool explicit_window,
                      size_t window)
{
    if (!ret) return;
    if (npoints == 0 || nbits == 0) { write_inf(ret); return; }
    if (nbits > 256 || (explicit_window && (window < 1 || window > 24)) || !points || !scalars ||
        !points[0] || !scalars[0]) {
        write_inf(ret);
        return;
    }
    if (npoints > 1 && scratch == nullptr) { write_inf(ret); return; }
    if (npoints > 0x7fffffffu) { write_inf(ret); return; }
    Ctx* ctx = get_ctx();
    if (!ctx) { write_inf(ret); return; }
    const size_t nbytes = (nbits + 7) / 8;
    bool e1, e2;
    const uint8_t* hp = gather(points, npoints, sizeof(blst_p1_affine), ctx->h_points, e1);
    const uint8_t* hs = gather(scalars, npoints, nbytes, ctx->h_scalars, e2);
    if (e1 || e2) { write_inf(ret); return; }
    void* dp = ctx->msm.points.get(npoints * sizeof(blst_p1_affine));
    void* ds = ctx->msm.scalars.get(npoints * nbytes + 16);
    if (!dp || !ds) { write_inf(ret); return; }
    uint64_t out[18];
    // Scalars first on the pipeline stream; the points on the copy stream,
    // overlapping the digit, scan and scatter stages (which need only the
    // scalars).  The pipeline waits for points_ready before reading points.
    cudaError_t err = cudaMemcpyAsync(ds, hs, npoints * nbytes, cudaMemcpyHostToDevice, ctx->stream);
    cudaEvent_t ready = nullptr;
    if (err == cudaSuccess) err = copy_points_async(ctx, dp, hp, npoints * sizeof(blst_p1_affine), &ready);
    if (err == cudaSuccess)
        err = msm_device(ctx, dp, (const uint8_t*)ds, (uint32_t)nbytes, npoints, (uint32_t)nbits, 0, out, ready);
    if (ready) cudaStreamSynchronize(ctx->copy_stream);   // the caller's points are not read after return
    if (err != cudaSuccess) { write_inf(ret); return; }
    std::memcpy(ret, out, sizeof(*ret));
}

// Common FFT driver.  domain == nullptr: one-shot (roots built from the
// primitive root, or its inverse); else the caller's prepared domain.
static bool fft_entry(blst_p1* values, size_t n, const blst_fr* domain, bool inverse, bool scaled, size_t xn = 0)
{
    using namespace catmsm_host;
    Ctx* ctx = get_ctx();
    if (!ctx) return false;
    cudaStream_t st = ctx->stream;
    FftWork& W = ctx->fft;
    void* dv = W.values.get(n * sizeof(blst_p1));
    uint32_t* dr = (uint32_t*)W.roots.get((n + 2) * sizeof(blst_fr));
    if (!dv || !dr) return false;
    cudaError_t err = cudaSuccess;
    const uint32_t* scale = nullptr;
    bool inv_from_fwd = false;
    if (domain) {
        err = cudaMemcpyAsync(dr, domain, (n + 1) * sizeof(blst_fr), cudaMemcpyHostToDevice, st);
        inv_from_fwd = inverse;
        if (inverse && scaled) scale = dr + 8 * n;
    } else {
        hfr w = fr_root_of_unity(log2_exact(n));
        if (inverse) w = fr_inv(w);
        hfr* hw = (hfr*)ctx->h_out.get(2 * sizeof(hfr));
        if (!hw) return false;
        hw[0] = w;
        hw[1] = fr_inv(fr_from_u64(n));
        err = cudaMemcpyAsync(dr + 8 * n, hw, 2 * sizeof(hfr), cudaMemcpyHostToDevice, st);
        if (err == cudaSuccess) err = fft_root_powers(ctx, dr + 8 * n, n, dr);
        if (err == cudaSuccess && inverse) {
            err = cudaMemcpyAsync(dr + 8 * n, dr + 8 * n + 8, sizeof(hfr), cudaMemcpyDeviceToDevice, st);
            scale = dr + 8 * n;
        }
    }
    if (err == cudaSuccess) err = cudaMemcpyAsync(dv, values, n * sizeof(blst_p1), cudaMemcpyHostToDevice, st);
    if (err == cudaSuccess) err = fft_run(ctx, dv, n, dr, inv_from_fwd, scale, xn);
    // Results go to pinned staging first so a late failure leaves values untouched.
    void* hstage = nullptr;
    if (err == cudaSuccess) {
        hstage = ctx->h_values.get(n * sizeof(blst_p1));
        if (!hstage) err = cudaErrorMemoryAllocation;
    }
    if (err == cudaSuccess) err = cudaMemcpyAsync(hstage, dv, n * sizeof(blst_p1), cudaMemcpyDeviceToHost, st);
    if (err == cudaSuccess) err = cudaStreamSynchronize(st);
    if (err != cudaSuccess) return false;
    host_copy(values, hstage, n * sizeof(blst_p1));
    return true;
}

static bool domain_tag_ok(size_t n, const blst_fr* domain, size_t domain_len)
{
    if (!domain || !valid_fft_size(n) || domain_len != n + 2) return false;
    catmsm_host::hfr tag = catmsm_host::fr_from_u64(n);
    return std::memcmp(&domain[n + 1], tag.l, 32) == 0;
}

}  // namespace catmsm

using namespace catmsm;

extern "C" {

size_t blst_p1s_mult_pippenger_scratch_sizeof(size_t npoints)
{
    if (npoints == 0) return 0;
    return (size_t)192 << (ref_window(npoints) - 1);
}

size_t blst_p1s_mult_pippenger_window_scratch_sizeof(size_t window)
{
    if (window < 1 || window > 24) return 0;
    return (size_t)192 << (window - 1);
}

void blst_p1s_mult_pippenger(blst_p1* ret, const blst_p1_affine* const points[], size_t npoints,
                             const blst_byte* const scalars[], size_t nbits, blst_limb_t* scratch)
{
    try {
        msm_entry(ret, points, npoints, scalars, nbits, scratch, false, 0);
    } catch (...) {
        if (ret) write_inf(ret);
    }
}

void blst_p1s_mult_pippenger_window(blst_p1* ret, const blst_p1_affine* const points[], size_t npoints,
                                    const blst_byte* const scalars[], size_t nbits, blst_limb_t* scratch,
                                    size_t window)
{
    try {
        msm_entry(ret, points, npoints, scalars, nbits, scratch, true, window);
    } catch (...) {
        if (ret) write_inf(ret);
    }
}

void blst_p1s_tile_pippenger(blst_p1* ret, const blst_p1_affine* const points[], size_t npoints,
                             const blst_byte* const scalars[], size_t nbits, blst_limb_t* scratch, size_t bit0,
                             size_t window)
{
    try {
        if (!ret) return;
        write_inf(ret);
        if (npoints == 0 || !points || !scalars || !points[0] || !scalars[0] || !scratch || window < 1 ||
            window > 24 || nbits == 0 || nbits > 256 || bit0 >= nbits || npoints > 0x7fffffffu)
            return;
        Ctx* ctx = get_ctx();
        if (!ctx) return;
        const size_t nbytes = (nbits + 7) / 8;
        bool e1, e2;
        const uint8_t* hp = gather(points, npoints, sizeof(blst_p1_affine), ctx->h_points, e1);
        const uint8_t* hs = gather(scalars, npoints, nbytes, ctx->h_scalars, e2);
        if (e1 || e2) return;
        void* dp = ctx->msm.points.get(npoints * sizeof(blst_p1_affine));
        void* ds = ctx->msm.scalars.get(npoints * nbytes + 16);
        if (!dp || !ds) return;
        uint64_t out[18];
        cudaError_t err = cudaMemcpyAsync(dp, hp, npoints * sizeof(blst_p1_affine), cudaMemcpyHostToDevice, ctx->stream);
        if (err == cudaSuccess) err = cudaMemcpyAsync(ds, hs, npoints * nbytes, cudaMemcpyHostToDevice, ctx->stream);
        if (err == cudaSuccess)
            err = msm_tile_device(ctx, dp, (const uint8_t*)ds, (uint32_t)nbytes, npoints, (uint32_t)nbits,
                                  (uint32_t)bit0, (uint32_t)window, out);
        if (err == cudaSuccess) std::memcpy(ret, out, sizeof(*ret));
    } catch (...) {
        if (ret) write_inf(ret);
    }
}

size_t blst_fr_fft_domain_len(size_t n) { return valid_fft_size(n) ? n + 2 : 0; }

bool blst_fr_fft_domain_init(blst_fr* domain, size_t domain_len, size_t n)
{
    using namespace catmsm_host;
    try {
        if (!domain || !valid_fft_size(n) || domain_len != n + 2) return false;
        Ctx* ctx = get_ctx();
        if (!ctx) return false;
        uint32_t* dr = (uint32_t*)ctx->fft.roots.get((n + 1) * sizeof(blst_fr));
        hfr* hw = (hfr*)ctx->h_out.get(sizeof(hfr));
        if (!dr || !hw) return false;
        hw[0] = fr_root_of_unity(log2_exact(n));
        cudaError_t err = cudaMemcpyAsync(dr + 8 * n, hw, sizeof(hfr), cudaMemcpyHostToDevice, ctx->stream);
        if (err == cudaSuccess) err = fft_root_powers(ctx, dr + 8 * n, n, dr);
        if (err == cudaSuccess)
            err = cudaMemcpyAsync(domain, dr, n * sizeof(blst_fr), cudaMemcpyDeviceToHost, ctx->stream);
        if (err == cudaSuccess) err = cudaStreamSynchronize(ctx->stream);
        if (err != cudaSuccess) return false;
        hfr nn = fr_from_u64(n);
        hfr inv = fr_inv(nn);
        std::memcpy(&domain[n], inv.l, 32);
        std::memcpy(&domain[n + 1], nn.l, 32);
        return true;
    } catch (...) {
        return false;
    }
}

bool blst_p1_fft(blst_p1* values, size_t n, bool inverse)
{
    try {
        if (!values || !valid_fft_size(n)) return false;
        return fft_entry(values, n, nullptr, inverse, true);
    } catch (...) {
        return false;
    }
}

bool blst_p1_fft_with_domain(blst_p1* values, size_t n, const blst_fr* domain, size_t domain_len, bool inverse)
{
    try {
        if (!values || !domain_tag_ok(n, domain, domain_len)) return false;
        return fft_entry(values, n, domain, inverse, true);
    } catch (...) {
        return false;
    }
}

bool blst_p1_ifft_unscaled_with_domain(blst_p1* values, size_t n, const blst_fr* domain, size_t domain_len)
{
    try {
        if (!values || !domain_tag_ok(n, domain, domain_len)) return false;
        return fft_entry(values, n, domain, true, false);
    } catch (...) {
        return false;
    }
}

bool catmsm_p1_fft_truncated_prefix(blst_p1* values, size_t n, size_t xn, const blst_fr* domain,
                                    size_t domain_len)
{
    try {
        if (!values || !domain_tag_ok(n, domain, domain_len) || xn == 0 || xn > n) return false;
        // the contract: every element of [xn, n) is the identity (z == 0)
        static const uint8_t zero[sizeof(blst_fp)] = {0};
        for (size_t i = xn; i < n; i++)
            if (std::memcmp(&values[i].z, zero, sizeof(blst_fp)) != 0) return false;
        return fft_entry(values, n, domain, false, false, xn);
    } catch (...) {
        return false;
    }
}

int catmsm_p1_fft_batch(blst_p1* const values[], const size_t ns[], const blst_fr* const domains[],
                        const int modes[], size_t count)
{
    try {
        if (!values || !ns || !domains || !modes) return (int)cudaErrorInvalidValue;
        size_t total = 0;
        for (size_t i = 0; i < count; i++) {
            if (!values[i] || modes[i] < 0 || modes[i] > 2 || !domain_tag_ok(ns[i], domains[i], ns[i] + 2))
                return (int)cudaErrorInvalidValue;
            total += ns[i];
        }
        if (count == 0) return 0;
        if (total >= 0x7fffffffu) return (int)cudaErrorInvalidValue;
        Ctx* ctx = get_ctx();
        if (!ctx) return (int)cudaErrorInitializationError;
        cudaStream_t st = ctx->stream;
        // distinct domains are uploaded once
        std::vector<const blst_fr*> uniq;
        std::vector<size_t> uoff, dom_of(count);
        size_t rtot = 0;
        for (size_t i = 0; i < count; i++) {
            size_t u = 0;
            while (u < uniq.size() && uniq[u] != domains[i]) u++;
            if (u == uniq.size()) {
                uniq.push_back(domains[i]);
                uoff.push_back(rtot);
                rtot += ns[i] + 1;
            }
            dom_of[i] = u;
        }
        blst_p1* dv = (blst_p1*)ctx->fft.values.get(total * sizeof(blst_p1));
        uint32_t* dr = (uint32_t*)ctx->fft.roots.get(rtot * sizeof(blst_fr));
        void* hstage = ctx->h_values.get(total * sizeof(blst_p1));
        if (!dv || !dr || !hstage) return (int)cudaErrorMemoryAllocation;
        cudaError_t err = cudaSuccess;
        for (size_t u = 0; u < uniq.size() && err == cudaSuccess; u++) {
            size_t n = 0;
            for (size_t i = 0; i < count; i++)
                if (domains[i] == uniq[u]) n = ns[i];
            err = cudaMemcpyAsync(dr + 8 * uoff[u], uniq[u], (n + 1) * sizeof(blst_fr), cudaMemcpyHostToDevice, st);
        }
        std::vector<FftSpec> specs(count);
        size_t off = 0;
        for (size_t i = 0; i < count && err == cudaSuccess; i++) {
            const uint32_t* r = dr + 8 * uoff[dom_of[i]];
            specs[i] = FftSpec{ns[i], r, modes[i] != 0, modes[i] == 1 ? r + 8 * ns[i] : nullptr};
            err = cudaMemcpyAsync(dv + off, values[i], ns[i] * sizeof(blst_p1), cudaMemcpyHostToDevice, st);
            off += ns[i];
        }
        if (err == cudaSuccess) err = fft_run_multi(ctx, dv, specs.data(), count);
        if (err == cudaSuccess)
            err = cudaMemcpyAsync(hstage, dv, total * sizeof(blst_p1), cudaMemcpyDeviceToHost, st);
        if (err == cudaSuccess) err = cudaStreamSynchronize(st);
        if (err != cudaSuccess) return (int)err;
        off = 0;
        for (size_t i = 0; i < count; i++) {
            host_copy(values[i], (const blst_p1*)hstage + off, ns[i] * sizeof(blst_p1));
            off += ns[i];
        }
        return 0;
    } catch (...) {
        return (int)cudaErrorUnknown;
    }
}

int catmsm_p1s_mult_pippenger_device(blst_p1* ret, const void* d_points, const void* d_scalars, size_t stride,
                                     size_t npoints, size_t nbits, size_t window)
{
    if (!ret) return (int)cudaErrorInvalidValue;
    write_inf(ret);
    if (npoints == 0 || nbits == 0) return 0;
    if (!d_points || !d_scalars || nbits > 256 || stride < (nbits + 7) / 8 || window > 24 ||
        (reinterpret_cast<uintptr_t>(d_points) & 15) != 0)
        return (int)cudaErrorInvalidValue;
    Ctx* ctx = get_ctx();
    if (!ctx) return (int)cudaErrorInitializationError;
    uint64_t out[18];
    cudaError_t err = msm_device(ctx, d_points, (const uint8_t*)d_scalars, (uint32_t)stride, npoints,
                                 (uint32_t)nbits, (uint32_t)window, out);
    if (err != cudaSuccess) return (int)err;
    std::memcpy(ret, out, sizeof(*ret));
    return 0;
}

int catmsm_p1_fft_device(void* d_values, size_t n, const void* d_domain, int mode)
{
    if (!d_values || !d_domain || !valid_fft_size(n) || mode < 0 || mode > 2 ||
        (reinterpret_cast<uintptr_t>(d_values) & 15) != 0)
        return (int)cudaErrorInvalidValue;
    Ctx* ctx = get_ctx();
    if (!ctx) return (int)cudaErrorInitializationError;
    const uint32_t* dr = (const uint32_t*)d_domain;
    cudaError_t err = fft_run(ctx, d_values, n, dr, mode != 0, mode == 1 ? dr + 8 * n : nullptr);
    if (err == cudaSuccess) err = cudaStreamSynchronize(ctx->stream);
    return (int)err;
}

void* catmsm_stream(void)
{
    Ctx* ctx = get_ctx();
    return ctx ? (void*)ctx->stream : nullptr;
}

long catmsm_launch_count(void) { return g_stats.launches; }

size_t catmsm_msm_window(size_t npoints) { return msm_default_window(npoints); }

int catmsm_msm_glv(int enable)
{
    Ctx* ctx = get_ctx();
    if (!ctx) return -1;
    const int prev = ctx->glv ? 1 : 0;
    if (enable >= 0) ctx->glv = enable != 0;
    return prev;
}

int catmsm_msm_affine_rounds(int rounds)
{
    Ctx* ctx = get_ctx();
    if (!ctx) return -2;
    const int prev = ctx->affine_rounds;
    if (rounds >= -1 && rounds <= 8) ctx->affine_rounds = rounds;
    return prev;
}

int catmsm_msm_affine_rounds_for(size_t npoints, size_t nbits)
{
    Ctx* ctx = get_ctx();
    if (!ctx || npoints == 0 || nbits == 0 || nbits > 256) return -1;
    uint32_t c, D, chunk, fan_in;
    size_t pts;
    msm_plan_detail(npoints, (uint32_t)nbits, ctx->glv, &c, &D, &pts, &chunk, &fan_in);
    if (ctx->affine_rounds >= 0) return ctx->affine_rounds;
    return (int)msm_affine_rounds(pts * D, (size_t)D << (c - 1));
}

int catmsm_msm_plan_detail(size_t npoints, size_t nbits, int glv, size_t* window, size_t* windows, size_t* points,
                           size_t* chunk, size_t* fan_in)
{
    if (npoints == 0 || nbits == 0 || nbits > 256 || !window || !windows || !points || !chunk || !fan_in) return -1;
    uint32_t c, D, L, S;
    size_t np;
    msm_plan_detail(npoints, (uint32_t)nbits, glv != 0, &c, &D, &np, &L, &S);
    *window = c;
    *windows = D;
    *points = np;
    *chunk = L;
    *fan_in = S;
    return 0;
}

int catmsm_msm_plan(size_t npoints, size_t nbits, size_t* window, size_t* windows, size_t* points)
{
    Ctx* ctx = get_ctx();
    if (!ctx || npoints == 0 || nbits == 0 || nbits > 256 || !window || !windows || !points) return -1;
    uint32_t c, D;
    size_t np;
    msm_plan(ctx, npoints, (uint32_t)nbits, &c, &D, &np);
    *window = c;
    *windows = D;
    *points = np;
    return 0;
}

int catmsm_p1_affines_from_scalars_device(void* d_out, const void* d_k32, size_t n)
{
    Ctx* ctx = get_ctx();
    if (!ctx) return (int)cudaErrorInitializationError;
    cudaError_t err = points_from_scalars_device(ctx, (const uint8_t*)d_k32, n, d_out);
    if (err == cudaSuccess) err = cudaStreamSynchronize(ctx->stream);
    return (int)err;
}

int catmsm_p1_affines_from_scalars(blst_p1_affine* out, const blst_byte* k32, size_t n)
{
    if (n == 0) return 0;
    if (!out || !k32) return (int)cudaErrorInvalidValue;
    Ctx* ctx = get_ctx();
    if (!ctx) return (int)cudaErrorInitializationError;
    void* dk = ctx->msm.scalars.get(32 * n);
    void* dp = ctx->msm.points.get(sizeof(blst_p1_affine) * n);
    if (!dk || !dp) return (int)cudaErrorMemoryAllocation;
    cudaError_t err = cudaMemcpyAsync(dk, k32, 32 * n, cudaMemcpyHostToDevice, ctx->stream);
    if (err == cudaSuccess) err = points_from_scalars_device(ctx, (const uint8_t*)dk, n, dp);
    if (err == cudaSuccess)
        err = cudaMemcpyAsync(out, dp, sizeof(blst_p1_affine) * n, cudaMemcpyDeviceToHost, ctx->stream);
    if (err == cudaSuccess) err = cudaStreamSynchronize(ctx->stream);
    return (int)err;
}

int catmsm_fp_inv(blst_fp* out, const blst_fp* a, size_t n)
{
    if (n == 0) return 0;
    if (!out || !a) return (int)cudaErrorInvalidValue;
    Ctx* ctx = get_ctx();
    if (!ctx) return (int)cudaErrorInitializationError;
    uint64_t* d = (uint64_t*)ctx->msm.digits.get(2 * n * sizeof(blst_fp));
    if (!d) return (int)cudaErrorMemoryAllocation;
    cudaError_t err = cudaMemcpyAsync(d, a, n * sizeof(blst_fp), cudaMemcpyHostToDevice, ctx->stream);
    if (err == cudaSuccess) err = fp_inv_test_device(ctx, d, d + 6 * n, n);
    if (err == cudaSuccess)
        err = cudaMemcpyAsync(out, d + 6 * n, n * sizeof(blst_fp), cudaMemcpyDeviceToHost, ctx->stream);
    if (err == cudaSuccess) err = cudaStreamSynchronize(ctx->stream);
    return (int)err;
}

int catmsm_host_fp_inv(blst_fp* out, const blst_fp* a, size_t n)
{
    if (n && (!out || !a)) return -1;
    for (size_t i = 0; i < n; i++) {
        catmsm_host::hfp x, r;
        std::memcpy(x.l, &a[i], 48);
        catmsm_host::inv(r, x);
        std::memcpy(&out[i], r.l, 48);
    }
    return 0;
}

int catmsm_host_fp_sqr(blst_fp* out, const blst_fp* a, size_t n)
{
    if (n && (!out || !a)) return -1;
    for (size_t i = 0; i < n; i++) {
        catmsm_host::hfp x, r;
        std::memcpy(x.l, &a[i], 48);
        catmsm_host::canon(x);
        catmsm_host::sqr(r, x);
        std::memcpy(&out[i], r.l, 48);
    }
    return 0;
}

int catmsm_host_fp_mul(blst_fp* out, const blst_fp* a, const blst_fp* b, size_t n)
{
    if (n && (!out || !a || !b)) return -1;
    for (size_t i = 0; i < n; i++) {
        catmsm_host::hfp x, y, r;
        std::memcpy(x.l, &a[i], 48);
        std::memcpy(y.l, &b[i], 48);
        catmsm_host::canon(x);
        catmsm_host::canon(y);
        catmsm_host::mul(r, x, y);
        std::memcpy(&out[i], r.l, 48);
    }
    return 0;
}

int catmsm_fp_mul(blst_fp* out, const blst_fp* a, const blst_fp* b, size_t n)
{
    if (n == 0) return 0;
    Ctx* ctx = get_ctx();
    if (!ctx) return (int)cudaErrorInitializationError;
    uint64_t* d = (uint64_t*)ctx->msm.digits.get(3 * n * sizeof(blst_fp));
    if (!d) return (int)cudaErrorMemoryAllocation;
    cudaError_t err = cudaMemcpyAsync(d, a, n * sizeof(blst_fp), cudaMemcpyHostToDevice, ctx->stream);
    if (err == cudaSuccess) err = cudaMemcpyAsync(d + 6 * n, b, n * sizeof(blst_fp), cudaMemcpyHostToDevice, ctx->stream);
    if (err == cudaSuccess) err = fp_mul_test_device(ctx, d, d + 6 * n, d + 12 * n, n, a == b);
    if (err == cudaSuccess)
        err = cudaMemcpyAsync(out, d + 12 * n, n * sizeof(blst_fp), cudaMemcpyDeviceToHost, ctx->stream);
    if (err == cudaSuccess) err = cudaStreamSynchronize(ctx->stream);
    return (int)err;
}

}  // extern "C"
