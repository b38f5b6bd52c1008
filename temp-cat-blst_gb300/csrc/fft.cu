// BLS12-381 G1 group-valued FFT on sm_103a.
//
// Drop-in for blst_p1_fft / blst_p1_fft_with_domain /
// blst_p1_ifft_unscaled_with_domain (reference fft_c_api.cpp:51-103,
// fft/ctFft.h:32-124, fft/context.h:182-215).  The transform is the same
// radix-2 decimation-in-time schedule with the same root indexing
// (root j * n/len, or n - j * n/len when the inverse reads forward roots), so
// outputs equal the reference's for any root table the caller supplies.
//
// Device layout: the Jacobian points (blst_p1 bytes, 144 B) of one or many
// transforms, concatenated in HBM; a job descriptor per transform.
//   k_roots_prepare    per root index: Montgomery Fr -> canonical -> GLV
//                      halves (k = k1 + lambda k2), stored as 8 words.
//   k_bitrev_multi     out-of-place bit-reversal permutation of every job.
//   k_fft_stage_multi  one launch per stage level for ALL jobs that have the
//                      level (a batch of transforms fills the GPU where one
//                      small transform cannot); inside a job, threads map
//                      first onto the non-trivial butterflies (j >= 1, one
//                      GLV scalar multiplication each), then onto the
//                      j == 0 butterflies, so a warp rarely mixes the two.
//                      Early stages (32 or more active groups) put the lanes
//                      of a warp on one root (width-5 NAF halves); later
//                      ones on consecutive roots (signed 5-bit fixed
//                      windows, the same digit positions for every root).
//                      Launches small enough to fit one wave at four lanes
//                      per butterfly use quad point operations.
//   k_fft_finish_multi the inverse 1/n scale (one GLV multiplication per
//                      element of scaled jobs) and canonical coordinates.
// Each butterfly is ~1.7k Fp multiplications (~1M IMAD) against 576 bytes of
// traffic, so large stages are IMAD-bound and read/write straight from
// HBM/L2; staging tiles in shared memory would save nothing measurable.
#include "common.cuh"
#include "curve.cuh"
#include "fr.cuh"
#include "catmsm_internal.h"

#include <cstring>
#include <vector>

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

// A batch of transforms shares one launch per stage level.  Job descriptor:
struct FftJob {
    uint32_t val_off;    // first element of this transform in the values buffer
    uint32_t n, logn;
    uint32_t glv_off;    // first prepared root (8 words each); glv_off + n: the scale
    int32_t inv_from_fwd;
    int32_t scaled;
    uint32_t xn;         // inputs [xn, n) are the identity: stage s runs only the
                         // min(xn, n / 2^s) groups holding a non-identity input
    uint32_t pad;
};

// thread t of a launch over per-job ranges: find the job whose range holds t
// (pre: exclusive prefix of the ranges, `cnt` entries; ids: job per entry)
__device__ __forceinline__ uint32_t find_range(const uint32_t* __restrict__ pre, uint32_t cnt, uint32_t t)
{
    uint32_t lo = 0, hi = cnt;
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (pre[mid] <= t) lo = mid;
        else hi = mid;
    }
    return lo;
}

__global__ void k_bitrev_multi(const jac* __restrict__ in, jac* __restrict__ out, const FftJob* __restrict__ jobs,
                               const uint32_t* __restrict__ pre, uint32_t njobs, uint32_t total)
{
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= total) return;
    const FftJob J = jobs[find_range(pre, njobs, t)];
    const uint32_t i = t - J.val_off;
    const uint32_t r = J.logn ? (__brev(i) >> (32 - J.logn)) : 0;
    jac p;
    load_jac(p, in + t);
    store_jac(out + J.val_off + r, p);
}

// Stage `len` over every job with n >= len.  lst: for this stage, pairs of
// (job id, exclusive prefix of n/2 butterflies), `cnt` entries.  Quad = true:
// a quad of lanes per butterfly (quad point operations), for stages with too
// few butterflies to fill the GPU, where the ~0.9M-cycle chain of one scalar
// multiplication, not the multiplier throughput, sets the stage time.
template <bool Quad>
__global__ void __launch_bounds__(64) k_fft_stage_multi(jac* __restrict__ a, const FftJob* __restrict__ jobs,
                                                        const uint32_t* __restrict__ lst_job,
                                                        const uint32_t* __restrict__ lst_pre, uint32_t cnt,
                                                        uint32_t total, uint32_t len, const uint32_t* __restrict__ glv)
{
    const uint32_t gt = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t t = Quad ? gt >> 2 : gt;
    if (t >= total) return;
    const quad_lane ql = quad_of(threadIdx.x & 31);
    const uint32_t e = find_range(lst_pre, cnt, t);
    const FftJob J = jobs[lst_job[e]];
    const uint32_t b = t - lst_pre[e];
    const uint32_t half = len >> 1;
    const uint32_t groups = J.n / len;
    const uint32_t active = min(groups, J.xn);
    const uint32_t nontriv = active * (half - 1);
    // Non-trivial butterflies: with at least 32 active groups (a multiple of
    // 32), the group index runs fastest, so the lanes of a warp share j and
    // its root and take the width-5 NAF multiplication; otherwise j runs
    // fastest and the lanes, on different roots, keep the fixed windows.
    uint32_t g, j;
    bool shared = false;
    if (b < nontriv) {
        if (!Quad && (active & 31u) == 0) {
            j = 1 + b / active;
            g = b % active;
            shared = true;
        } else {
            g = b / (half - 1);
            j = 1 + b % (half - 1);
        }
    } else {
        g = b - nontriv;
        j = 0;
    }
    // After the bit-reversal permutation, position p holds input bitrev(p);
    // group g of this stage (positions g len .. g len + len - 1) holds a
    // non-identity input iff bitrev(g) over log2(groups) bits is below xn, so
    // the active groups are the bit reversals of 0 .. active - 1.
    if (active < groups) g = __brev(g) >> (32 - (J.logn - (31 - __clz(len))));
    jac* base = a + J.val_off;
    const uint32_t i0 = g * len + j, i1 = i0 + half;
    jac u, v;
    load_jac(u, base + i0);
    load_jac(v, base + i1);
    if (j) {
        uint32_t idx = j * (J.n / len);
        if (J.inv_from_fwd) idx = J.n - idx;
        const uint32_t* r = glv + 8 * (size_t)(J.glv_off + idx);
        if (Quad) jac_mult_glv_quad(v, v, r, r + 4, ql);
        else if (shared) jac_mult_glv_shared(v, v, r, r + 4);
        else jac_mult_glv(v, v, r, r + 4);
    }
    jac s = u;
    if (Quad) {
        jac_add_quad(s, v, ql);
        jac_neg(v);
        jac_add_quad(u, v, ql);
        if (ql.k == 0) store_jac(base + i0, s);
        if (ql.k == 1) store_jac(base + i1, u);
    } else {
        jac_add(s, v);
        jac_neg(v);
        jac_add(u, v);
        store_jac(base + i0, s);
        store_jac(base + i1, u);
    }
}

// inverse scale (jobs with scaled != 0) and canonicalisation of every element
template <bool Quad>
__global__ void __launch_bounds__(64) k_fft_finish_multi(jac* __restrict__ a, const FftJob* __restrict__ jobs,
                                                         const uint32_t* __restrict__ pre, uint32_t njobs,
                                                         uint32_t total, const uint32_t* __restrict__ glv,
                                                         int do_scale)
{
    const uint32_t gt = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t t = Quad ? gt >> 2 : gt;
    if (t >= total) return;
    const quad_lane ql = quad_of(threadIdx.x & 31);
    const FftJob J = jobs[find_range(pre, njobs, t)];
    jac v;
    load_jac(v, a + t);
    if (do_scale && J.scaled) {
        const uint32_t* r = glv + 8 * (size_t)(J.glv_off + J.n);
        if (Quad) jac_mult_glv_quad(v, v, r, r + 4, ql);
        else jac_mult_glv_shared(v, v, r, r + 4);        // one scale per job, shared by its lanes
    }
    if (jac_is_inf(v)) {
        jac_set_inf(v);
    } else {
        fp_canon(v.x, v.x);
        fp_canon(v.y, v.y);
        fp_canon(v.z, v.z);
    }
    if (!Quad || ql.k == 0) store_jac(a + t, v);
}

// Launches with at most this many scalar multiplications use quads: four
// lanes each still fit in one wave of resident threads, and the stage time is
// one multiplication's latency, which quads cut ~1.8x.  Larger launches are
// throughput-bound and keep one lane per butterfly (quads cost ~1.6x the
// multiplier work).
static size_t fft_quad_max()
{
    static std::atomic<size_t> by_dev[64];          // shared by every calling thread
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev >= 0 && dev < 64) {
        const size_t v = by_dev[dev].load(std::memory_order_relaxed);
        if (v) return v;
    }
    int sms = 0, per_sm = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_fft_stage_multi<true>, 64, 0);
    size_t v = (sms > 0 && per_sm > 0) ? (size_t)sms * per_sm * 64 / 4 : (size_t)device_sms() * 64;
    if (dev >= 0 && dev < 64) by_dev[dev].store(v, std::memory_order_relaxed);
    return v;
}

// Runs every job of `specs` over the concatenated values in d_values
// (job i at element offset sum_{j<i} n_j); results land back in d_values.
cudaError_t fft_run_multi(Ctx* ctx, void* d_values, const FftSpec* specs, size_t count)
{
    cudaStream_t st = ctx->stream;
    FftWork& W = ctx->fft;
    std::vector<FftJob> jobs(count);
    std::vector<uint32_t> vpre(count + 1);
    size_t total = 0, glv_total = 0;
    uint32_t maxlog = 0;
    bool any_scale = false;
    for (size_t i = 0; i < count; i++) {
        const size_t n = specs[i].n;
        uint32_t lg = 0;
        while (((size_t)1 << lg) < n) lg++;
        jobs[i].val_off = (uint32_t)total;
        jobs[i].n = (uint32_t)n;
        jobs[i].logn = lg;
        jobs[i].inv_from_fwd = specs[i].inv_from_fwd ? 1 : 0;
        jobs[i].scaled = specs[i].scale_mont ? 1 : 0;
        jobs[i].glv_off = (uint32_t)glv_total;
        jobs[i].xn = (uint32_t)(specs[i].xn && specs[i].xn < n ? specs[i].xn : n);
        jobs[i].pad = 0;
        vpre[i] = (uint32_t)total;
        total += n;
        glv_total += n + 1;
        maxlog = lg > maxlog ? lg : maxlog;
        any_scale |= specs[i].scale_mont != nullptr;
    }
    vpre[count] = (uint32_t)total;
    if (total >= 0x7fffffffu) return cudaErrorInvalidValue;
    // per-stage (job, prefix) lists
    std::vector<uint32_t> lst_job, lst_pre, st_off(maxlog + 2), st_cnt(maxlog + 2), st_tot(maxlog + 2);
    for (uint32_t s = 1; s <= maxlog; s++) {
        st_off[s] = (uint32_t)lst_job.size();
        uint32_t acc = 0;
        for (size_t i = 0; i < count; i++) {
            if (jobs[i].logn >= s) {
                lst_job.push_back((uint32_t)i);
                lst_pre.push_back(acc);
                const uint32_t groups = jobs[i].n >> s;
                acc += (groups < jobs[i].xn ? groups : jobs[i].xn) << (s - 1);
            }
        }
        st_cnt[s] = (uint32_t)lst_job.size() - st_off[s];
        st_tot[s] = acc;
    }
    const size_t meta_words = count * (sizeof(FftJob) / 4) + (count + 1) + 2 * lst_job.size() + 8;
    jac* tmp = (jac*)W.scratch.get(total * sizeof(jac));
    uint32_t* glv = (uint32_t*)W.glv.get(glv_total * 32);
    uint32_t* meta = (uint32_t*)W.meta.get(meta_words * 4);
    uint32_t* hmeta = (uint32_t*)ctx->h_meta.get(meta_words * 4);
    if (!tmp || !glv || !meta || !hmeta) return cudaErrorMemoryAllocation;
    uint32_t* hp = hmeta;
    std::memcpy(hp, jobs.data(), count * sizeof(FftJob));
    hp += count * (sizeof(FftJob) / 4);
    std::memcpy(hp, vpre.data(), (count + 1) * 4);
    hp += count + 1;
    if (!lst_job.empty()) {
        std::memcpy(hp, lst_job.data(), lst_job.size() * 4);
        std::memcpy(hp + lst_job.size(), lst_pre.data(), lst_pre.size() * 4);
    }
    CATMSM_CHECK(cudaMemcpyAsync(meta, hmeta, meta_words * 4, cudaMemcpyHostToDevice, st));
    const FftJob* d_jobs = reinterpret_cast<const FftJob*>(meta);
    const uint32_t* d_vpre = meta + count * (sizeof(FftJob) / 4);
    const uint32_t* d_lst_job = d_vpre + count + 1;
    const uint32_t* d_lst_pre = d_lst_job + lst_job.size();
    // prepared roots per job (jobs sharing a root table share the work only
    // through the L2; preparation is O(n) next to O(n log n) scalar mults)
    for (size_t i = 0; i < count; i++) {
        k_roots_prepare<<<div_up(jobs[i].n, 256), 256, 0, st>>>(specs[i].roots_mont, jobs[i].n, glv + 8 * (size_t)jobs[i].glv_off);
        if (specs[i].scale_mont)
            k_roots_prepare<<<1, 32, 0, st>>>(specs[i].scale_mont, 1, glv + 8 * (size_t)(jobs[i].glv_off + jobs[i].n));
        g_stats.launches += 1 + (specs[i].scale_mont ? 1 : 0);
    }
    k_bitrev_multi<<<div_up(total, 256), 256, 0, st>>>((const jac*)d_values, tmp, d_jobs, d_vpre, (uint32_t)count,
                                                       (uint32_t)total);
    g_stats.launches++;
    const size_t qmax = fft_quad_max();
    for (uint32_t s = 1; s <= maxlog; s++) {
        if (st_tot[s] <= qmax)
            k_fft_stage_multi<true><<<div_up(4 * (size_t)st_tot[s], 64), 64, 0, st>>>(
                tmp, d_jobs, d_lst_job + st_off[s], d_lst_pre + st_off[s], st_cnt[s], st_tot[s], 1u << s, glv);
        else
            k_fft_stage_multi<false><<<div_up(st_tot[s], 64), 64, 0, st>>>(
                tmp, d_jobs, d_lst_job + st_off[s], d_lst_pre + st_off[s], st_cnt[s], st_tot[s], 1u << s, glv);
        g_stats.launches++;
    }
    if (any_scale && total <= qmax)
        k_fft_finish_multi<true><<<div_up(4 * total, 64), 64, 0, st>>>(tmp, d_jobs, d_vpre, (uint32_t)count,
                                                                       (uint32_t)total, glv, 1);
    else
        k_fft_finish_multi<false><<<div_up(total, 64), 64, 0, st>>>(tmp, d_jobs, d_vpre, (uint32_t)count,
                                                                    (uint32_t)total, glv, any_scale ? 1 : 0);
    g_stats.launches++;
    CATMSM_CHECK(cudaGetLastError());
    CATMSM_CHECK(cudaMemcpyAsync(d_values, tmp, total * sizeof(jac), cudaMemcpyDeviceToDevice, st));
    return cudaSuccess;
}

// single transform: d_values n Jacobian points; d_roots_mont the n
// Montgomery roots the butterflies index; d_scale_mont optional scale
cudaError_t fft_run(Ctx* ctx, void* d_values, size_t n, const uint32_t* d_roots_mont, bool inv_from_fwd,
                    const uint32_t* d_scale_mont, size_t xn)
{
    FftSpec sp{n, d_roots_mont, inv_from_fwd, d_scale_mont, xn};
    return fft_run_multi(ctx, d_values, &sp, 1);
}

cudaError_t fft_root_powers(Ctx* ctx, const uint32_t* d_w_mont, size_t n, uint32_t* d_out)
{
    k_root_powers<<<div_up(n, 256), 256, 0, ctx->stream>>>(d_w_mont, (uint32_t)n, d_out);
    g_stats.launches++;
    return cudaGetLastError();
}

}  // namespace catmsm
