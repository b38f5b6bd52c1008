// Batched commitments over a resident basis (no reference counterpart; the
// reference's closest API is the fixed-base wbits MSM, c_api.cpp:1310-1369).
//
// A basis of n affine points is uploaded once and expanded into fixed-base
// tables T[w][i] = 2^(c w) P_i (affine, w < D = 256/c + 1).  A batch of MSMs,
// MSM j over the first k_j basis points with 255/256-bit scalars, then needs
// no window fold: sum_i k_ji P_i = sum_i sum_w d_jiw T[w][i], so every
// (point, window) digit of MSM j drops into ONE set of 2^(c-1) buckets owned
// by that MSM.  The kernels of the plain pipeline (counting sort, chunked
// accumulation, fixup, running-sum reduction) run unchanged over the key
// space (msm, bucket); the reduction's root is each MSM's result.
//
// The device sequence of a batch (one launch per stage, sizes read from
// device memory) is captured once per (batch size, window, chunk) into a CUDA
// graph and replayed: one graph launch per batch.  A small autotuner times
// candidate (window, chunk) pairs on a caller batch and remembers the winner
// per (device, basis size, batch size, points-per-MSM class) in a text cache.
#include "common.cuh"
#include "curve.cuh"
#include "host_curve.hpp"
#include "catmsm_internal.h"
#include "catmsm_gpu.h"

#include <sys/stat.h>

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <new>
#include <string>
#include <vector>

namespace catmsm {

// plain-pipeline kernels (msm.cu)
__global__ void k_scan_local(const uint32_t* __restrict__ in, uint32_t* __restrict__ out,
                             uint32_t* __restrict__ block_sums, uint32_t M);
__global__ void k_scan_top(uint32_t* __restrict__ block_sums, uint32_t nb, uint32_t* __restrict__ total_out);
__global__ void k_scan_add(uint32_t* __restrict__ out, const uint32_t* __restrict__ block_sums, uint32_t M);
__global__ void k_accumulate(const affine* __restrict__ pts, const uint32_t* __restrict__ sorted_pt,
                             const uint32_t* __restrict__ sorted_key, const uint32_t* __restrict__ total_ptr,
                             uint32_t L, xyzz* __restrict__ buckets, xyzz* __restrict__ head,
                             xyzz* __restrict__ tail);
__global__ void k_fixup(const uint32_t* __restrict__ sorted_key, const uint32_t* __restrict__ offsets,
                        const uint32_t* __restrict__ total_ptr, uint32_t L, xyzz* __restrict__ buckets,
                        const xyzz* __restrict__ head, const xyzz* __restrict__ tail,
                        uint2* __restrict__ hot_list, uint32_t* __restrict__ hot_count);
__global__ void k_fixup_hot(uint2* __restrict__ hot_list, uint32_t* __restrict__ hot_count,
                            const uint32_t* __restrict__ offsets, uint32_t L, xyzz* __restrict__ buckets,
                            const xyzz* __restrict__ head, const xyzz* __restrict__ tail);
__global__ void k_fixup_seg(const uint32_t* __restrict__ sorted_key, const uint32_t* __restrict__ total_ptr,
                            uint32_t L, xyzz* __restrict__ head);
__global__ void k_fixup_join(const uint32_t* __restrict__ sorted_key, const uint32_t* __restrict__ offsets,
                             const uint32_t* __restrict__ total_ptr, uint32_t L, xyzz* __restrict__ buckets,
                             const xyzz* __restrict__ head, const xyzz* __restrict__ tail,
                             uint2* __restrict__ hot_list, uint32_t* __restrict__ hot_count);
__global__ void k_fixup_hot_seg(uint2* __restrict__ hot_list, uint32_t* __restrict__ hot_count,
                                const uint32_t* __restrict__ offsets, uint32_t L, xyzz* __restrict__ buckets,
                                const xyzz* __restrict__ head, const xyzz* __restrict__ tail);
__global__ void k_reduce_level(const xyzz* __restrict__ inA, const xyzz* __restrict__ inQ, uint32_t m_in,
                               uint32_t F, uint32_t lgF, uint32_t D, int first, xyzz* __restrict__ outA,
                               xyzz* __restrict__ outQ);

constexpr int kScanTileB = 1024 * 4;

// ---------------------------------------------------------------- tables
// T[w][i] = 2^(c w) P_i, one point per thread: D-1 runs of c doublings, then
// Montgomery's simultaneous inversion over the D multiples (one field
// inversion per point).  q: D xyzz scratch per point, pre: D prefix products.
__global__ void __launch_bounds__(64) k_build_tables(const affine* __restrict__ pts, uint32_t n, uint32_t c,
                                                     uint32_t D, affine* __restrict__ table, xyzz* __restrict__ tmp,
                                                     fp* __restrict__ pre_buf)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const affine p = pts[i];
    xyzz* q = tmp + (size_t)i * D;
    fp* pre = pre_buf + (size_t)i * D;
    xyzz acc;
    if (aff_is_inf(p)) {
        xyzz_set_inf(acc);
    } else {
        acc.x = p.x; acc.y = p.y;
        fp_set_one(acc.zz); fp_set_one(acc.zzz);
    }
    fp prod;
    fp_set_one(prod);
    for (uint32_t w = 0; w < D; w++) {
        if (w)
            for (uint32_t k = 0; k < c; k++) xyzz_dbl(acc);
        q[w] = acc;
        pre[w] = prod;
        if (!xyzz_is_inf(acc)) {
            fp t;
            fp_mul(t, acc.zz, acc.zzz);
            fp_mul(prod, prod, t);
        }
    }
    fp inv;
    fp_inv(inv, prod);                           // 1 / prod of all (zz zzz)
    for (int w = (int)D - 1; w >= 0; w--) {
        const xyzz e = q[w];
        affine o;
        if (xyzz_is_inf(e)) {
            fp_zero(o.x); fp_zero(o.y);
        } else {
            fp zz_zzz, ie, t;
            fp_mul(zz_zzz, e.zz, e.zzz);
            fp_mul(ie, inv, pre[w]);             // 1 / (zz zzz) of entry w
            fp_mul(inv, inv, zz_zzz);            // drop entry w from the running inverse
            fp_mul(t, ie, e.zzz);                // 1 / zz
            fp_mul(o.x, e.x, t);
            fp_mul(t, ie, e.zz);                 // 1 / zzz
            fp_mul(o.y, e.y, t);
            fp_canon(o.x, o.x);
            fp_canon(o.y, o.y);
        }
        table[(size_t)w * n + i] = o;
    }
}

// ---------------------------------------------------------------- digits
// One thread per (MSM, point) pair in flat order; off[j] = first pair of MSM
// j (off[nmsm] = total pairs).  Digits are the same signed c-bit recoding as
// the plain pipeline; the key is j * B + (|d| - 1) and the point index the
// table slot w * n + i.
__global__ void k_digits_batch(const uint8_t* __restrict__ scalars, const uint32_t* __restrict__ off,
                               uint32_t nmsm, uint32_t n, uint32_t nbits, uint32_t c, uint32_t D, uint32_t cap,
                               uint32_t* __restrict__ digits, uint32_t* __restrict__ ranks,
                               uint32_t* __restrict__ pidx, uint32_t* __restrict__ counts)
{
    const uint32_t f = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t P = off[nmsm];
    if (f >= P || f >= cap) return;
    uint32_t lo = 0, hi = nmsm;                   // find j with off[j] <= f < off[j+1]
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (off[mid] <= f) lo = mid;
        else hi = mid;
    }
    const uint32_t j = lo, i = f - off[j];
    const uint4 a = __ldg(reinterpret_cast<const uint4*>(scalars + (size_t)f * 32));
    const uint4 b = __ldg(reinterpret_cast<const uint4*>(scalars + (size_t)f * 32) + 1);
    uint32_t k[9] = {a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w, 0};
#pragma unroll
    for (uint32_t q = 0; q < 8; q++) {
        if (nbits <= 32 * q) k[q] = 0;
        else if (nbits < 32 * (q + 1)) k[q] &= (1u << (nbits - 32 * q)) - 1;
    }
    const uint32_t B = 1u << (c - 1);
    const uint32_t cmask = (1u << c) - 1;
    uint32_t carry = 0;
    for (uint32_t w = 0; w < D; w++) {
        const uint32_t bit = w * c, word = bit >> 5, sh = bit & 31;
        uint32_t raw = k[word] >> sh;
        if (sh && word + 1 < 9) raw |= k[word + 1] << (32 - sh);
        raw &= cmask;
        int32_t d = (int32_t)(raw + carry);
        if (d > (int32_t)B) { d -= (int32_t)(cmask + 1); carry = 1; }
        else carry = 0;
        const size_t o = (size_t)f * D + w;
        if (d == 0) {
            digits[o] = 0xffffffffu;
        } else {
            // plain atomics: an MSM of the batch has at most n points per
            // bucket, and warp aggregation cost more than it saved here
            const uint32_t mag = d < 0 ? (uint32_t)(-d) : (uint32_t)d;
            const uint32_t key = j * B + (mag - 1);
            ranks[o] = atomicAdd(&counts[key], 1u);
            digits[o] = key | (d < 0 ? 0x80000000u : 0u);
            pidx[o] = w * n + i;
        }
    }
}

__global__ void k_scatter_batch(const uint32_t* __restrict__ digits, const uint32_t* __restrict__ ranks,
                                const uint32_t* __restrict__ pidx, const uint32_t* __restrict__ offsets,
                                const uint32_t* __restrict__ off, uint32_t nmsm, uint32_t D, uint32_t cap,
                                uint32_t* __restrict__ sorted_pt, uint32_t* __restrict__ sorted_key)
{
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t nD = off[nmsm] * D;
    if (t >= nD || t >= cap) return;
    const uint32_t dg = digits[t];
    if (dg == 0xffffffffu) return;
    const uint32_t key = dg & 0x7fffffffu;
    const uint32_t pos = offsets[key] + ranks[t];
    sorted_pt[pos] = pidx[t] | (dg & 0x80000000u);
    sorted_key[pos] = key;
}

// results: root Q (xyzz) of each MSM -> Jacobian with canonical coordinates
__global__ void k_batch_out(const xyzz* __restrict__ roots, uint32_t nmsm, jac* __restrict__ out)
{
    const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= nmsm) return;
    xyzz p = roots[j];
    jac o;
    xyzz_to_jac(o, p);
    if (!fp_is_zero(o.z)) {
        fp_canon(o.x, o.x);
        fp_canon(o.y, o.y);
        fp_canon(o.z, o.z);
    } else {
        jac_set_inf(o);
    }
    out[j] = o;
}

// ---------------------------------------------------------------- basis object
struct BatchGraph {
    cudaGraphExec_t exec = nullptr;
    uint32_t nmsm = 0, c = 0, L = 0;
    size_t cap = 0;
};

// Device/pinned workspace of one batch pipeline instance (a basis has one;
// a server worker has its own, sharing the basis tables).
struct BatchWork {
    DevBuf scal, off, digits, ranks, pidx, counts, offsets, bsums, sorted_pt, sorted_key, buckets, head, tail,
        hot, seg, out;
    PinnedBuf h_scal, h_off, h_out;
    BatchGraph graph;
    void release()
    {
        if (graph.exec) cudaGraphExecDestroy(graph.exec);
        graph = BatchGraph();
        DevBuf* bufs[] = {&scal, &off, &digits, &ranks, &pidx, &counts, &offsets, &bsums, &sorted_pt,
                          &sorted_key, &buckets, &head, &tail, &hot, &seg, &out};
        for (DevBuf* d : bufs) d->release();
        PinnedBuf* hb[] = {&h_scal, &h_off, &h_out};
        for (PinnedBuf* h : hb) {
            if (h->p) cudaFreeHost(h->p);
            h->p = nullptr;
            h->cap = 0;
        }
    }
};

struct Basis {
    int device = -1;
    size_t n = 0;
    uint32_t c = 0, D = 0, L = 16;
    cudaStream_t stream = nullptr;
    DevBuf points, table, tmp;
    BatchWork work;
    std::mutex mu;     // serialises the direct calls (batches, reconfiguration, autotuning): they share the
                       // basis's workspace and stream, and a rebuild replaces the tables a batch reads
};

static cudaError_t build_tables(Basis* b, uint32_t c)
{
    const uint32_t D = 256 / c + 1;
    affine* table = (affine*)b->table.get((size_t)D * b->n * sizeof(affine));
    xyzz* tmp = (xyzz*)b->tmp.get((size_t)D * b->n * (sizeof(xyzz) + sizeof(fp)));
    if (!table || !tmp) return cudaErrorMemoryAllocation;
    k_build_tables<<<div_up(b->n, 64), 64, 0, b->stream>>>((const affine*)b->points.p, (uint32_t)b->n, c, D,
                                                          table, tmp, (fp*)(tmp + (size_t)D * b->n));
    CATMSM_CHECK(cudaGetLastError());
    CATMSM_CHECK(cudaStreamSynchronize(b->stream));
    b->tmp.release();
    b->c = c;
    b->D = D;
    if (b->work.graph.exec) {
        cudaGraphExecDestroy(b->work.graph.exec);
        b->work.graph = BatchGraph();
    }
    return cudaSuccess;
}

// Workspace for batches of up to nmsm MSMs and cap pairs.
static cudaError_t ensure_work(const Basis* b, BatchWork* w, uint32_t nmsm, size_t cap)
{
    const uint32_t B = 1u << (b->c - 1);
    const size_t M = (size_t)nmsm * B;
    const size_t nD = cap * b->D;
    const size_t chunks = (nD + b->L - 1) / b->L + 1;
    const size_t lvl1 = (size_t)nmsm * ((B + 7) / 8);
    const size_t lvl2 = (size_t)nmsm * ((B + 15) / 16) + nmsm;
    bool ok = w->scal.get(cap * 32) && w->off.get((nmsm + 1) * 4) && w->digits.get(nD * 4) &&
              w->ranks.get(nD * 4) && w->pidx.get(nD * 4) && w->counts.get(M * 4) && w->offsets.get((M + 1) * 4) &&
              w->bsums.get(((M + kScanTileB - 1) / kScanTileB) * 4 + 4) && w->sorted_pt.get(nD * 4) &&
              w->sorted_key.get(nD * 4) && w->buckets.get(M * sizeof(xyzz)) &&
              w->head.get(chunks * sizeof(xyzz)) && w->tail.get(chunks * sizeof(xyzz)) &&
              w->hot.get(256 + chunks * sizeof(uint2)) && w->seg.get(2 * (lvl1 + lvl2) * sizeof(xyzz)) &&
              w->out.get((size_t)nmsm * sizeof(jac)) && w->h_scal.get(cap * 32) && w->h_off.get((nmsm + 1) * 4) &&
              w->h_out.get((size_t)nmsm * sizeof(jac));
    return ok ? cudaSuccess : cudaErrorMemoryAllocation;
}

// The device sequence of one batch (everything after the input copies).
// Returns the number of kernels it launched.
static uint32_t enqueue_batch(const Basis* b, BatchWork* w, cudaStream_t st, uint32_t nmsm, size_t cap)
{
    const uint32_t c = b->c, D = b->D, L = b->L, B = 1u << (c - 1);
    const size_t M = (size_t)nmsm * B;
    const size_t nD = cap * D;
    const size_t chunks = (nD + L - 1) / L + 1;
    const uint32_t nblocks = (uint32_t)((M + kScanTileB - 1) / kScanTileB);
    const size_t lvl1 = (size_t)nmsm * ((B + 7) / 8);
    const size_t lvl2 = (size_t)nmsm * ((B + 15) / 16) + nmsm;
    uint32_t* off = (uint32_t*)w->off.p;
    uint32_t* counts = (uint32_t*)w->counts.p;
    uint32_t* offsets = (uint32_t*)w->offsets.p;
    uint32_t* total = offsets + M;
    uint32_t* hot_count = (uint32_t*)w->hot.p;
    uint2* hot_list = reinterpret_cast<uint2*>(hot_count + 64);
    xyzz* buckets = (xyzz*)w->buckets.p;
    xyzz* head = (xyzz*)w->head.p;
    xyzz* tail = (xyzz*)w->tail.p;
    xyzz* seg = (xyzz*)w->seg.p;
    cudaMemsetAsync(counts, 0, M * 4, st);
    cudaMemsetAsync(buckets, 0, M * sizeof(xyzz), st);
    cudaMemsetAsync(hot_count, 0, 12, st);
    k_digits_batch<<<div_up(cap, 256), 256, 0, st>>>((const uint8_t*)w->scal.p, off, nmsm, (uint32_t)b->n, 256, c,
                                                    D, (uint32_t)cap, (uint32_t*)w->digits.p,
                                                    (uint32_t*)w->ranks.p, (uint32_t*)w->pidx.p, counts);
    k_scan_local<<<nblocks, 1024, 0, st>>>(counts, offsets, (uint32_t*)w->bsums.p, (uint32_t)M);
    k_scan_top<<<1, 1024, 0, st>>>((uint32_t*)w->bsums.p, nblocks, total);
    k_scan_add<<<div_up(M, 256), 256, 0, st>>>(offsets, (uint32_t*)w->bsums.p, (uint32_t)M);
    k_scatter_batch<<<div_up(nD, 256), 256, 0, st>>>((const uint32_t*)w->digits.p, (const uint32_t*)w->ranks.p,
                                                    (const uint32_t*)w->pidx.p, offsets, off, nmsm, D,
                                                    (uint32_t)nD, (uint32_t*)w->sorted_pt.p,
                                                    (uint32_t*)w->sorted_key.p);
    k_accumulate<<<div_up(chunks, 128), 128, 0, st>>>((const affine*)b->table.p, (const uint32_t*)w->sorted_pt.p,
                                                      (const uint32_t*)w->sorted_key.p, total, L, buckets, head,
                                                      tail);
    k_fixup_seg<<<div_up(chunks, 128), 128, 0, st>>>((const uint32_t*)w->sorted_key.p, total, L, head);
    k_fixup_join<<<div_up(chunks, 128), 128, 0, st>>>((const uint32_t*)w->sorted_key.p, offsets, total, L, buckets,
                                                      head, tail, hot_list, hot_count);
    k_fixup_hot_seg<<<2 * device_sms(), 128, 0, st>>>(hot_list, hot_count, offsets, L, buckets, head, tail);
    fixup_giants(hot_list, hot_count, offsets, L, buckets, head, tail, true, st);
    xyzz* bufA[2] = {seg, seg + 2 * lvl1};
    xyzz* bufQ[2] = {seg + lvl1, seg + 2 * lvl1 + lvl2};
    const xyzz* inA = buckets;
    const xyzz* inQ = nullptr;
    uint32_t m = B, pp = 0, launches = 12;      // digits .. fixup giants (11) and batch_out
    bool first = true;
    while (m > 1) {
        launches++;
        if (!first && m <= msm_reduce_tail_max(nmsm)) {
            msm_reduce_tail(inA, inQ, m, nmsm, bufQ[pp], st);
            inQ = bufQ[pp];
            break;
        }
        const uint32_t F = first ? 8 : 2;
        const uint32_t m_out = (m + F - 1) / F;
        if (first)
            k_reduce_level<<<div_up((size_t)nmsm * m_out, 128), 128, 0, st>>>(inA, inQ, m, F, 3, nmsm, 1, bufA[pp],
                                                                              bufQ[pp]);
        else
            msm_reduce_pair(inA, inQ, m, nmsm, bufA[pp], bufQ[pp], st);
        inA = bufA[pp];
        inQ = bufQ[pp];
        pp ^= 1;
        m = m_out;
        first = false;
    }
    k_batch_out<<<div_up(nmsm, 128), 128, 0, st>>>(inQ ? inQ : inA, nmsm, (jac*)w->out.p);
    return launches;
}

// exact_cap: size the work for exactly the pairs of this batch (serving);
// otherwise for full-basis MSMs, so one captured graph serves every batch of
// the same size.
static cudaError_t run_batch(Basis* b, BatchWork* w, cudaStream_t st, blst_p1* out, uint32_t nmsm,
                             const size_t* counts, const uint8_t* scalars, bool use_graph, bool exact_cap)
{
    std::vector<uint32_t> off(nmsm + 1);
    size_t P = 0;
    for (uint32_t j = 0; j < nmsm; j++) {
        if (counts[j] > b->n) return cudaErrorInvalidValue;
        off[j] = (uint32_t)P;
        P += counts[j];
    }
    off[nmsm] = (uint32_t)P;
    const size_t cap = exact_cap ? (P ? P : 1) : (size_t)nmsm * b->n;
    if (cap * b->D >= 0x7fffffffu) return cudaErrorInvalidValue;
    CATMSM_CHECK(ensure_work(b, w, nmsm, cap));
    host_copy(w->h_scal.p, scalars, P * 32);
    std::memcpy(w->h_off.p, off.data(), (nmsm + 1) * 4);
    CATMSM_CHECK(cudaMemcpyAsync(w->scal.p, w->h_scal.p, P * 32, cudaMemcpyHostToDevice, st));
    CATMSM_CHECK(cudaMemcpyAsync(w->off.p, w->h_off.p, (nmsm + 1) * 4, cudaMemcpyHostToDevice, st));
    if (use_graph) {
        BatchGraph& g = w->graph;
        if (!g.exec || g.nmsm != nmsm || g.c != b->c || g.L != b->L || g.cap != cap) {
            if (g.exec) cudaGraphExecDestroy(g.exec);
            g = BatchGraph();
            cudaGraph_t graph;
            CATMSM_CHECK(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
            enqueue_batch(b, w, st, nmsm, cap);
            CATMSM_CHECK(cudaStreamEndCapture(st, &graph));
            cudaError_t e = cudaGraphInstantiate(&g.exec, graph, 0);
            cudaGraphDestroy(graph);
            CATMSM_CHECK(e);
            g.nmsm = nmsm;
            g.c = b->c;
            g.L = b->L;
            g.cap = cap;
        }
        CATMSM_CHECK(cudaGraphLaunch(g.exec, st));
        g_stats.launches += 1;
    } else {
        g_stats.launches += enqueue_batch(b, w, st, nmsm, cap);
    }
    CATMSM_CHECK(cudaGetLastError());
    CATMSM_CHECK(cudaMemcpyAsync(w->h_out.p, w->out.p, (size_t)nmsm * sizeof(jac), cudaMemcpyDeviceToHost, st));
    CATMSM_CHECK(cudaStreamSynchronize(st));
    std::memcpy(out, w->h_out.p, (size_t)nmsm * sizeof(jac));
    return cudaSuccess;
}

BatchWork* batch_work_new() { return new (std::nothrow) BatchWork(); }

void batch_work_free(BatchWork* w)
{
    if (!w) return;
    w->release();
    delete w;
}

cudaError_t batch_run(Basis* b, BatchWork* w, cudaStream_t st, blst_p1* out, uint32_t nmsm, const size_t* counts,
                      const uint8_t* scalars)
{
    return run_batch(b, w, st, out, nmsm, counts, scalars, false, true);
}

size_t basis_points(const Basis* b) { return b->n; }
uint32_t basis_window(const Basis* b) { return b->c; }
int basis_device(const Basis* b) { return b->device; }
const void* basis_points_device(const Basis* b) { return b->points.p; }

// ---------------------------------------------------------------- autotune cache
static std::mutex g_tune_mu;

static std::string tune_path()
{
    const char* p = std::getenv("CATMSM_TUNE_CACHE");
    if (p && *p) return p;
    const char* home = std::getenv("HOME");
    return std::string(home && *home ? home : "/tmp") + "/.cache/catmsm_tune.txt";
}

static std::string tune_key(size_t n, uint32_t nmsm, size_t pairs)
{
    char name[256] = "gpu";
    cudaDeviceProp prop;
    int dev = 0;
    if (cudaGetDevice(&dev) == cudaSuccess && cudaGetDeviceProperties(&prop, dev) == cudaSuccess)
        std::snprintf(name, sizeof(name), "%s", prop.name);
    for (char* q = name; *q; q++)
        if (*q == ' ') *q = '_';
    // points-per-MSM class: log2 of the mean, rounded
    const double mean = nmsm ? (double)pairs / nmsm : 0;
    int cls = 0;
    while ((double)(1u << (cls + 1)) <= mean) cls++;
    char key[384];
    std::snprintf(key, sizeof(key), "%s n=%zu nmsm=%u mean2^%d", name, n, nmsm, cls);
    return key;
}

static bool tune_lookup(const std::string& key, uint32_t* c, uint32_t* L)
{
    std::lock_guard<std::mutex> lk(g_tune_mu);
    FILE* f = std::fopen(tune_path().c_str(), "r");
    if (!f) return false;
    char line[512];
    bool found = false;
    while (std::fgets(line, sizeof(line), f)) {
        char* bar = std::strchr(line, '|');
        if (!bar) continue;
        *bar = 0;
        unsigned cc = 0, ll = 0;
        if (key == line && std::sscanf(bar + 1, "%u %u", &cc, &ll) == 2) {
            *c = cc;
            *L = ll;
            found = true;
        }
    }
    std::fclose(f);
    return found;
}

static void tune_store(const std::string& key, uint32_t c, uint32_t L)
{
    std::lock_guard<std::mutex> lk(g_tune_mu);
    const std::string path = tune_path();
    for (size_t pos = path.find('/', 1); pos != std::string::npos; pos = path.find('/', pos + 1))
        mkdir(path.substr(0, pos).c_str(), 0755);    // existing directories are fine
    FILE* f = std::fopen(path.c_str(), "a");
    if (!f) return;
    std::fprintf(f, "%s|%u %u\n", key.c_str(), c, L);
    std::fclose(f);
}

}  // namespace catmsm

using namespace catmsm;

extern "C" {

void* catmsm_basis_create(const blst_p1_affine* points, size_t n, size_t window)
{
    if (!points || n == 0 || n > (1u << 24) || window > 20 || (window != 0 && window < 2)) return nullptr;
    Basis* b = new (std::nothrow) Basis();
    if (!b) return nullptr;
    if (cudaGetDevice(&b->device) != cudaSuccess || msm_setup_device() != cudaSuccess ||
        cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess) {
        delete b;
        return nullptr;
    }
    b->n = n;
    void* dp = b->points.get(n * sizeof(affine));
    if (!dp || cudaMemcpy(dp, points, n * sizeof(affine), cudaMemcpyHostToDevice) != cudaSuccess ||
        build_tables(b, window ? (uint32_t)window : 11) != cudaSuccess) {
        catmsm_basis_destroy(b);
        return nullptr;
    }
    return b;
}

void catmsm_basis_destroy(void* handle)
{
    Basis* b = (Basis*)handle;
    if (!b) return;
    b->work.release();
    b->points.release();
    b->table.release();
    b->tmp.release();
    if (b->stream) cudaStreamDestroy(b->stream);
    delete b;
}

int catmsm_basis_config(void* handle, size_t* window, size_t* chunk)
{
    Basis* b = (Basis*)handle;
    if (!b) return (int)cudaErrorInvalidValue;
    std::lock_guard<std::mutex> lk(b->mu);
    if (window) *window = b->c;
    if (chunk) *chunk = b->L;
    return 0;
}

// catmsm_basis_set_config with b->mu held by the caller.
static int set_config_locked(Basis* b, size_t window, size_t chunk)
{
    if (window < 2 || window > 20 || chunk < 2 || chunk > 256) return (int)cudaErrorInvalidValue;
    b->L = (uint32_t)chunk;
    if (window != b->c) return (int)build_tables(b, (uint32_t)window);
    return 0;
}

int catmsm_basis_set_config(void* handle, size_t window, size_t chunk)
{
    Basis* b = (Basis*)handle;
    if (!b) return (int)cudaErrorInvalidValue;
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess || dev != b->device) return (int)cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lk(b->mu);
    return set_config_locked(b, window, chunk);
}

int catmsm_basis_msm_batch(void* handle, blst_p1* out, size_t nmsm, const size_t* counts, const blst_byte* scalars,
                           int use_graph)
{
    Basis* b = (Basis*)handle;
    if (!b || !out || !counts || (!scalars && nmsm) || nmsm == 0 || nmsm > (1u << 20)) return (int)cudaErrorInvalidValue;
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess || dev != b->device) return (int)cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lk(b->mu);
    return (int)run_batch(b, &b->work, b->stream, out, (uint32_t)nmsm, counts, scalars, use_graph != 0, false);
}

int catmsm_basis_autotune(void* handle, size_t nmsm, const size_t* counts, const blst_byte* scalars, int force)
{
    Basis* b = (Basis*)handle;
    if (!b || !counts || !scalars || nmsm == 0) return (int)cudaErrorInvalidValue;
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess || dev != b->device) return (int)cudaErrorInvalidDevice;
    size_t pairs = 0;
    for (size_t j = 0; j < nmsm; j++) pairs += counts[j];
    const std::string key = tune_key(b->n, (uint32_t)nmsm, pairs);
    uint32_t c = 0, L = 0;
    std::lock_guard<std::mutex> lk(b->mu);       // the whole sweep: it reconfigures and runs the basis
    if (!force && tune_lookup(key, &c, &L)) return set_config_locked(b, c, L);
    std::vector<blst_p1> out(nmsm);
    cudaEvent_t e0, e1;
    CATMSM_CHECK(cudaEventCreate(&e0));
    CATMSM_CHECK(cudaEventCreate(&e1));
    float best = 1e30f;
    uint32_t bc = b->c, bl = b->L;
    const uint32_t cs[] = {9, 10, 11, 12, 13};
    const uint32_t ls[] = {8, 16, 32, 48, 64, 96, 128, 192, 256};   // chunk lengths (96 measured best at 1024 x ~1.4k)
    for (uint32_t cc : cs) {
        for (uint32_t ll : ls) {
            if (set_config_locked(b, cc, ll) != 0) continue;
            if (run_batch(b, &b->work, b->stream, out.data(), (uint32_t)nmsm, counts, scalars, true, false) !=
                cudaSuccess)
                continue;
            float tot = 0.f;
            for (int r = 0; r < 2; r++) {
                cudaEventRecord(e0, b->stream);
                if (run_batch(b, &b->work, b->stream, out.data(), (uint32_t)nmsm, counts, scalars, true, false) !=
                    cudaSuccess)
                    break;
                cudaEventRecord(e1, b->stream);
                cudaEventSynchronize(e1);
                float ms = 0.f;
                cudaEventElapsedTime(&ms, e0, e1);
                tot += ms;
            }
            if (tot < best) {
                best = tot;
                bc = cc;
                bl = ll;
            }
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    int rc = set_config_locked(b, bc, bl);
    if (rc == 0) tune_store(key, bc, bl);
    return rc;
}

}  // extern "C"
