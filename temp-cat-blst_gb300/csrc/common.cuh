// Shared host/device plumbing for the sm_103a BLS12-381 G1 library:
// per-thread CUDA context (stream, grow-only device and pinned buffers) and
// error helpers.  All public entry points are synchronous and fail closed.
#pragma once
#include <cuda_runtime.h>
#include <atomic>
#include <cstring>
#include <cstddef>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <thread>
#include <vector>

namespace catmsm {

// SMs of a GB300 (two dies of 76): used only by host-side plan models that
// run without a device; launches size their grids from device_sms().
constexpr int kGB300SMs = 152;

// SM count of the current device, queried once per device (devices past the
// cache are queried on every call); grids are sized in multiples of it.  The
// cache is shared by every calling thread: atomic entries, each written with
// the same value by whichever thread gets there first.
inline int device_sms()
{
    static std::atomic<int> cache[64];
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess) dev = -1;
    if (dev >= 0 && dev < 64) {
        const int v = cache[dev].load(std::memory_order_relaxed);
        if (v > 0) return v;
    }
    int sms = 0;
    if (dev < 0 || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms <= 0)
        return kGB300SMs;   // only reached with a broken context; the next launch reports the error
    if (dev < 64) cache[dev].store(sms, std::memory_order_relaxed);
    return sms;
}

struct DevBuf {
    void* p = nullptr;
    size_t cap = 0;
    void* get(size_t bytes)
    {
        if (bytes == 0) bytes = 256;
        if (bytes > cap) {
            if (p) cudaFree(p);
            p = nullptr;
            cap = 0;
            if (cudaMalloc(&p, bytes) != cudaSuccess) {
                p = nullptr;
                return nullptr;
            }
            cap = bytes;
        }
        return p;
    }
    void release()
    {
        if (p) cudaFree(p);
        p = nullptr;
        cap = 0;
    }
};

struct PinnedBuf {
    void* p = nullptr;
    size_t cap = 0;
    void* get(size_t bytes)
    {
        if (bytes == 0) bytes = 256;
        if (bytes > cap) {
            if (p) cudaFreeHost(p);
            p = nullptr;
            cap = 0;
            if (cudaHostAlloc(&p, bytes, cudaHostAllocDefault) != cudaSuccess) {
                p = nullptr;
                return nullptr;
            }
            cap = bytes;
        }
        return p;
    }
    void release()
    {
        if (p) cudaFreeHost(p);
        p = nullptr;
        cap = 0;
    }
};

// Device workspaces of one MSM pipeline instance.
struct MsmWork {
    DevBuf points, scalars, digits, ranks, counts, offsets, block_sums, sorted_pt, sorted_key,
        buckets, head, tail, seg, wins, total, status, misc, glv_pts, glv_sc, glv_sign;
    // batch-affine accumulation rounds (bucket_affine.cu)
    DevBuf aff_pts0, aff_pts1, aff_key0, aff_key1, aff_meta, aff_pairpos, aff_prefix, aff_ttot, aff_btot;
    void release()
    {
        for (DevBuf* b : {&points, &scalars, &digits, &ranks, &counts, &offsets, &block_sums, &sorted_pt,
                          &sorted_key, &buckets, &head, &tail, &seg, &wins, &total, &status, &misc, &glv_pts,
                          &glv_sc, &glv_sign, &aff_pts0, &aff_pts1, &aff_key0, &aff_key1, &aff_meta, &aff_pairpos,
                          &aff_prefix, &aff_ttot, &aff_btot})
            b->release();
    }
};

struct FftWork {
    DevBuf values, roots, glv, scratch, meta;
    void release()
    {
        for (DevBuf* b : {&values, &roots, &glv, &scratch, &meta}) b->release();
    }
};

// Per-stage CUDA-event timing of the MSM pipeline (off by default).
constexpr int kMsmStages = 8;   // prep (memsets, GLV scalar split), digits, scan, scatter (+ GLV points), accumulate, fixup, reduce, host fold
struct StageProfile {
    bool enabled = false;
    cudaEvent_t ev[kMsmStages + 1] = {};
    double ms[kMsmStages] = {};
    long calls = 0;
    double entries = 0;   // bucket entries (nonzero digits) accumulated
};

struct Ctx {
    int device = -1;
    cudaStream_t stream = nullptr;
    MsmWork msm;
    FftWork fft;
    PinnedBuf h_points, h_scalars, h_out, h_values, h_meta;
    StageProfile prof;
    bool glv = true;   // GLV split of scalars wider than 128 bits (catmsm_msm_glv)
    int affine_rounds = -1;   // batch-affine accumulation rounds (-1: by size; catmsm_msm_affine_rounds)
    cudaStream_t copy_stream = nullptr;    // host->device point copies that overlap the scalar stages
    cudaEvent_t points_ready = nullptr;
    // second half of the batch-affine rounds (bucket_affine.cu), forked from and joined to `stream`
    cudaStream_t aff_stream = nullptr;
    cudaEvent_t aff_fork = nullptr, aff_join = nullptr;
};

// Per-thread context bound to the thread's current device.  A thread's
// contexts (their streams, events and grow-only workspaces: ~15 GB after a
// 2^22-point MSM) are released when the thread exits; the main thread's are
// left to process teardown.
Ctx* get_ctx();

// Launch-time stats, readable through catmsm_last_launches() for the bench.
struct LaunchStats {
    int launches = 0;
};
extern thread_local LaunchStats g_stats;

#define CATMSM_CHECK(x)                    \
    do {                                   \
        cudaError_t e__ = (x);             \
        if (e__ != cudaSuccess) return e__; \
    } while (0)

inline unsigned div_up(size_t a, size_t b) { return (unsigned)((a + b - 1) / b); }

// Host copy between caller memory and pinned staging.  Large copies are
// split over up to 8 host threads: one core moves ~10-20 GB/s, and a batch's
// scalars or an FFT batch's values (tens of MB) would otherwise cost
// milliseconds next to a device pass of similar length.
inline void host_copy(void* dst, const void* src, size_t bytes)
{
    constexpr size_t kSplit = size_t(8) << 20;
    if (bytes < kSplit) {
        std::memcpy(dst, src, bytes);
        return;
    }
    unsigned nt = std::thread::hardware_concurrency();
    nt = nt < 2 ? 1 : (nt > 8 ? 8 : nt);
    if (nt == 1) {
        std::memcpy(dst, src, bytes);
        return;
    }
    const size_t part = ((bytes + nt - 1) / nt + 63) & ~size_t(63);
    std::vector<std::thread> th;
    th.reserve(nt);
    for (unsigned k = 0; k < nt; k++) {
        const size_t off = (size_t)k * part;
        if (off >= bytes) break;
        const size_t len = bytes - off < part ? bytes - off : part;
        try {
            th.emplace_back([=] { std::memcpy((char*)dst + off, (const char*)src + off, len); });
        } catch (...) {
            std::memcpy((char*)dst + off, (const char*)src + off, len);
        }
    }
    for (auto& t : th) t.join();
}

// Gather the descriptor walk of multi_scalar.cpp:830-841 into contiguous
// host staging; returns the contiguous base directly when possible.
// Rank of this lane's entry within bucket `key` (kNoBucket: no entry), with
// one atomic per distinct key of the warp: lanes that share a bucket take
// consecutive ranks.  Uniform scalars rarely share one (no measurable cost at
// 2^20); all-equal scalars or 0/1 coefficients put whole warps on one counter,
// which serialised the digit kernels (2^20 equal scalars: 1.93 -> 0.07 ms).
// All 32 lanes of the warp must call it together.
constexpr uint32_t kNoBucket = 0xffffffffu;

__device__ __forceinline__ uint32_t warp_bucket_rank(uint32_t key, uint32_t* counts)
{
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t peers = __match_any_sync(0xffffffffu, key);
    const uint32_t leader = __ffs(peers) - 1;
    uint32_t base = 0;
    if (key != kNoBucket && lane == leader) base = atomicAdd(&counts[key], (uint32_t)__popc(peers));
    base = __shfl_sync(0xffffffffu, base, leader);
    return base + __popc(peers & ((1u << lane) - 1));
}

template <typename T>
inline const uint8_t* gather(const T* const arr[], size_t n, size_t elem, PinnedBuf& stage, bool& err)
{
    err = false;
    if (n == 1 || arr[1] == nullptr) return reinterpret_cast<const uint8_t*>(arr[0]);
    uint8_t* dst = (uint8_t*)stage.get(n * elem);
    if (!dst) { err = true; return nullptr; }
    const uint8_t* cur = reinterpret_cast<const uint8_t*>(arr[0]);
    const T* const* next = arr + 1;
    std::memcpy(dst, cur, elem);
    for (size_t i = 1; i < n; i++) {
        if (*next) cur = reinterpret_cast<const uint8_t*>(*next++);
        else cur += elem;
        std::memcpy(dst + i * elem, cur, elem);
    }
    return dst;
}

}  // namespace catmsm
