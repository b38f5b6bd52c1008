// An MSM entry point that allocates nothing.
//
// Who needs it: callers that must not (or cannot) allocate device memory at
// call time.  Typical cases are a process where another framework has
// reserved nearly all of the GPU's memory in its own pool, so a cudaMalloc
// from this library would fail or fragment that pool; and latency-critical
// code that cannot afford cudaMalloc/cudaFree, which may synchronise the whole
// device.  The regular entry points grow per-thread workspaces on demand; this
// one instead works inside one fixed scratch array that the CUDA runtime
// reserves when the library is loaded, and it also avoids pinned host buffers,
// streams it would have to create, and any host heap allocation.
//
// Limits and sharing rules:
//  * at most CATMSM_NOALLOC_MAX_POINTS (4096) points and nbits <= 256; larger calls are
//    rejected with CATMSM_NOALLOC_TOO_LARGE and write infinity;
//  * the scratch array (7,167,488 bytes of device memory) is held by every GPU
//    that loads the library, until the process exits;
//  * all calls share that one array and it keeps the previous call's
//    contents: every region that must start at zero is cleared by each call;
//  * calls that overlap on the GPU (from several host threads, or on several
//    streams) race on the shared array and give wrong results: serialise them;
//  * the first call on each device looks up the array's device address
//    (cudaGetSymbolAddress) with that device current.  With the CUDA
//    runtime's default lazy module loading, that lookup is also the moment
//    the device reserves the array: make the first call on each device early,
//    before another framework claims the GPU's memory (or it can fail with an
//    out-of-memory error although the call itself allocates nothing) and
//    before any stream capture;
//  * devices are indexed 0..63 (a call on a device with a higher index
//    returns cudaErrorInvalidDevice);
//  * a call that fails after queueing work waits for that work before it
//    returns, so a caller that serialises calls on the host never overlaps
//    them on the GPU.
// The kernels are the regular pipeline's (msm.cu); only the workspace differs.
#include "common.cuh"
#include "curve.cuh"
#include "host_curve.hpp"
#include "catmsm_internal.h"
#include "catmsm_gpu.h"

#include <cstring>
#include <mutex>

namespace catmsm {

// kernels of the regular pipeline (defined in msm.cu)
__global__ void k_digits(const uint8_t* __restrict__ scalars, uint32_t stride, uint32_t n, uint32_t nbits,
                         uint32_t c, uint32_t D, uint32_t* __restrict__ digits, uint32_t* __restrict__ ranks,
                         uint32_t* __restrict__ counts);
__global__ void k_scan_local(const uint32_t* __restrict__ in, uint32_t* __restrict__ out,
                             uint32_t* __restrict__ block_sums, uint32_t M);
__global__ void k_scan_top(uint32_t* __restrict__ block_sums, uint32_t nb, uint32_t* __restrict__ total_out);
__global__ void k_scan_add(uint32_t* __restrict__ out, const uint32_t* __restrict__ block_sums, uint32_t M);
__global__ void k_scatter(const uint32_t* __restrict__ digits, const uint32_t* __restrict__ ranks,
                          const uint32_t* __restrict__ offsets, uint32_t n, uint32_t nD,
                          uint32_t* __restrict__ sorted_pt, uint32_t* __restrict__ sorted_key);
__global__ void k_accumulate(const affine* __restrict__ pts, const uint32_t* __restrict__ sorted_pt,
                             const uint32_t* __restrict__ sorted_key, const uint32_t* __restrict__ total_ptr,
                             uint32_t L, xyzz* __restrict__ buckets, xyzz* __restrict__ head,
                             xyzz* __restrict__ tail);
__global__ void k_fixup(const uint32_t* __restrict__ sorted_key, const uint32_t* __restrict__ offsets,
                        const uint32_t* __restrict__ total_ptr, uint32_t L, xyzz* __restrict__ buckets,
                        const xyzz* __restrict__ head, const xyzz* __restrict__ tail,
                        uint2* __restrict__ hot_list, uint32_t* __restrict__ hot_count, uint32_t cap);
__global__ void k_fixup_rest(const uint2* __restrict__ hot_list, const uint32_t* __restrict__ hot_count,
                             uint32_t cap, const uint32_t* __restrict__ offsets, uint32_t L,
                             xyzz* __restrict__ buckets, const xyzz* __restrict__ head);
__global__ void k_fixup_hot(uint2* __restrict__ hot_list, uint32_t* __restrict__ hot_count,
                            const uint32_t* __restrict__ offsets, uint32_t L, xyzz* __restrict__ buckets,
                            const xyzz* __restrict__ head, const xyzz* __restrict__ tail);
__global__ void k_reduce_level(const xyzz* __restrict__ inA, const xyzz* __restrict__ inQ, uint32_t m_in,
                               uint32_t F, uint32_t lgF, uint32_t D, int first, xyzz* __restrict__ outA,
                               xyzz* __restrict__ outQ);

namespace {

// Fixed plan: window c = 8 (128 buckets per window), chunks of 16 entries.
constexpr size_t kMaxPoints = CATMSM_NOALLOC_MAX_POINTS;
constexpr uint32_t kC = 8;
constexpr uint32_t kB = 1u << (kC - 1);
constexpr uint32_t kMaxD = 256 / kC + 1;
constexpr size_t kM = (size_t)kMaxD * kB;
constexpr size_t kND = kMaxPoints * kMaxD;
constexpr uint32_t kL = 16;
constexpr size_t kChunks = (kND + kL - 1) / kL;
// A bucket holds at most kMaxPoints entries, so its carries span at most
// kMaxPoints / kL + 1 chunks: within k_fixup_hot's block join (1024
// partials), and the grid-wide joins of the regular pipeline are not needed.
static_assert(kMaxPoints / kL + 1 <= 1024, "noalloc buckets must stay within the block join");
constexpr size_t kLvl1 = (size_t)kMaxD * (kB / 8);
constexpr size_t kLvl2 = (size_t)kMaxD * (kB / 16) + kMaxD;

constexpr size_t al(size_t x) { return (x + 255) & ~(size_t)255; }

// byte offsets of the regions inside the scratch array
constexpr size_t oPoints = 0;
constexpr size_t oScalars = oPoints + al(kMaxPoints * 96);
constexpr size_t oDigits = oScalars + al(kMaxPoints * 32);
constexpr size_t oRanks = oDigits + al(kND * 4);
constexpr size_t oCounts = oRanks + al(kND * 4);
constexpr size_t oOffsets = oCounts + al(kM * 4);
constexpr size_t oBsums = oOffsets + al((kM + 1) * 4);
constexpr size_t oSortedPt = oBsums + al(((kM + kScanTile - 1) / kScanTile) * 4);
constexpr size_t oSortedKey = oSortedPt + al(kND * 4);
constexpr size_t oBuckets = oSortedKey + al(kND * 4);
constexpr size_t oHead = oBuckets + al(kM * sizeof(xyzz));
constexpr size_t oTail = oHead + al(kChunks * sizeof(xyzz));
constexpr size_t oHot = oTail + al(kChunks * sizeof(xyzz));
constexpr size_t oSeg = oHot + al(256 + kChunks * sizeof(uint2));
constexpr size_t oWins = oSeg + al(2 * (kLvl1 + kLvl2) * sizeof(xyzz));
constexpr size_t kScratchBytes = oWins + al((size_t)kMaxD * sizeof(xyzz));

}  // namespace

// The whole workspace of catmsm_p1s_mult_pippenger_noalloc.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

// Device address of g_noalloc_scratch per device, looked up once per device.
static unsigned char* g_noalloc_ptr[64];
static std::mutex g_noalloc_mu;

static cudaError_t noalloc_setup(unsigned char** out)
{
    int dev = 0;
    CATMSM_CHECK(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    if (!g_noalloc_ptr[dev]) {
        void* p = nullptr;
        CATMSM_CHECK(cudaGetSymbolAddress(&p, g_noalloc_scratch));
        g_noalloc_ptr[dev] = static_cast<unsigned char*>(p);
    }
    *out = g_noalloc_ptr[dev];
    return cudaSuccess;
}

// Queues the whole pipeline on st; the D window sums land in h_wins once st
// is synchronised.
static cudaError_t noalloc_queue(unsigned char* base, const blst_p1_affine* points, const blst_byte* scalars,
                                 size_t n, uint32_t nbits, cudaStream_t st, uint64_t* h_wins)
{
    const uint32_t D = nbits / kC + 1;
    const size_t M = (size_t)D * kB;
    const size_t nD = n * D;
    const size_t chunks = (nD + kL - 1) / kL;
    const uint32_t nbytes = (nbits + 7) / 8;
    const uint32_t nblocks = (uint32_t)((M + kScanTile - 1) / kScanTile);

    affine* d_pts = reinterpret_cast<affine*>(base + oPoints);
    uint8_t* d_sc = base + oScalars;
    uint32_t* digits = reinterpret_cast<uint32_t*>(base + oDigits);
    uint32_t* ranks = reinterpret_cast<uint32_t*>(base + oRanks);
    uint32_t* counts = reinterpret_cast<uint32_t*>(base + oCounts);
    uint32_t* offsets = reinterpret_cast<uint32_t*>(base + oOffsets);
    uint32_t* bsums = reinterpret_cast<uint32_t*>(base + oBsums);
    uint32_t* sorted_pt = reinterpret_cast<uint32_t*>(base + oSortedPt);
    uint32_t* sorted_key = reinterpret_cast<uint32_t*>(base + oSortedKey);
    xyzz* buckets = reinterpret_cast<xyzz*>(base + oBuckets);
    xyzz* head = reinterpret_cast<xyzz*>(base + oHead);
    xyzz* tail = reinterpret_cast<xyzz*>(base + oTail);
    uint32_t* hot_count = reinterpret_cast<uint32_t*>(base + oHot);
    uint2* hot_list = reinterpret_cast<uint2*>(base + oHot + 256);
    xyzz* seg = reinterpret_cast<xyzz*>(base + oSeg);
    xyzz* wins = reinterpret_cast<xyzz*>(base + oWins);
    uint32_t* total = offsets + M;

    CATMSM_CHECK(cudaMemcpyAsync(d_pts, points, n * sizeof(blst_p1_affine), cudaMemcpyHostToDevice, st));
    CATMSM_CHECK(cudaMemcpyAsync(d_sc, scalars, n * nbytes, cudaMemcpyHostToDevice, st));
    // regions read before they are written in this call start at zero
    CATMSM_CHECK(cudaMemsetAsync(counts, 0, M * 4, st));
    CATMSM_CHECK(cudaMemsetAsync(buckets, 0, M * sizeof(xyzz), st));
    CATMSM_CHECK(cudaMemsetAsync(hot_count, 0, 12, st));
    k_digits<<<div_up(n, 256), 256, 0, st>>>(d_sc, nbytes, (uint32_t)n, nbits, kC, D, digits, ranks, counts);
    k_scan_local<<<nblocks, kScanThreads, 0, st>>>(counts, offsets, bsums, (uint32_t)M);
    k_scan_top<<<1, kScanThreads, 0, st>>>(bsums, nblocks, total);
    k_scan_add<<<div_up(M, 256), 256, 0, st>>>(offsets, bsums, (uint32_t)M);
    k_scatter<<<div_up(nD, 256), 256, 0, st>>>(digits, ranks, offsets, (uint32_t)n, (uint32_t)nD, sorted_pt,
                                              sorted_key);
    k_accumulate<<<div_up(chunks, 128), 128, 0, st>>>(d_pts, sorted_pt, sorted_key, total, kL, buckets, head, tail);
    k_fixup<<<div_up(chunks, 128), 128, 0, st>>>(sorted_key, offsets, total, kL, buckets, head, tail, hot_list,
                                                 hot_count, (uint32_t)kChunks);
    k_fixup_hot<<<device_sms(), 128, 0, st>>>(hot_list, hot_count, offsets, kL, buckets, head, tail);
    k_fixup_rest<<<device_sms(), 128, 0, st>>>(hot_list, hot_count, (uint32_t)kChunks, offsets, kL, buckets, head);
    xyzz* bufA[2] = {seg, seg + 2 * kLvl1};
    xyzz* bufQ[2] = {seg + kLvl1, seg + 2 * kLvl1 + kLvl2};
    const xyzz* inA = buckets;
    const xyzz* inQ = nullptr;
    uint32_t m = kB, pp = 0;
    bool first = true;
    while (m > 1) {
        const uint32_t F = first ? 8 : 2, lgF = first ? 3 : 1;
        const uint32_t m_out = (m + F - 1) / F;
        k_reduce_level<<<div_up((size_t)D * m_out, 128), 128, 0, st>>>(inA, inQ, m, F, lgF, D, first ? 1 : 0,
                                                                      bufA[pp], bufQ[pp]);
        inA = bufA[pp];
        inQ = bufQ[pp];
        pp ^= 1;
        m = m_out;
        first = false;
    }
    CATMSM_CHECK(cudaMemcpyAsync(wins, inQ, (size_t)D * sizeof(xyzz), cudaMemcpyDeviceToDevice, st));
    CATMSM_CHECK(cudaGetLastError());
    CATMSM_CHECK(cudaMemcpyAsync(h_wins, wins, (size_t)D * sizeof(xyzz), cudaMemcpyDeviceToHost, st));
    return cudaSuccess;
}

static cudaError_t noalloc_run(const blst_p1_affine* points, const blst_byte* scalars, size_t n, uint32_t nbits,
                               uint64_t out[18])
{
    unsigned char* base = nullptr;
    CATMSM_CHECK(noalloc_setup(&base));
    cudaStream_t st = cudaStreamPerThread;
    const uint32_t D = nbits / kC + 1;
    uint64_t h_wins[kMaxD * 24];
    const cudaError_t qerr = noalloc_queue(base, points, scalars, n, nbits, st, h_wins);
    // wait also when queueing failed part-way: work already queued may still
    // be using the shared array, and the next call must not overlap it
    const cudaError_t serr = cudaStreamSynchronize(st);
    if (qerr != cudaSuccess) return qerr;
    CATMSM_CHECK(serr);

    using namespace catmsm_host;
    hjac ret;
    std::memset(&ret, 0, sizeof(ret));
    for (uint32_t w = D; w-- > 0;) {
        hjac tile;
        from_device_xyzz(tile, h_wins + (size_t)w * 24);
        jac_add(ret, ret, tile);
        if (w)
            for (uint32_t i = 0; i < kC; i++) jac_dbl(ret, ret);
    }
    hjac norm;
    normalize(norm, ret);
    std::memcpy(out, &norm, 144);
    return cudaSuccess;
}

}  // namespace catmsm

extern "C" int catmsm_p1s_mult_pippenger_noalloc(blst_p1* ret, const blst_p1_affine* points, size_t npoints,
                                                 const blst_byte* scalars, size_t nbits)
{
    if (!ret) return CATMSM_NOALLOC_BAD_ARGUMENT;
    std::memset(ret, 0, sizeof(*ret));
    if (npoints == 0 || nbits == 0) return 0;
    if (npoints > catmsm::kMaxPoints || nbits > 256) return CATMSM_NOALLOC_TOO_LARGE;
    if (!points || !scalars) return CATMSM_NOALLOC_BAD_ARGUMENT;
    uint64_t out[18];
    const cudaError_t err = catmsm::noalloc_run(points, scalars, npoints, (uint32_t)nbits, out);
    if (err != cudaSuccess) return (int)err;
    std::memcpy(ret, out, sizeof(*ret));
    return 0;
}
