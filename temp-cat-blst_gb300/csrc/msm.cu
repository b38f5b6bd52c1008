// BLS12-381 G1 Pippenger MSM on sm_103a.
//
// Drop-in for blst_p1s_mult_pippenger (reference c_api.cpp:1382-1418,
// multi_scalar.cpp:806-923).  The result is the same group element
// sum_i (k_i mod 2^nbits) * P_i; the device pipeline is:
//
//   0. k_glv_scalars (scalars wider than 128 bits) the GLV split: the points
//                    are prime-order subgroup elements (the reference's
//                    contract, blst_scalar.h:539), where phi(x, y) =
//                    (beta x, y) = lambda P, so k P = s1 m1 P + s2 m2 phi(P)
//                    with m1, m2 < 2^127: an n-point 255-bit MSM becomes a
//                    2n-point 127-bit MSM with the same bucket entries and
//                    half the windows to reduce and fold.  k_glv_points
//                    writes the signed points +-P, +-phi(P) just before the
//                    accumulation, so a host copy of the points can overlap
//                    the scalar stages.
//   1. k_digits      signed c-bit window digits (carry recoding, digit in
//                    [-2^(c-1), 2^(c-1)]), one thread per scalar; each nonzero
//                    digit takes a rank in its bucket (one atomicAdd per
//                    bucket and warp).
//   2. k_scan_*      exclusive scan of the D * 2^(c-1) bucket counts.
//   3. k_scatter     counting-sort scatter of (point index | sign) into bucket
//                    order, plus each entry's bucket key.
//   4. k_accumulate  load-balanced bucket accumulation: every thread owns a
//                    fixed chunk of L sorted entries and folds runs of equal
//                    keys with XYZZ mixed adds; runs that cross a chunk edge
//                    go to head/tail carry slots.
//   5. k_fixup (+ k_fixup_hot), or k_fixup_seg / k_fixup_join (+
//                    k_fixup_hot_seg) when buckets average more than two
//                    chunks: join the carry slots of buckets that span
//                    chunks; long spans go to a hot list joined by a warp
//                    (quad point operations) or, above 160 partials, a block.
//   6. k_reduce_level / k_reduce_pair / k_reduce_tail  sum_d d * S_d per
//                    window as a tree of running sums (no scalar
//                    multiplications): fan-in 8 (or the pair rule, for few
//                    buckets) over the buckets, then fan-in 2 levels with the
//                    Q and A of a node on two warps, quads on small levels,
//                    and the last levels of every window in one launch.
//   8. host          folds the D window sums: ret = 2^c ret + W_w, top first
//                    (reference multi_scalar.cpp:913-922), then normalises.
#include "common.cuh"
#include "curve.cuh"
#include "fr.cuh"
#include "host_curve.hpp"
#include "catmsm_internal.h"

#include <algorithm>
#include <cmath>
#include <mutex>

namespace catmsm {

thread_local LaunchStats g_stats;

// ----------------------------------------------------------------- 1. digits
// k = the low nbits bits of a little-endian scalar of `stride` bytes
__device__ __forceinline__ void load_scalar(uint32_t* k, const uint8_t* s, uint32_t stride, uint32_t nbits)
{
#pragma unroll
    for (int j = 0; j < 8; j++) k[j] = 0;
    const uint32_t nbytes = (nbits + 7) >> 3;
    if (stride == 32 && (reinterpret_cast<uintptr_t>(s) & 15) == 0) {
        const uint4 a = __ldg(reinterpret_cast<const uint4*>(s));
        const uint4 b = __ldg(reinterpret_cast<const uint4*>(s) + 1);
        k[0] = a.x; k[1] = a.y; k[2] = a.z; k[3] = a.w;
        k[4] = b.x; k[5] = b.y; k[6] = b.z; k[7] = b.w;
    } else if (stride == 16 && (reinterpret_cast<uintptr_t>(s) & 15) == 0) {
        const uint4 a = __ldg(reinterpret_cast<const uint4*>(s));
        k[0] = a.x; k[1] = a.y; k[2] = a.z; k[3] = a.w;
    } else {
        for (uint32_t b = 0; b < nbytes; b++) k[b >> 2] |= (uint32_t)s[b] << (8 * (b & 3));
    }
#pragma unroll
    for (uint32_t j = 0; j < 8; j++) {
        if (nbits <= 32 * j) k[j] = 0;
        else if (nbits < 32 * (j + 1)) k[j] &= (1u << (nbits - 32 * j)) - 1;
    }
}

// ----------------------------------------------------------------- 0. GLV split
// Thread i: k = k_i mod r = k1 + k2 lambda (0 <= k1 < lambda, k2 <= lambda + 1),
// balanced to k = s1 m1 + s2 m2 lambda with m1, m2 <= (lambda + 1) / 2:
//   k1 >= (lambda+1)/2:  k1 -> k1 - lambda,  k2 -> k2 + 1
//   k2 >= (lambda+1)/2:  k2 -> k2 - lambda - 1,  k1 -> k1 - 1
// (the second uses lambda^2 = -lambda - 1 mod r).  Writes the 16-byte
// magnitudes m1 -> gsc[i], m2 -> gsc[n + i] and the signs s1 | s2 << 1 ->
// sgn[i].  Needs only the scalars, so it runs while the points may still be
// in flight from the host.
__global__ void k_glv_scalars(const uint8_t* __restrict__ scalars, uint32_t stride, uint32_t n, uint32_t nbits,
                              uint4* __restrict__ gsc, uint8_t* __restrict__ sgn)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    uint32_t k[8];
    load_scalar(k, scalars + (size_t)i * stride, stride, nbits);
    uint32_t m1[4], m2[4];
    bool s1, s2;
    fr_glv_balanced(m1, m2, s1, s2, k);
    gsc[i] = make_uint4(m1[0], m1[1], m1[2], m1[3]);
    gsc[n + i] = make_uint4(m2[0], m2[1], m2[2], m2[3]);
    sgn[i] = (uint8_t)((s1 ? 1 : 0) | (s2 ? 2 : 0));
}

// The signed points of the split: s1 P -> gpts[i], s2 phi(P) -> gpts[n + i].
__global__ void k_glv_points(const affine* __restrict__ pts, const uint8_t* __restrict__ sgn, uint32_t n,
                             affine* __restrict__ gpts)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t sg = sgn[i];
    affine p;
    load_affine(p.x, p.y, pts + i);
    affine a = p, b = p;
    if (!aff_is_inf(p)) {
        fp beta;
#pragma unroll
        for (int w = 0; w < 12; w++) beta.v[w] = FP_BETA[w];
        fp_mul(b.x, p.x, beta);
        fp_canon(b.x, b.x);
        if (sg & 1) fp_neg(a.y, p.y);
        if (sg & 2) fp_neg(b.y, p.y);
    }
    store_affine(gpts + i, a);
    store_affine(gpts + n + i, b);
}

__global__ void k_digits(const uint8_t* __restrict__ scalars, uint32_t stride, uint32_t n,
                         uint32_t nbits, uint32_t c, uint32_t D, uint32_t* __restrict__ digits,
                         uint32_t* __restrict__ ranks, uint32_t* __restrict__ counts)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    const bool valid = i < n;
    uint32_t k[9];
    if (valid) load_scalar(k, scalars + (size_t)i * stride, stride, nbits);
    else
        for (int j = 0; j < 8; j++) k[j] = 0;
    k[8] = 0;
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
        const size_t o = (size_t)w * n + i;
        const uint32_t mag = d < 0 ? (uint32_t)(-d) : (uint32_t)d;
        const uint32_t key = (valid && d != 0) ? w * B + (mag - 1) : kNoBucket;
        const uint32_t rank = warp_bucket_rank(key, counts);
        if (!valid) continue;
        if (d == 0) {
            digits[o] = 0xffffffffu;
        } else {
            ranks[o] = rank;
            digits[o] = key | (d < 0 ? 0x80000000u : 0u);
        }
    }
}

// One window of the reference's tile (blst_p1s_tile_pippenger, c_api.cpp:
// 1585-1612 -> multi_scalar.cpp:806-864; WindowExtract, multi_scalar.h:
// 350-404): bits [bit0, bit0 + window) of each scalar with the bit below as
// the overlap (none at bit0 = 0), Booth-encoded over enc = min(nbits - bit0
// + 1, window) bits: digit magnitude in [0, 2^(enc-1)], bucket |d| - 1.
__global__ void k_tile_digits(const uint8_t* __restrict__ scalars, uint32_t stride, uint32_t n, uint32_t nbits,
                              uint32_t bit0, uint32_t window, uint32_t enc, uint32_t* __restrict__ digits,
                              uint32_t* __restrict__ ranks, uint32_t* __restrict__ counts)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    const bool valid = i < n;
    uint32_t k[9];
    if (valid) load_scalar(k, scalars + (size_t)i * stride, stride, nbits);
    else
        for (int j = 0; j < 8; j++) k[j] = 0;
    k[8] = 0;
    const uint32_t begin = bit0 > 0 ? bit0 - 1 : 0;
    const uint32_t endb = min(bit0 + window, nbits);
    const uint32_t size = endb - begin;                    // <= 25
    const uint32_t word = begin >> 5, sh = begin & 31;
    uint32_t v = k[word] >> sh;
    if (sh && word + 1 < 9) v |= k[word + 1] << (32 - sh);
    v &= (1u << size) - 1;
    if (bit0 == 0) v <<= 1;                                 // no overlap bit below bit 0
    const uint32_t sign = (v >> enc) & 1;
    const uint32_t val = (v + 1) >> 1;
    const uint32_t mag = sign ? (1u << enc) - val : val;
    const uint32_t key = (valid && mag != 0) ? mag - 1 : kNoBucket;
    const uint32_t rank = warp_bucket_rank(key, counts);
    if (!valid) return;
    if (mag == 0) {
        digits[i] = 0xffffffffu;
        return;
    }
    ranks[i] = rank;
    digits[i] = key | (sign ? 0x80000000u : 0u);
}

// ----------------------------------------------------------------- 2. scan

__device__ __forceinline__ uint32_t block_exclusive_scan(uint32_t v, uint32_t* smem_warp, uint32_t* total)
{
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    uint32_t x = v;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        uint32_t y = __shfl_up_sync(0xffffffffu, x, d);
        if (lane >= d) x += y;
    }
    if (lane == 31) smem_warp[wid] = x;
    __syncthreads();
    if (wid == 0) {
        const int nw = blockDim.x >> 5;
        uint32_t t = lane < nw ? smem_warp[lane] : 0;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            uint32_t y = __shfl_up_sync(0xffffffffu, t, d);
            if (lane >= d) t += y;
        }
        if (lane < nw) smem_warp[lane] = t;
    }
    __syncthreads();
    const uint32_t warp_prefix = wid ? smem_warp[wid - 1] : 0;
    *total = smem_warp[(blockDim.x >> 5) - 1];
    return warp_prefix + x - v;
}

__global__ void __launch_bounds__(kScanThreads) k_scan_local(const uint32_t* __restrict__ in,
                                                              uint32_t* __restrict__ out,
                                                              uint32_t* __restrict__ block_sums, uint32_t M)
{
    __shared__ uint32_t sw[32];
    const size_t base = (size_t)blockIdx.x * kScanTile + (size_t)threadIdx.x * kScanPer;
    uint32_t v[kScanPer], s = 0;
#pragma unroll
    for (int j = 0; j < kScanPer; j++) {
        v[j] = base + j < M ? in[base + j] : 0;
        s += v[j];
    }
    uint32_t total;
    uint32_t pre = block_exclusive_scan(s, sw, &total);
#pragma unroll
    for (int j = 0; j < kScanPer; j++) {
        if (base + j < M) out[base + j] = pre;
        pre += v[j];
    }
    if (threadIdx.x == 0) block_sums[blockIdx.x] = total;
}

// Single block: exclusive scan of the block sums; writes grand total to *total_out.
__global__ void __launch_bounds__(kScanThreads) k_scan_top(uint32_t* __restrict__ block_sums, uint32_t nb,
                                                            uint32_t* __restrict__ total_out)
{
    __shared__ uint32_t sw[32];
    const uint32_t per = (nb + kScanThreads - 1) / kScanThreads;
    const uint32_t b0 = threadIdx.x * per;
    uint32_t s = 0;
    for (uint32_t j = 0; j < per; j++)
        if (b0 + j < nb) s += block_sums[b0 + j];
    uint32_t total;
    uint32_t pre = block_exclusive_scan(s, sw, &total);
    for (uint32_t j = 0; j < per; j++) {
        if (b0 + j < nb) {
            uint32_t t = block_sums[b0 + j];
            block_sums[b0 + j] = pre;
            pre += t;
        }
    }
    if (threadIdx.x == 0) *total_out = total;
}

__global__ void k_scan_add(uint32_t* __restrict__ out, const uint32_t* __restrict__ block_sums, uint32_t M)
{
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < M) out[i] += block_sums[i / kScanTile];
}

// ----------------------------------------------------------------- 3. scatter
__global__ void k_scatter(const uint32_t* __restrict__ digits, const uint32_t* __restrict__ ranks,
                          const uint32_t* __restrict__ offsets, uint32_t n, uint32_t nD,
                          uint32_t* __restrict__ sorted_pt, uint32_t* __restrict__ sorted_key)
{
    const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= nD) return;
    const uint32_t dg = digits[j];
    if (dg == 0xffffffffu) return;
    const uint32_t key = dg & 0x7fffffffu;
    const uint32_t pos = offsets[key] + ranks[j];
    sorted_pt[pos] = (j % n) | (dg & 0x80000000u);
    sorted_key[pos] = key;
}

// ----------------------------------------------------------------- 4. accumulate
__device__ __forceinline__ void madd_entry(xyzz& acc, const affine* __restrict__ pts, uint32_t v)
{
    fp x, y;
    load_affine(x, y, pts + (v & 0x7fffffffu));
    if (fp_is_zero_raw(x) && fp_is_zero_raw(y)) return;   // infinity contributes nothing
    if (v >> 31) fp_neg(y, y);
    xyzz_madd(acc, x, y);
}

__global__ void __launch_bounds__(128, 4) k_accumulate(const affine* __restrict__ pts,
                                                    const uint32_t* __restrict__ sorted_pt,
                                                    const uint32_t* __restrict__ sorted_key,
                                                    const uint32_t* __restrict__ total_ptr, uint32_t L,
                                                    xyzz* __restrict__ buckets, xyzz* __restrict__ head,
                                                    xyzz* __restrict__ tail)
{
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t E = *total_ptr;
    const size_t start = (size_t)t * L;
    if (start >= E) return;
    const uint32_t end = (uint32_t)min((size_t)E, start + L);
    uint32_t cur = sorted_key[start];
    const bool starts_before = start > 0 && sorted_key[start - 1] == cur;
    bool first_run = true;
    xyzz acc;
    xyzz_set_inf(acc);
    for (uint32_t e = (uint32_t)start; e < end; e++) {
        const uint32_t key = sorted_key[e];
        if (key != cur) {
            if (first_run && starts_before) store_xyzz(head + t, acc);
            else store_xyzz(buckets + cur, acc);
            first_run = false;
            xyzz_set_inf(acc);
            cur = key;
        }
        madd_entry(acc, pts, sorted_pt[e]);
    }
    const bool continues_after = end < E && sorted_key[end] == cur;
    if (first_run && starts_before) store_xyzz(head + t, acc);
    else if (continues_after) store_xyzz(tail + t, acc);
    else store_xyzz(buckets + cur, acc);
}

// ----------------------------------------------------------------- 5. fixup
// A bucket whose entries cross chunk edges has partial sums in tail[t0]
// (its first chunk) and head[t0+1 .. t1].  Spans of up to kHotSpan chunks
// are joined by one thread (k_fixup: the first join; k_fixup_rest: the rest
// of 3..kHotSpan-chunk spans).  Longer spans (the narrow top window's
// buckets, repeated scalars) go to a hot list joined by one warp (up to
// kWarpJoinMax partials), one block (up to kGiantMin) or the whole grid
// (k_fixup_giant), so no serial chain grows with the span.
constexpr uint32_t kHotSpan = 4;
constexpr int kHotThreads = 128;

__global__ void __launch_bounds__(128) k_fixup(const uint32_t* __restrict__ sorted_key,
                                               const uint32_t* __restrict__ offsets,
                                               const uint32_t* __restrict__ total_ptr, uint32_t L,
                                               xyzz* __restrict__ buckets, const xyzz* __restrict__ head,
                                               const xyzz* __restrict__ tail, uint2* __restrict__ hot_list,
                                               uint32_t* __restrict__ hot_count, uint32_t cap)
{
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t E = *total_ptr;
    const size_t start = (size_t)t * L;
    if (start >= E) return;
    const uint32_t end = (uint32_t)min((size_t)E, start + L);
    const uint32_t last = sorted_key[end - 1];
    if (!(end < E && sorted_key[end] == last)) return;                 // bucket ends here
    const bool single = sorted_key[start] == last;
    const bool starts_before = start > 0 && sorted_key[start - 1] == sorted_key[start];
    if (single && starts_before) return;                               // a middle chunk
    const uint32_t t1 = (offsets[last + 1] - 1) / L;                   // last chunk of this bucket
    if (t1 - t + 1 > kHotSpan) {
        const uint32_t h = atomicAdd(hot_count, 1u);
        hot_list[h] = make_uint2(last, t);
        return;
    }
    xyzz acc, part;
    load_xyzz(acc, tail + t);
    load_xyzz(part, head + t + 1);
    xyzz_add(acc, part);
    store_xyzz(buckets + last, acc);
    if (t1 > t + 1) {
        // the rest of a 3..kHotSpan-chunk bucket: k_fixup_rest, so the
        // warp's other lanes do not wait through a second addition
        const uint32_t h = atomicAdd(hot_count + 1, 1u);
        hot_list[cap - 1 - h] = make_uint2(last, t);
    }
}

// Finishes the buckets k_fixup left after their first join (list at the top
// of the hot-list buffer, count hot_count[1]): heads t0 + 2 .. t1, one
// thread per bucket, grid-stride.
__global__ void __launch_bounds__(128) k_fixup_rest(const uint2* __restrict__ hot_list,
                                                    const uint32_t* __restrict__ hot_count, uint32_t cap,
                                                    const uint32_t* __restrict__ offsets, uint32_t L,
                                                    xyzz* __restrict__ buckets, const xyzz* __restrict__ head)
{
    const uint32_t nr = hot_count[1];
    for (uint32_t h = blockIdx.x * blockDim.x + threadIdx.x; h < nr; h += gridDim.x * blockDim.x) {
        const uint2 e = hot_list[cap - 1 - h];
        const uint32_t key = e.x, t0 = e.y;
        const uint32_t t1 = (offsets[key + 1] - 1) / L;
        xyzz acc, part;
        load_xyzz(acc, buckets + key);
        for (uint32_t u = t0 + 2; u <= t1; u++) {
            load_xyzz(part, head + u);
            xyzz_add(acc, part);
        }
        store_xyzz(buckets + key, acc);
    }
}

__device__ __forceinline__ void shfl_down_xyzz(xyzz& o, const xyzz& v, int d)
{
    const uint32_t* pv = reinterpret_cast<const uint32_t*>(&v);
    uint32_t* po = reinterpret_cast<uint32_t*>(&o);
#pragma unroll
    for (int k = 0; k < 48; k++) po[k] = __shfl_down_sync(0xffffffffu, pv[k], d);
}

// Sum of `span` partials of one bucket by one warp: the warp's eight quads
// each add every 8th partial with quad point operations, then a tree over the quads as deep as the span needs: a span
// of s <= 8 costs 1 + ceil(log2 s) quad additions (~10k cycles each against
// ~26k for one lane's addition).  Lane 0 ends with the sum.
template <class PartAt>
__device__ __forceinline__ void warp_join(xyzz& acc, uint32_t span, uint32_t lane, PartAt part_at)
{
    const quad_lane ql = quad_of(lane);
    const uint32_t qi = lane >> 2;
    xyzz part;
    xyzz_set_inf(acc);
    for (uint32_t i = qi; i < span; i += 8) {
        load_xyzz(part, part_at(i));
        xyzz_add_quad(acc, part, ql);
    }
    const uint32_t width = min(span, 8u);
    for (uint32_t d = 1; d < width; d <<= 1) {
        xyzz o;
        shfl_down_xyzz(o, acc, (int)(4 * d));
        if ((qi & (2 * d - 1)) == 0 && qi + d < width) xyzz_add_quad(acc, o, ql);
    }
}

// The same for a bucket too large for one warp (a narrow top window, one
// repeated scalar): the whole block, span / blockDim additions per thread,
// then a tree over lanes and over the block's warps.  Thread 0 gets the sum.
constexpr uint32_t kWarpJoinMax = 160;   // larger spans are joined by a block
constexpr uint32_t kGiantMin = 1024;     // larger spans are joined by the grid (k_fixup_giant)
constexpr uint32_t kGiantSlice = 256;

template <class PartAt>
__device__ __forceinline__ void block_join(xyzz& acc, uint32_t span, PartAt part_at, xyzz* sh)
{
    const uint32_t lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    xyzz part;
    xyzz_set_inf(acc);
    for (uint32_t i = threadIdx.x; i < span; i += blockDim.x) {
        load_xyzz(part, part_at(i));
        xyzz_add(acc, part);
    }
    for (uint32_t d = 1; d < 32; d <<= 1) {
        xyzz o;
        shfl_down_xyzz(o, acc, (int)d);
        if ((lane & (2 * d - 1)) == 0) xyzz_add(acc, o);
    }
    __syncthreads();                       // sh is free (previous bucket done)
    if (lane == 0) sh[wid] = acc;
    __syncthreads();
    if (threadIdx.x == 0)
        for (uint32_t w = 1; w < blockDim.x / 32; w++) xyzz_add(acc, sh[w]);
}

__global__ void __launch_bounds__(kHotThreads) k_fixup_hot(uint2* __restrict__ hot_list,
                                                           uint32_t* __restrict__ hot_count,
                                                           const uint32_t* __restrict__ offsets, uint32_t L,
                                                           xyzz* __restrict__ buckets, const xyzz* __restrict__ head,
                                                           const xyzz* __restrict__ tail)
{
    __shared__ xyzz sh[kHotThreads / 32];
    const uint32_t nh = *hot_count;
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t warps = gridDim.x * (blockDim.x / 32);
    for (uint32_t h = (blockIdx.x * blockDim.x + threadIdx.x) / 32; h < nh; h += warps) {
        const uint2 e = hot_list[h];
        const uint32_t key = e.x, t0 = e.y;
        const uint32_t span = (offsets[key + 1] - 1) / L - t0 + 1;
        if (span > kWarpJoinMax) continue;
        xyzz acc;
        warp_join(acc, span, lane, [&](uint32_t i) { return i == 0 ? tail + t0 : head + t0 + i; });
        if (lane == 0) store_xyzz(buckets + key, acc);
    }
    for (uint32_t h = blockIdx.x; h < nh; h += gridDim.x) {
        const uint2 e = hot_list[h];
        const uint32_t key = e.x, t0 = e.y;
        const uint32_t span = (offsets[key + 1] - 1) / L - t0 + 1;
        if (span <= kWarpJoinMax) continue;
        if (span > kGiantMin) {                                        // joined by the grid: the giant list
            if (threadIdx.x == 0) hot_list[nh + atomicAdd(hot_count + 2, 1u)] = e;
            continue;
        }
        xyzz acc;
        block_join(acc, span, [&](uint32_t i) { return i == 0 ? tail + t0 : head + t0 + i; }, sh);
        if (threadIdx.x == 0) store_xyzz(buckets + key, acc);
    }
}

// Segmented fixup (the MSM and batch pipelines; the fixed-scratch entry keeps
// the serial k_fixup above).  A bucket spanning chunks t0..t1 is the sum of
// tail[t0] and head[t0+1..t1].  k_fixup_seg reduces the head partials of
// each warp's chunks per bucket with a tree over lanes (depth 5, one
// addition per partial) and writes each warp-local piece's sum to the
// piece's first head slot; k_fixup_join then adds tail[t0] and one piece per
// warp the bucket spans.  A 16-chunk bucket costs 4 + 1 dependent additions
// instead of 15.
constexpr uint32_t kNoKey = 0xffffffffu;
constexpr uint32_t kHotSpanSeg = 128;

__global__ void __launch_bounds__(128) k_fixup_seg(const uint32_t* __restrict__ sorted_key,
                                                   const uint32_t* __restrict__ total_ptr, uint32_t L,
                                                   xyzz* __restrict__ head)
{
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t E = *total_ptr;
    const size_t start = (size_t)t * L;
    uint32_t hk = kNoKey;                     // bucket of head[t], if chunk t starts inside one
    if (start < E && start > 0) {
        const uint32_t kf = sorted_key[start];
        if (sorted_key[start - 1] == kf) hk = kf;
    }
    xyzz v;
    if (hk != kNoKey) load_xyzz(v, head + t);
    else xyzz_set_inf(v);
    const uint32_t prev = __shfl_up_sync(0xffffffffu, hk, 1);
    const uint32_t starts = __ballot_sync(0xffffffffu, lane == 0 || prev != hk);
    const uint32_t first = 31 - __clz(starts & (0xffffffffu >> (31 - lane)));
    const uint32_t off = lane - first;        // position within the lane segment
    for (int d = 1; d < 32; d <<= 1) {
        xyzz o;
        shfl_down_xyzz(o, v, d);
        const uint32_t ok = __shfl_down_sync(0xffffffffu, hk, d);
        if (hk != kNoKey && (off & (2 * d - 1)) == 0 && lane + d < 32 && ok == hk) xyzz_add(v, o);
    }
    if (hk != kNoKey && off == 0) store_xyzz(head + t, v);
}

__global__ void __launch_bounds__(128) k_fixup_join(const uint32_t* __restrict__ sorted_key,
                                                    const uint32_t* __restrict__ offsets,
                                                    const uint32_t* __restrict__ total_ptr, uint32_t L,
                                                    xyzz* __restrict__ buckets, const xyzz* __restrict__ head,
                                                    const xyzz* __restrict__ tail, uint2* __restrict__ hot_list,
                                                    uint32_t* __restrict__ hot_count)
{
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t E = *total_ptr;
    const size_t start = (size_t)t * L;
    if (start >= E) return;
    const uint32_t end = (uint32_t)min((size_t)E, start + L);
    const uint32_t last = sorted_key[end - 1];
    if (!(end < E && sorted_key[end] == last)) return;                 // bucket ends here
    const bool single = sorted_key[start] == last;
    const bool starts_before = start > 0 && sorted_key[start - 1] == sorted_key[start];
    if (single && starts_before) return;                               // a middle chunk
    const uint32_t t1 = (offsets[last + 1] - 1) / L;                   // last chunk of this bucket
    if (t1 - t + 1 > kHotSpanSeg) {
        const uint32_t h = atomicAdd(hot_count, 1u);
        hot_list[h] = make_uint2(last, t);
        return;
    }
    xyzz acc, part;
    load_xyzz(acc, tail + t);
    for (uint32_t u = t + 1; u <= t1; u = (u | 31u) + 1) {           // one piece per warp
        load_xyzz(part, head + u);
        xyzz_add(acc, part);
    }
    store_xyzz(buckets + last, acc);
}

// k_fixup_hot over the pieces k_fixup_seg left: tail[t0], head[t0 + 1] and
// the head slot at each later warp boundary up to t1.
__global__ void __launch_bounds__(kHotThreads) k_fixup_hot_seg(uint2* __restrict__ hot_list,
                                                               uint32_t* __restrict__ hot_count,
                                                               const uint32_t* __restrict__ offsets, uint32_t L,
                                                               xyzz* __restrict__ buckets,
                                                               const xyzz* __restrict__ head,
                                                               const xyzz* __restrict__ tail)
{
    __shared__ xyzz sh[kHotThreads / 32];
    const uint32_t nh = *hot_count;
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t warps = gridDim.x * (blockDim.x / 32);
    auto piece = [&](uint32_t t0, uint32_t i) {
        return i == 0 ? tail + t0 : head + (i == 1 ? t0 + 1 : (((t0 + 1) | 31u) + 1 + 32 * (i - 2)));
    };
    for (uint32_t h = (blockIdx.x * blockDim.x + threadIdx.x) / 32; h < nh; h += warps) {
        const uint2 e = hot_list[h];
        const uint32_t key = e.x, t0 = e.y;
        const uint32_t t1 = (offsets[key + 1] - 1) / L;
        const uint32_t np = 2 + (t1 >> 5) - ((t0 + 1) >> 5);          // tail + pieces
        if (np > kWarpJoinMax) continue;
        xyzz acc;
        warp_join(acc, np, lane, [&](uint32_t i) { return piece(t0, i); });
        if (lane == 0) store_xyzz(buckets + key, acc);
    }
    for (uint32_t h = blockIdx.x; h < nh; h += gridDim.x) {
        const uint2 e = hot_list[h];
        const uint32_t key = e.x, t0 = e.y;
        const uint32_t t1 = (offsets[key + 1] - 1) / L;
        const uint32_t np = 2 + (t1 >> 5) - ((t0 + 1) >> 5);
        if (np <= kWarpJoinMax) continue;
        if (np > kGiantMin) {                                          // joined by the grid: the giant list
            if (threadIdx.x == 0) hot_list[nh + atomicAdd(hot_count + 2, 1u)] = e;
            continue;
        }
        xyzz acc;
        block_join(acc, np, [&](uint32_t i) { return piece(t0, i); }, sh);
        if (threadIdx.x == 0) store_xyzz(buckets + key, acc);
    }
}

// Buckets of more than kGiantMin partials (all-equal scalars, a forced narrow
// top window; k_fixup_hot / k_fixup_hot_seg list them after the hot list,
// count hot_count[2]) are joined by the whole grid instead of one block: every block
// reduces kGiantSlice-partial slices and writes each slice's sum over the
// slice's first partial (k_fixup_giant), then one block per bucket joins the
// slice sums (k_fixup_giant_join).  The slices of all giants are dealt to
// the blocks round-robin.  A bucket of 2^20 entries (~14k chunks) costs
// ~2 + 7 + 7 dependent additions instead of span / 128 + 7.  Seg: the pieces k_fixup_seg
// left, as in k_fixup_hot_seg; otherwise tail[t0] and head[t0 + 1 .. t1].
template <bool Seg>
__device__ __forceinline__ xyzz* hot_part(xyzz* head, xyzz* tail, uint32_t t0, uint32_t i)
{
    if (i == 0) return tail + t0;
    if (!Seg || i == 1) return head + t0 + i;
    return head + (((t0 + 1) | 31u) + 1 + 32 * (i - 2));
}

template <bool Seg>
__device__ __forceinline__ uint32_t hot_parts(uint32_t key, uint32_t t0, const uint32_t* offsets, uint32_t L)
{
    const uint32_t t1 = (offsets[key + 1] - 1) / L;
    return Seg ? 2 + (t1 >> 5) - ((t0 + 1) >> 5) : t1 - t0 + 1;
}

template <bool Seg>
__global__ void __launch_bounds__(kHotThreads) k_fixup_giant(const uint2* __restrict__ hot_list,
                                                             const uint32_t* __restrict__ hot_count,
                                                             const uint32_t* __restrict__ offsets, uint32_t L,
                                                             xyzz* __restrict__ head, xyzz* __restrict__ tail)
{
    __shared__ xyzz sh[kHotThreads / 32];
    const uint2* giants = hot_list + hot_count[0];
    const uint32_t ng = hot_count[2];
    uint32_t base = 0;                      // slices of the giants before this one
    for (uint32_t h = 0; h < ng; h++) {
        const uint2 e = giants[h];
        const uint32_t np = hot_parts<Seg>(e.x, e.y, offsets, L);
        if (np <= kGiantMin) continue;
        const uint32_t ns = (np + kGiantSlice - 1) / kGiantSlice;
        // global slice base + sl goes to block (base + sl) mod gridDim.x, so
        // the slices of every giant run at once
        const uint32_t first = (blockIdx.x + gridDim.x - base % gridDim.x) % gridDim.x;
        base += ns;
        for (uint32_t sl = first; sl < ns; sl += gridDim.x) {
            const uint32_t b0 = sl * kGiantSlice;
            xyzz acc;
            block_join(acc, min(kGiantSlice, np - b0), [&](uint32_t i) { return hot_part<Seg>(head, tail, e.y, b0 + i); },
                       sh);
            if (threadIdx.x == 0) store_xyzz(hot_part<Seg>(head, tail, e.y, b0), acc);
        }
    }
}

template <bool Seg>
__global__ void __launch_bounds__(kHotThreads) k_fixup_giant_join(const uint2* __restrict__ hot_list,
                                                                  const uint32_t* __restrict__ hot_count,
                                                                  const uint32_t* __restrict__ offsets, uint32_t L,
                                                                  xyzz* __restrict__ buckets, xyzz* __restrict__ head,
                                                                  xyzz* __restrict__ tail)
{
    __shared__ xyzz sh[kHotThreads / 32];
    const uint2* giants = hot_list + hot_count[0];
    const uint32_t ng = hot_count[2];
    for (uint32_t h = blockIdx.x; h < ng; h += gridDim.x) {
        const uint2 e = giants[h];
        const uint32_t np = hot_parts<Seg>(e.x, e.y, offsets, L);
        if (np <= kGiantMin) continue;
        const uint32_t ns = (np + kGiantSlice - 1) / kGiantSlice;
        xyzz acc;
        block_join(acc, ns, [&](uint32_t sl) { return hot_part<Seg>(head, tail, e.y, sl * kGiantSlice); }, sh);
        if (threadIdx.x == 0) store_xyzz(buckets + e.x, acc);
    }
}

void fixup_giants(const void* hot_list, const uint32_t* hot_count, const uint32_t* offsets, uint32_t L,
                  void* buckets, void* head, void* tail, bool seg, cudaStream_t st)
{
    const uint2* hl = (const uint2*)hot_list;
    if (seg) {
        k_fixup_giant<true><<<2 * device_sms(), kHotThreads, 0, st>>>(hl, hot_count, offsets, L, (xyzz*)head, (xyzz*)tail);
        k_fixup_giant_join<true><<<2 * device_sms(), kHotThreads, 0, st>>>(hl, hot_count, offsets, L, (xyzz*)buckets,
                                                                   (xyzz*)head, (xyzz*)tail);
    } else {
        k_fixup_giant<false><<<2 * device_sms(), kHotThreads, 0, st>>>(hl, hot_count, offsets, L, (xyzz*)head, (xyzz*)tail);
        k_fixup_giant_join<false><<<2 * device_sms(), kHotThreads, 0, st>>>(hl, hot_count, offsets, L, (xyzz*)buckets,
                                                                    (xyzz*)head, (xyzz*)tail);
    }
}

// ----------------------------------------------------------------- 6/7. reduce
// Window sum W = sum_{b<B} (b+1) S_b.  Write F0(x) = sum_i i x_i.  Grouping the
// inputs of a level in runs of F (node u owns children uF .. uF+F-1):
//   F0(x) = sum_u T_u + F0(F r),  r_u = sum_j x_{uF+j},  T_u = sum_j j x_{uF+j}
// so every node emits Q_u = T_u + (its children's Q) and A_u = F r_u, and the
// root's Q is the window sum.  Level 1 uses weights j+1 (giving W directly)
// with fan-in 8: a 2-addition-per-bucket running sum that keeps every SM
// busy.  Upper levels use fan-in 2 (one addition, one doubling, two Q
// additions), keeping the dependent chain per level short: with few threads
// the cost of a level is its serial latency, not its work.
__global__ void __launch_bounds__(128) k_reduce_level(const xyzz* __restrict__ inA, const xyzz* __restrict__ inQ,
                                                      uint32_t m_in, uint32_t F, uint32_t lgF, uint32_t D,
                                                      int first, xyzz* __restrict__ outA, xyzz* __restrict__ outQ)
{
    const uint32_t m_out = (m_in + F - 1) / F;
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= D * m_out) return;
    const uint32_t w = t / m_out, u = t % m_out;
    const uint32_t c0 = u * F;
    const uint32_t cnt = min(F, m_in - c0);
    const xyzz* a = inA + (size_t)w * m_in + c0;
    xyzz r, tt, b;
    xyzz_set_inf(r);
    xyzz_set_inf(tt);
    for (int j = (int)cnt - 1; j >= 1; j--) {
        load_xyzz(b, a + j);
        xyzz_add(r, b);
        xyzz_add(tt, r);
    }
    load_xyzz(b, a);
    xyzz_add(r, b);
    if (first) xyzz_add(tt, r);
    if (inQ) {
        const xyzz* q = inQ + (size_t)w * m_in + c0;
        for (uint32_t j = 0; j < cnt; j++) {
            load_xyzz(b, q + j);
            xyzz_add(tt, b);
        }
    }
    if (m_out > 1) {
        for (uint32_t k = 0; k < lgF; k++) xyzz_dbl(r);
        store_xyzz(outA + (size_t)w * m_out + u, r);
    }
    store_xyzz(outQ + (size_t)w * m_out + u, tt);
}

// Binary levels with two threads per node: the Q thread computes
// Q = A_1 + Q_0 + Q_1 and the A thread A = 2 (A_0 + A_1), concurrently (one
// thread doing both ran 3 additions and a doubling back to back; the level's
// dependent chain is now 2 additions).  A node with one child keeps Q_0 and
// doubles A_0.  This is k_reduce_level's rule with fan-in 2.  Quad = true:
// each of the two is a quad of lanes (quad point operations), for levels
// too small to fill the GPU.
template <bool Quad>
__device__ __forceinline__ void add_op(xyzz& p, const xyzz& o, const quad_lane& q)
{
    if (Quad) xyzz_add_quad(p, o, q);
    else xyzz_add(p, o);
}

template <bool Quad>
__device__ __forceinline__ void pair_node(xyzz& out, const xyzz* a, const xyzz* q, uint32_t cnt, bool q_role,
                                          const quad_lane& ql)
{
    xyzz b;
    if (q_role) {
        load_xyzz(out, q);
        if (cnt == 2) {
            load_xyzz(b, a + 1);
            add_op<Quad>(out, b, ql);
            load_xyzz(b, q + 1);
            add_op<Quad>(out, b, ql);
        }
    } else {
        load_xyzz(out, a);
        if (cnt == 2) {
            load_xyzz(b, a + 1);
            add_op<Quad>(out, b, ql);
        }
        if (Quad) xyzz_dbl_quad(out, ql);
        else xyzz_dbl(out);
    }
}

// Thread g's node and role.  The role is uniform per warp (even warps Q, odd
// warps A): lanes of one warp taking different roles would run both paths one
// after the other.  A warp covers 32 nodes, or 8 with quads.
template <bool Quad>
__device__ __forceinline__ void pair_slot(uint32_t g, uint32_t& node, bool& q_role)
{
    node = Quad ? (g >> 6) * 8 + ((g >> 2) & 7) : (g >> 6) * 32 + (g & 31);
    q_role = ((g >> 5) & 1) == 0;
}

// One binary level over D windows of m_in (A, Q) pairs.
template <bool Quad>
__global__ void __launch_bounds__(128) k_reduce_pair(const xyzz* __restrict__ inA, const xyzz* __restrict__ inQ,
                                                     uint32_t m_in, uint32_t D, xyzz* __restrict__ outA,
                                                     xyzz* __restrict__ outQ)
{
    const uint32_t m_out = (m_in + 1) / 2;
    uint32_t t;
    bool q_role;
    pair_slot<Quad>(blockIdx.x * blockDim.x + threadIdx.x, t, q_role);
    if (t >= D * m_out || (!q_role && m_out == 1)) return;
    const quad_lane ql = quad_of(threadIdx.x & 31);
    const uint32_t w = t / m_out, u = t % m_out;
    const size_t base = (size_t)w * m_in + 2 * u;
    xyzz r;
    pair_node<Quad>(r, inA + base, inQ + base, min(2u, m_in - 2 * u), q_role, ql);
    if (!Quad || ql.k == 0) store_xyzz((q_role ? outQ : outA) + (size_t)w * m_out + u, r);
}

// The last binary levels in one launch: block w reduces window w's m_in
// (A, Q) pairs (m_in <= kTailThreads / 4) to its root Q in shared memory with
// one barrier per level, instead of one launch and a global round trip per
// level.  Quads placed as in k_reduce_pair<true>; the block is sized to the
// first level so that many windows fit on an SM.
constexpr int kTailThreads = 256;
constexpr size_t kFanIn8MinBuckets = size_t(1) << 18;   // all windows' buckets
constexpr size_t kFanIn16MinBuckets = size_t(1) << 20;
constexpr uint32_t kQuadMaxNodes = 8192;                  // a level of at most this many nodes uses quads

__global__ void __launch_bounds__(kTailThreads) k_reduce_tail(const xyzz* __restrict__ inA,
                                                              const xyzz* __restrict__ inQ, uint32_t m_in,
                                                              xyzz* __restrict__ outQ)
{
    extern __shared__ __align__(16) unsigned char tail_smem[];
    const uint32_t nodes = blockDim.x / 8;
    xyzz* shA = reinterpret_cast<xyzz*>(tail_smem);
    xyzz* shQ = shA + nodes;
    const uint32_t w = blockIdx.x;
    const quad_lane ql = quad_of(threadIdx.x & 31);
    uint32_t t;
    bool q_role;
    pair_slot<true>(threadIdx.x, t, q_role);
    uint32_t m = m_in;
    const xyzz* srcA = inA + (size_t)w * m_in;
    const xyzz* srcQ = inQ + (size_t)w * m_in;
    while (m > 1) {
        const uint32_t m_out = (m + 1) / 2;
        xyzz r;
        const bool act = t < m_out && (q_role || m_out > 1);
        if (act) pair_node<true>(r, srcA + 2 * t, srcQ + 2 * t, min(2u, m - 2 * t), q_role, ql);
        __syncthreads();
        if (act && ql.k == 0) (q_role ? shQ : shA)[t] = r;
        __syncthreads();
        srcA = shA;
        srcQ = shQ;
        m = m_out;
    }
    if (threadIdx.x == 0) store_xyzz(outQ + w, m_in == 1 ? srcQ[0] : shQ[0]);
}

// ----------------------------------------------------------------- host driver
static uint32_t ilog2(size_t n)
{
    uint32_t k = 0;
    while (n >>= 1) k++;
    return k;
}

uint32_t msm_default_window(size_t n)
{
    const uint32_t lg = ilog2(n);
    int c = (int)lg - 4;
    if (c < 4) c = 4;
    if (c > 20) c = 20;
    return (uint32_t)c;
}

// Window for the GLV halves (n2 points of 127-bit scalars): among widths whose
// top window keeps at least half of c bits (a narrow top window concentrates
// its entries in a few hot buckets), the c in [2, 20] minimising bucket
// entries + 4 x buckets (reducing a bucket costs about four accumulated
// entries on this GPU).  Measured best: 16 for n2 = 2^21, 19 for n2 = 2^23.
uint32_t msm_glv_window(size_t n2)
{
    double best = 0;
    uint32_t bc = 0;
    for (uint32_t c = 2; c <= 20; c++) {
        const uint32_t D = 127 / c + 1;
        const uint32_t top = 127 - (D - 1) * c;
        if (2 * top < c) continue;
        const double entries = (double)n2 * ((D - 1) + (1.0 - std::ldexp(1.0, -(int)top)));
        const double cost = entries + 4.0 * D * std::ldexp(1.0, (int)c - 1);
        if (bc == 0 || cost < best) { best = cost; bc = c; }
    }
    // Up to 2^15 points the MSM is latency-bound: a bucket-reduction level is
    // a chain of dependent additions, so fewer, fuller buckets win over the
    // work model (measured: 2^13 points c = 8 0.467 ms against c = 10 0.493;
    // 2^15 points c = 10 0.634 against c = 11 0.677; 2^11 points c = 8 best).
    uint32_t lg = 0;
    while ((size_t(2) << lg) <= n2) lg++;
    if (n2 <= (size_t(1) << 15)) bc = std::min(bc, std::max(8u, lg - 5));
    return bc;
}

cudaError_t msm_setup_device()
{
    return cudaFuncSetAttribute(k_reduce_tail, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)(kTailThreads / 8 * 2 * sizeof(xyzz)));
}

// The tail takes a window set once m <= msm_reduce_tail_max(D), with quads
// (its levels are latency-bound).  Above kTailMaxSets sets (a batch of MSMs)
// it is not used: one block per set leaves the later levels of every block
// nearly empty, and the global pair levels (many sets per launch) finish
// sooner (1024 sets of 128 pairs: tail 0.81 ms; pair levels about a third of
// that).
constexpr uint32_t kTailMaxSets = 64;

uint32_t msm_reduce_tail_max(uint32_t D) { return D > kTailMaxSets ? 1 : kTailThreads / 4; }

void msm_reduce_tail(const void* inA, const void* inQ, uint32_t m, uint32_t D, void* outQ, cudaStream_t st)
{
    const uint32_t T = ((m + 1) / 2 + 7) / 8 * 64;   // a Q warp and an A warp per 8 first-level nodes
    k_reduce_tail<<<D, T, T / 8 * 2 * sizeof(xyzz), st>>>((const xyzz*)inA, (const xyzz*)inQ, m, (xyzz*)outQ);
}

void msm_reduce_pair(const void* inA, const void* inQ, uint32_t m, uint32_t D, void* outA, void* outQ,
                     cudaStream_t st)
{
    const size_t nodes = (size_t)D * ((m + 1) / 2);
    if (nodes <= kQuadMaxNodes) {
        const size_t threads = (nodes + 7) / 8 * 64;
        k_reduce_pair<true><<<div_up(threads, 128), 128, 0, st>>>((const xyzz*)inA, (const xyzz*)inQ, m, D,
                                                                  (xyzz*)outA, (xyzz*)outQ);
    } else {
        const size_t threads = (nodes + 31) / 32 * 64;
        k_reduce_pair<false><<<div_up(threads, 128), 128, 0, st>>>((const xyzz*)inA, (const xyzz*)inQ, m, D,
                                                                   (xyzz*)outA, (xyzz*)outQ);
    }
}

// Entries per k_accumulate thread.  Small inputs: the L in [4, 48] of least
// modelled accumulate + fixup time (below).  Once a chunk of 48 fills every
// resident block slot: the L in [48, 96] that minimises ceil(W / L) L, W =
// entries per resident thread slot, i.e. the launch ends on (just under) a
// whole number of waves instead of a short last wave (measured at 2^20, GLV:
// L = 64 -> 3.4 waves, 7.35 ms; L = 72 -> 3.0 waves, 7.14 ms); ties go to the
// larger L (fewer chunk carries to join).
static uint32_t accumulate_chunk(size_t nD)
{
    // Shared by every calling thread: sms is stored before slots (release)
    // and read after it (acquire), so a thread that sees slots sees sms.
    static std::atomic<int> slots_by_dev[64], sms_by_dev[64];
    int dev = 0;
    cudaGetDevice(&dev);
    const bool cached = dev >= 0 && dev < 64;
    int slots = cached ? slots_by_dev[dev].load(std::memory_order_acquire) : 0;
    int sms = cached ? sms_by_dev[dev].load(std::memory_order_relaxed) : 0;
    if (slots == 0) {
        int per_sm = 0;
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_accumulate, 128, 0);
        if (sms <= 0 || per_sm <= 0) {
            sms = device_sms();
            per_sm = 4;
        }
        slots = sms * per_sm * 128;
        if (cached) {
            sms_by_dev[dev].store(sms, std::memory_order_relaxed);
            slots_by_dev[dev].store(slots, std::memory_order_release);
        }
    }
    const double W = (double)nD / slots;
    if (W < 48) {
        // Less than about one full wave.  The accumulate time is the busiest
        // SM's work, its blocks x L entries (below ~1.5 blocks per SM the
        // chain of L dependent additions sets it instead), and the fixup
        // costs about one addition per chunk:
        //   cost(L) = max(blocks per SM, 1.5) L + 4.7e-4 nD / L
        // in units of one entry of a resident block (fitted on GB300 to
        // 2^10..2^17-point MSMs).
        uint32_t best = 4;
        double best_cost = 0;
        for (uint32_t L = 4; L <= 48; L++) {
            const double bpsm = std::ceil(std::ceil((double)nD / L / 128) / sms);
            const double cost = std::max(bpsm, 1.5) * L + 4.7e-4 * (double)nD / L;
            if (L == 4 || cost < best_cost) {
                best_cost = cost;
                best = L;
            }
        }
        return best;
    }
    uint32_t best = 64;
    double best_cost = 0;
    for (uint32_t L = 48; L <= 96; L++) {
        const double cost = std::ceil(W / L) * L;
        if (L == 48 || cost <= best_cost) { best_cost = cost; best = L; }
    }
    return best;
}

// Batch-affine rounds for nD bucket entries over M buckets.  A round pairs
// entries of one bucket inside one chunk, so it pays only when buckets hold
// many entries; each round costs three launches per half and one inversion
// per block.  Measured on GB300 (accumulate stage, ms, rounds 0 / 2 / 3 / 4):
// 2^20 points 5.38 / 5.03 / 4.89 / 4.93; 2^22 18.45 / 17.48 / 17.10 / 17.15;
// 2^18 1.43 / 1.51 / 1.61 / 1.72 (fewer entries per bucket: no gain).
uint32_t msm_affine_rounds(size_t nD, size_t M)
{
    const double per = (double)nD / (double)(M ? M : 1);
    if (nD < (size_t(1) << 24) || per < 16) return 0;
    return 3;
}

static bool use_glv(const Ctx* ctx, size_t n, uint32_t nbits)
{
    return ctx->glv && nbits > 128 && n < (1u << 30);
}

static uint32_t level1_fan_in(size_t M)
{
    return M >= kFanIn16MinBuckets ? 16 : M >= kFanIn8MinBuckets ? 8 : 2;
}

// The plan without a context (host arithmetic only; off a GPU the chunk
// model uses 152 SMs x 4 resident blocks, the GB300's figures): window,
// windows, pipeline points, accumulate chunk length and level-1 fan-in.
void msm_plan_detail(size_t n, uint32_t nbits, bool glv, uint32_t* c, uint32_t* windows, size_t* points,
                     uint32_t* chunk, uint32_t* fan_in)
{
    const bool g = glv && nbits > 128 && n < (1u << 30);
    const size_t np = g ? 2 * n : n;
    *c = g ? msm_glv_window(np) : msm_default_window(np);
    *windows = (g ? 127 : nbits) / *c + 1;
    *points = np;
    *chunk = accumulate_chunk(np * *windows);
    *fan_in = level1_fan_in((size_t)*windows << (*c - 1));
}

void msm_plan(const Ctx* ctx, size_t n, uint32_t nbits, uint32_t* c, uint32_t* windows, size_t* points)
{
    const bool g = use_glv(ctx, n, nbits);
    const size_t np = g ? 2 * n : n;
    const uint32_t nb = g ? 127 : nbits;
    *c = g ? msm_glv_window(np) : msm_default_window(np);
    *windows = nb / *c + 1;
    *points = np;
}

// Runs the device pipeline over device-resident points/scalars on the context
// stream and returns the folded, normalised result in `out` (144 bytes).
// tile_window != 0: one window of the reference's tile (bit0, window) instead
// of the whole MSM (no GLV split, D = 1, c = the window's encode size).
static cudaError_t msm_run(Ctx* ctx, const void* d_points, const uint8_t* d_scalars, uint32_t stride, size_t n,
                           uint32_t nbits, uint32_t c, uint64_t* out, cudaEvent_t points_ready, uint32_t tile_bit0,
                           uint32_t tile_window)
{
    cudaStream_t st = ctx->stream;
    MsmWork& W = ctx->msm;
    if (n == 0 || n > 0x7fffffffu) return cudaErrorInvalidValue;
    StageProfile& P = ctx->prof;
    if (P.enabled && !P.ev[0]) {
        for (int i = 0; i <= kMsmStages; i++) CATMSM_CHECK(cudaEventCreate(&P.ev[i]));
    }
    auto mark = [&](int i) {
        if (P.enabled) cudaEventRecord(P.ev[i], st);
    };
    mark(0);
    // The points are read only from the point stage on (after the scatter):
    // points_ready, if given, is an event on another stream (a host copy in
    // flight) that the pipeline waits for just before that stage.
    const affine* src_points = (const affine*)d_points;
    affine* gpts = nullptr;
    uint8_t* sgn = nullptr;
    const size_t n_in = n;
    if (!tile_window && use_glv(ctx, n, nbits)) {
        gpts = (affine*)W.glv_pts.get(2 * n * sizeof(affine));
        uint4* gsc = (uint4*)W.glv_sc.get(2 * n * sizeof(uint4));
        sgn = (uint8_t*)W.glv_sign.get(n);
        if (!gpts || !gsc || !sgn) return cudaErrorMemoryAllocation;
        k_glv_scalars<<<div_up(n, 128), 128, 0, st>>>(d_scalars, stride, (uint32_t)n, nbits, gsc, sgn);
        g_stats.launches++;
        d_points = gpts;
        d_scalars = reinterpret_cast<const uint8_t*>(gsc);
        stride = 16;
        n *= 2;
        nbits = 127;
        if (c == 0) c = msm_glv_window(n);
    }
    uint32_t D;
    if (tile_window) {
        c = min(nbits - tile_bit0 + 1, tile_window);    // encode size
        D = 1;
        if (c < 1 || c > 24) return cudaErrorInvalidValue;
    } else {
        if (c == 0) c = msm_default_window(n);
        if (c < 2 || c > 22) return cudaErrorInvalidValue;
        D = nbits / c + 1;
    }
    const uint32_t B = 1u << (c - 1);
    const size_t M = (size_t)D * B;
    const size_t nD = (size_t)n * D;
    if (nD > 0xffffffffu - 1) return cudaErrorInvalidValue;
    const uint32_t L = accumulate_chunk(nD);
    const size_t chunks = (nD + L - 1) / L;
    // Level 1 of the reduction: fan-in 8 (about 2.4 additions per bucket, but
    // a 19-operation dependent chain) when there are enough buckets to keep
    // every SM busy, fan-in 16 (about 2.1 per bucket and half the nodes for
    // the levels above; a 34-operation chain) when there are many more;
    // otherwise fan-in 2 with the pair kernel straight from the buckets
    // (Q = B_0 + 2 B_1, A = 2 (B_0 + B_1): two operations per level).
    const uint32_t S = level1_fan_in(M);
    const size_t lvl1 = (size_t)D * ((B + S - 1) / S);
    const size_t lvl2 = (size_t)D * ((B + 2 * S - 1) / (2 * S)) + D;

    uint32_t* digits = (uint32_t*)W.digits.get(nD * 4);
    uint32_t* ranks = (uint32_t*)W.ranks.get(nD * 4);
    uint32_t* counts = (uint32_t*)W.counts.get(M * 4);
    uint32_t* offsets = (uint32_t*)W.offsets.get((M + 1) * 4);
    const uint32_t nblocks = div_up(M, kScanTile);
    uint32_t* bsums = (uint32_t*)W.block_sums.get((size_t)nblocks * 4);
    uint32_t* sorted_pt = (uint32_t*)W.sorted_pt.get(nD * 4);
    uint32_t* sorted_key = (uint32_t*)W.sorted_key.get(nD * 4);
    xyzz* buckets = (xyzz*)W.buckets.get(M * sizeof(xyzz));
    xyzz* head = (xyzz*)W.head.get(chunks * sizeof(xyzz));
    xyzz* tail = (xyzz*)W.tail.get(chunks * sizeof(xyzz));
    xyzz* seg = (xyzz*)W.seg.get(2 * (lvl1 + lvl2) * sizeof(xyzz));
    xyzz* wins = (xyzz*)W.wins.get((size_t)D * sizeof(xyzz));
    uint64_t* h_wins = (uint64_t*)ctx->h_out.get((size_t)D * sizeof(xyzz));
    uint32_t* hot_count = (uint32_t*)W.status.get(256 + chunks * sizeof(uint2));
    uint2* hot_list = reinterpret_cast<uint2*>(hot_count + 64);
    if (!digits || !ranks || !counts || !offsets || !bsums || !sorted_pt || !sorted_key || !buckets ||
        !head || !tail || !seg || !wins || !h_wins || !hot_count)
        return cudaErrorMemoryAllocation;
    uint32_t* total = offsets + M;

    CATMSM_CHECK(cudaMemsetAsync(counts, 0, M * 4, st));
    CATMSM_CHECK(cudaMemsetAsync(buckets, 0, M * sizeof(xyzz), st));
    CATMSM_CHECK(cudaMemsetAsync(hot_count, 0, 12, st));  // hot, rest and giant list counts
    mark(1);
    if (tile_window)
        k_tile_digits<<<div_up(n, 256), 256, 0, st>>>(d_scalars, stride, (uint32_t)n, nbits, tile_bit0, tile_window, c,
                                                      digits, ranks, counts);
    else
        k_digits<<<div_up(n, 256), 256, 0, st>>>(d_scalars, stride, (uint32_t)n, nbits, c, D, digits, ranks,
                                                counts);
    mark(2);
    k_scan_local<<<nblocks, kScanThreads, 0, st>>>(counts, offsets, bsums, (uint32_t)M);
    k_scan_top<<<1, kScanThreads, 0, st>>>(bsums, nblocks, total);
    k_scan_add<<<div_up(M, 256), 256, 0, st>>>(offsets, bsums, (uint32_t)M);
    mark(3);
    k_scatter<<<div_up(nD, 256), 256, 0, st>>>(digits, ranks, offsets, (uint32_t)n, (uint32_t)nD, sorted_pt,
                                              sorted_key);
    if (points_ready) CATMSM_CHECK(cudaStreamWaitEvent(st, points_ready, 0));
    if (gpts) {
        k_glv_points<<<div_up(n_in, 128), 128, 0, st>>>(src_points, sgn, (uint32_t)n_in, gpts);
        g_stats.launches++;
    }
    mark(4);
    const uint32_t rounds = tile_window ? 0
                          : ctx->affine_rounds >= 0 ? (uint32_t)ctx->affine_rounds : msm_affine_rounds(nD, M);
    if (rounds)
        CATMSM_CHECK(msm_accumulate_affine(ctx, d_points, sorted_pt, sorted_key, total, L, chunks, rounds, buckets,
                                           head, tail, st));
    else
        k_accumulate<<<div_up(chunks, 128), 128, 0, st>>>((const affine*)d_points, sorted_pt, sorted_key, total, L,
                                                          buckets, head, tail);
    mark(5);
    if (nD > 2 * (size_t)L * M) {
        // buckets average more than two chunks: tree over each warp's chunks
        k_fixup_seg<<<div_up(chunks, 128), 128, 0, st>>>(sorted_key, total, L, head);
        k_fixup_join<<<div_up(chunks, 128), 128, 0, st>>>(sorted_key, offsets, total, L, buckets, head, tail,
                                                          hot_list, hot_count);
        k_fixup_hot_seg<<<2 * device_sms(), kHotThreads, 0, st>>>(hot_list, hot_count, offsets, L, buckets, head, tail);
        fixup_giants(hot_list, hot_count, offsets, L, buckets, head, tail, true, st);
        g_stats.launches += 3;
    } else {
        // short spans: one thread joins each bucket's few carries
        k_fixup<<<div_up(chunks, 128), 128, 0, st>>>(sorted_key, offsets, total, L, buckets, head, tail, hot_list,
                                                     hot_count, (uint32_t)chunks);
        k_fixup_hot<<<2 * device_sms(), kHotThreads, 0, st>>>(hot_list, hot_count, offsets, L, buckets, head, tail);
        k_fixup_rest<<<2 * device_sms(), 128, 0, st>>>(hot_list, hot_count, (uint32_t)chunks, offsets, L, buckets, head);
        fixup_giants(hot_list, hot_count, offsets, L, buckets, head, tail, false, st);
        g_stats.launches += 3;
    }
    mark(6);
    {
        // level 1: fan-in S over the buckets; then fan-in 2 to the root.  With
        // fan-in 2 throughout, level 1 is the pair rule with Q = A = buckets.
        xyzz* bufA[2] = {seg, seg + 2 * lvl1};
        xyzz* bufQ[2] = {seg + lvl1, seg + 2 * lvl1 + lvl2};
        const xyzz* inA = buckets;
        const xyzz* inQ = S == 2 ? buckets : nullptr;
        uint32_t m = B, pp = 0;
        bool first = S != 2;
        while (m > 1) {
            if (!first && m <= msm_reduce_tail_max(D)) {
                msm_reduce_tail(inA, inQ, m, D, bufQ[pp], st);
                g_stats.launches++;
                inQ = bufQ[pp];
                m = 1;
                break;
            }
            const uint32_t F = first ? S : 2;
            const uint32_t m_out = (m + F - 1) / F;
            if (first)
                k_reduce_level<<<div_up((size_t)D * m_out, 128), 128, 0, st>>>(inA, inQ, m, F, S == 16 ? 4 : 3, D, 1,
                                                                              bufA[pp], bufQ[pp]);
            else
                msm_reduce_pair(inA, inQ, m, D, bufA[pp], bufQ[pp], st);
            g_stats.launches++;
            inA = bufA[pp];
            inQ = bufQ[pp];
            pp ^= 1;
            m = m_out;
            first = false;
        }
        CATMSM_CHECK(cudaMemcpyAsync(wins, inQ ? inQ : inA, (size_t)D * sizeof(xyzz), cudaMemcpyDeviceToDevice, st));
    }
    g_stats.launches += 8;
    CATMSM_CHECK(cudaGetLastError());
    CATMSM_CHECK(cudaMemcpyAsync(h_wins, wins, (size_t)D * sizeof(xyzz), cudaMemcpyDeviceToHost, st));
    mark(7);
    CATMSM_CHECK(cudaStreamSynchronize(st));

    using namespace catmsm_host;
    hjac ret;
    std::memset(&ret, 0, sizeof(ret));
    for (uint32_t w = D; w-- > 0;) {
        hjac tile;
        from_device_xyzz(tile, h_wins + (size_t)w * 24);
        jac_add(ret, ret, tile);
        if (w)
            for (uint32_t i = 0; i < c; i++) jac_dbl(ret, ret);
    }
    hjac norm;
    normalize(norm, ret);
    std::memcpy(out, &norm, 144);
    if (P.enabled) {
        CATMSM_CHECK(cudaEventRecord(P.ev[kMsmStages], st));
        CATMSM_CHECK(cudaEventSynchronize(P.ev[kMsmStages]));
        for (int i = 0; i < kMsmStages; i++) {
            float ms = 0.f;
            CATMSM_CHECK(cudaEventElapsedTime(&ms, P.ev[i], P.ev[i + 1]));
            P.ms[i] += ms;
        }
        uint32_t E = 0;
        CATMSM_CHECK(cudaMemcpy(&E, total, 4, cudaMemcpyDeviceToHost));
        P.entries += E;
        P.calls++;
    }
    return cudaSuccess;
}

cudaError_t msm_device(Ctx* ctx, const void* d_points, const uint8_t* d_scalars, uint32_t stride, size_t n,
                       uint32_t nbits, uint32_t c, uint64_t* out, cudaEvent_t points_ready)
{
    return msm_run(ctx, d_points, d_scalars, stride, n, nbits, c, out, points_ready, 0, 0);
}

cudaError_t msm_tile_device(Ctx* ctx, const void* d_points, const uint8_t* d_scalars, uint32_t stride, size_t n,
                            uint32_t nbits, uint32_t bit0, uint32_t window, uint64_t* out)
{
    if (window < 1 || window > 24 || nbits == 0 || nbits > 256 || bit0 >= nbits) return cudaErrorInvalidValue;
    return msm_run(ctx, d_points, d_scalars, stride, n, nbits, 0, out, nullptr, bit0, window);
}

}  // namespace catmsm
