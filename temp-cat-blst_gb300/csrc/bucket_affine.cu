// Batch-affine bucket accumulation: the first rounds of every bucket's sum as
// affine additions behind Montgomery batch inversions, the rest with the XYZZ
// mixed addition.
//
// Reference precedent: the CPU batch-affine Pippenger
// (blst/scalar/curve/multi_scalar_batch_affine.cpp, bulk_addition.h), which
// adds points into affine buckets and shares one inversion among a batch of
// independent additions.  An affine addition P + Q = (l^2 - x1 - x2,
// l (x1 - x3) - y1) with l = (y2 - y1) / (x2 - x1) costs 2M + 1S plus its
// share of the inversion; Montgomery's trick makes that share 3M for a batch,
// so an addition is ~5M + 1S (3336 IMAD) against 8M + 2S for the XYZZ mixed
// addition (5340 IMAD as executed here).
//
// The sorted bucket entries are split into the same chunks of L entries as
// k_accumulate (thread t owns chunk t), so the fixup stage that joins buckets
// across chunks is unchanged.  A round halves each thread's runs: within each
// run of equal bucket keys, items (0,1), (2,3), ... are added and an odd last
// item passes through; the results form the thread's list for the next
// round, still in bucket order.  Round 1 reads the sorted entries (a gather
// of signed points); later rounds read the list the previous round wrote.
// A thread's lists, pair positions and prefix products are slot-major (see
// Slots), so a warp's accesses at one step of the loops are adjacent.
// One round is three launches:
//   forward   each thread walks its pairs from first to last, storing the
//             running product of the denominators before each pair (its
//             prefix) and ending with its total; the block multiplies its
//             threads' totals in a shared-memory tree;
//   invert    one thread per block inverts the block's product
//             (fp_inv_vartime: tens of microseconds, not Fermat's ~0.45 ms);
//   backward  the block re-forms the tree, pushes the inverse down to a
//             per-thread inverse of its total, and each thread walks its
//             pairs from last to first: inv(d_j) = prefix_j * I, I *= d_j,
//             then the affine sum.  The same kernel then runs the next
//             round's forward pass, or, after the last round, folds the
//             remaining list into the chunk's bucket / head / tail exactly as
//             k_accumulate does (XYZZ mixed additions).
// Special cases keep the group law complete: an infinity operand (all-zero
// affine) returns the other operand, x1 = x2 with y1 = y2 doubles
// (l = 3 x1^2 / 2 y1), x1 = x2 with y1 = -y2 gives infinity; their batch
// slots use the denominator 1 (or 2 y1 for the doubling).
#include "common.cuh"
#include "curve.cuh"
#include "fpinv.cuh"
#include "catmsm_internal.h"

namespace catmsm {

constexpr int kAffThreads = 128;
// Resident blocks per SM the round kernels are compiled for (register limit
// 65536 / (128 x this)).
#ifndef CATMSM_AFF_MIN_BLOCKS
#define CATMSM_AFF_MIN_BLOCKS 4
#endif

// 48 bytes (one coordinate) from a 16-byte aligned address.  Mutable: data
// this launch may write (a thread's own list slots, prefix products and
// totals, which only that thread writes and reads back), with plain loads --
// coherent with the thread's own earlier stores and cached in L1, so the two
// 16-byte halves of a sector and a thread's consecutive keys hit L1.  The
// others (read-only for the whole launch) take the read-only path.
template <bool Mutable>
__device__ __forceinline__ void load_coord(fp& c, const uint4* q)
{
#pragma unroll
    for (int k = 0; k < 3; k++) {
        const uint4 v = Mutable ? q[k] : __ldg(q + k);
        c.v[4 * k + 0] = v.x; c.v[4 * k + 1] = v.y; c.v[4 * k + 2] = v.z; c.v[4 * k + 3] = v.w;
    }
}

// 48-byte field elements in global memory as three 16-byte accesses (a
// plain struct copy is twelve 4-byte ones, each a separate sector per lane).
__device__ __forceinline__ void stg_fp(fp* dst, const fp& v)
{
    uint4* q = reinterpret_cast<uint4*>(dst);
#pragma unroll
    for (int k = 0; k < 3; k++) q[k] = make_uint4(v.v[4 * k], v.v[4 * k + 1], v.v[4 * k + 2], v.v[4 * k + 3]);
}

template <bool Mutable>
__device__ __forceinline__ fp ldg_fp(const fp* src)
{
    fp v;
    load_coord<Mutable>(v, reinterpret_cast<const uint4*>(src));
    return v;
}

// An item's 96-byte row and whether its y is negated.
struct Row {
    const uint4* p;
    bool neg;
};

// Items of round 1: sorted entry base + i, a signed point of the GLV array
// (read-only for the whole accumulation).
struct SrcSorted {
    static constexpr bool kMutable = false;
    const affine* pts;
    const uint32_t* sorted_pt;
    const uint32_t* sorted_key;
    size_t base;
    __device__ __forceinline__ uint32_t key(uint32_t i) const { return sorted_key[base + i]; }
    __device__ __forceinline__ Row row(uint32_t i) const
    {
        const uint32_t v = sorted_pt[base + i];
        return Row{reinterpret_cast<const uint4*>(pts + (v & 0x7fffffffu)), (v >> 31) != 0};
    }
};

// A thread's private arrays (lists, pair positions, prefix products) are
// slot-major: slot i of thread t is element i T + t (T threads in all), so
// the lanes of a warp at the same step of their loops touch adjacent
// elements instead of elements L apart.
struct Slots {
    size_t t, T;
    __device__ __forceinline__ size_t at(uint32_t i) const { return (size_t)i * T + t; }
};

// Items of later rounds: the thread's list.  Its slots may have been written
// earlier in the same launch (by this thread only).
struct SrcList {
    static constexpr bool kMutable = true;
    const affine* pts;
    const uint32_t* keys;
    Slots sl;
    __device__ __forceinline__ uint32_t key(uint32_t i) const { return keys[sl.at(i)]; }
    __device__ __forceinline__ Row row(uint32_t i) const
    {
        return Row{reinterpret_cast<const uint4*>(pts + sl.at(i)), false};
    }
};

template <class Src>
__device__ __forceinline__ void row_x(const Row& r, fp& x)
{
    load_coord<Src::kMutable>(x, r.p);
}

template <class Src>
__device__ __forceinline__ void row_y(const Row& r, fp& y)
{
    load_coord<Src::kMutable>(y, r.p + 3);
    if (r.neg) fp_neg(y, y);
}

enum : uint32_t { kPairAdd = 0, kPairDbl = 1, kPairInf = 2, kPairTakeA = 3, kPairTakeB = 4 };

// Kind of the pair (A, B) and its batch denominator.  Only x is needed for
// the common case; y is loaded when an x is zero or the x coordinates agree.
template <class Src>
__device__ __forceinline__ uint32_t pair_den(const Row& ra, const Row& rb, const fp& x1, const fp& x2, fp& d)
{
    fp_sub(d, x2, x1);
    if (!fp_is_zero_raw(x1) && !fp_is_zero_raw(x2) && !fp_is_zero(d)) return kPairAdd;
    fp y1, y2;
    row_y<Src>(ra, y1);
    row_y<Src>(rb, y2);
    fp_set_one(d);
    if (fp_is_zero_raw(x1) && fp_is_zero_raw(y1)) return kPairTakeB;
    if (fp_is_zero_raw(x2) && fp_is_zero_raw(y2)) return kPairTakeA;
    fp t;
    fp_sub(t, x2, x1);
    if (!fp_is_zero(t)) {
        fp_sub(d, x2, x1);
        return kPairAdd;
    }
    fp_sub(t, y2, y1);
    if (!fp_is_zero(t) || fp_is_zero(y1)) return kPairInf;   // P + (-P), or 2-torsion
    fp_dbl(d, y1);
    return kPairDbl;
}

template <class Src>
__device__ __forceinline__ void copy_item(const Src& src, uint32_t i, affine* dst)
{
    const Row r = src.row(i);
    affine a;
    row_x<Src>(r, a.x);
    row_y<Src>(r, a.y);
    store_affine(dst, a);
}

// Forward pass of one round over the thread's items [0, cnt).
//  Pairing: within each run of equal keys, items (0,1), (2,3), ... pair and an
//  odd last item is a singleton, copied to the output list now; pair slots get
//  their keys.  Keys are read four at a time, so the walk does not wait on one
//  load per item.
//  Prefix products: pair j stores d_0 ... d_{j-1}; the next pair's rows are
//  fetched before this pair's multiplication, so the row lookups (for round 1
//  an index load, then the point) overlap it.
// Returns the product of all denominators; *np_out = pairs, *cnt_out = items
// of the output list.
template <class Src>
__device__ __forceinline__ fp aff_forward(const Src& src, uint32_t cnt, affine* outP, uint32_t* outK, Slots os,
                                          uint32_t* pairpos, fp* prefix, Slots ps, uint32_t* np_out,
                                          uint32_t* cnt_out)
{
    uint32_t o = 0, np = 0, pi = 0, pk = 0;
    bool pend = false;
    for (uint32_t i0 = 0; i0 < cnt; i0 += 4) {
        uint32_t kk[4];
#pragma unroll
        for (int u = 0; u < 4; u++) kk[u] = i0 + u < cnt ? src.key(i0 + u) : 0;
#pragma unroll
        for (int u = 0; u < 4; u++) {
            const uint32_t i = i0 + u;
            if (i < cnt) {
                if (pend && kk[u] == pk) {
                    pairpos[ps.at(np)] = (pi << 16) | o;
                    outK[os.at(o)] = pk;
                    np++;
                    o++;
                    pend = false;
                } else {
                    if (pend) {
                        copy_item(src, pi, outP + os.at(o));
                        outK[os.at(o)] = pk;
                        o++;
                    }
                    pend = true;
                    pi = i;
                    pk = kk[u];
                }
            }
        }
    }
    if (pend) {
        copy_item(src, pi, outP + os.at(o));
        outK[os.at(o)] = pk;
        o++;
    }
    *np_out = np;
    *cnt_out = o;
    fp q;
    fp_set_one(q);
    if (np == 0) return q;
    uint32_t ip = pairpos[ps.at(0)] >> 16;
    Row ra = src.row(ip), rb = src.row(ip + 1);
    for (uint32_t j = 0; j < np; j++) {
        fp x1, x2, d;
        row_x<Src>(ra, x1);
        row_x<Src>(rb, x2);
        const Row ca = ra, cb = rb;
        if (j + 1 < np) {
            ip = pairpos[ps.at(j + 1)] >> 16;
            ra = src.row(ip);
            rb = src.row(ip + 1);
        }
        pair_den<Src>(ca, cb, x1, x2, d);
        stg_fp(prefix + ps.at(j), q);
        fp_mul(q, q, d);
    }
    return q;
}

// Backward pass of one round, pairs from last to first: I = inverse of
// d_0 ... d_j, inv(d_j) = prefix_j I, then I = I d_j; pair j's sum goes to
// its output slot.  The previous pair's rows are fetched before this pair's
// arithmetic.
template <class Src>
__device__ __forceinline__ void aff_backward(const Src& src, uint32_t np, affine* outP, Slots os,
                                             const uint32_t* pairpos, const fp* prefix, Slots ps, fp I)
{
    if (np == 0) return;
    uint32_t pp = pairpos[ps.at(np - 1)];
    Row ra = src.row(pp >> 16), rb = src.row((pp >> 16) + 1);
    for (uint32_t j = np; j-- > 0;) {
        fp x1, y1, x2, y2, d;
        row_x<Src>(ra, x1);
        row_x<Src>(rb, x2);
        row_y<Src>(ra, y1);
        row_y<Src>(rb, y2);
        const Row ca = ra, cb = rb;
        const uint32_t o = pp & 0xffffu;
        if (j > 0) {
            pp = pairpos[ps.at(j - 1)];
            ra = src.row(pp >> 16);
            rb = src.row((pp >> 16) + 1);
        }
        const uint32_t kind = pair_den<Src>(ca, cb, x1, x2, d);
        fp inv;
        fp_mul(inv, ldg_fp<true>(prefix + ps.at(j)), I);   // rewritten by the next forward pass
        fp_mul(I, I, d);
        affine r;
        if (kind == kPairAdd || kind == kPairDbl) {
            fp num, lam, t;
            if (kind == kPairAdd) {
                fp_sub(num, y2, y1);
            } else {
                fp_sqr(t, x1);
                fp_dbl(num, t);
                fp_add(num, num, t);
            }
            fp_mul(lam, num, inv);
            fp_sqr(t, lam);
            fp_sub(t, t, x1);
            fp_sub(r.x, t, x2);
            fp_sub(t, x1, r.x);
            fp_mul(t, lam, t);
            fp_sub(r.y, t, y1);
        } else if (kind == kPairTakeA) {
            r.x = x1;
            r.y = y1;
        } else if (kind == kPairTakeB) {
            r.x = x2;
            r.y = y2;
        } else {
            fp_zero(r.x);
            fp_zero(r.y);
        }
        store_affine(outP + os.at(o), r);
    }
}

// Product of the block's leaves in a shared-memory tree nd[1 .. 2T) (leaf of
// thread i at T + i, node n = nd[2n] * nd[2n + 1]); returns the root.
__device__ __forceinline__ fp block_product(fp* nd, const fp& leaf)
{
    const uint32_t T = kAffThreads, tid = threadIdx.x;
    nd[T + tid] = leaf;
    __syncthreads();
    for (uint32_t s = T / 2; s > 0; s >>= 1) {
        if (tid < s) fp_mul(nd[s + tid], nd[2 * (s + tid)], nd[2 * (s + tid) + 1]);
        __syncthreads();
    }
    return nd[1];
}

// With the tree of block_product in nd and the root's inverse: each node's
// inverse times its sibling is the sibling's inverse, top down; returns the
// inverse of this thread's leaf.
__device__ __forceinline__ fp block_leaf_inverse(fp* nd, const fp& root_inv)
{
    const uint32_t T = kAffThreads, tid = threadIdx.x;
    if (tid == 0) nd[1] = root_inv;
    __syncthreads();
    for (uint32_t s = 1; s < T; s <<= 1) {
        if (tid < s) {
            const uint32_t n = s + tid;
            const fp v = nd[n], a = nd[2 * n], b = nd[2 * n + 1];
            fp ia, ib;
            fp_mul(ia, v, b);
            fp_mul(ib, v, a);
            nd[2 * n] = ia;
            nd[2 * n + 1] = ib;
        }
        __syncthreads();
    }
    return nd[T + tid];
}

// k_accumulate's fold over the thread's final list: runs of equal keys are
// summed with XYZZ mixed additions; the chunk's first run goes to head[t] if
// the bucket started in an earlier chunk, its last run to tail[t] if the
// bucket continues into the next chunk, every other run to its bucket.
__device__ __forceinline__ void aff_fold(const SrcList& list, uint32_t cnt, const uint32_t* sorted_key,
                                         size_t start, uint32_t E, uint32_t L, uint32_t t, xyzz* buckets,
                                         xyzz* head, xyzz* tail)
{
    if (cnt == 0) return;
    const uint32_t end = (uint32_t)min((size_t)E, start + L);
    uint32_t cur = list.key(0);
    const bool starts_before = start > 0 && sorted_key[start - 1] == cur;
    bool first_run = true;
    xyzz acc;
    xyzz_set_inf(acc);
    for (uint32_t i = 0; i < cnt; i++) {
        const uint32_t key = list.key(i);
        if (key != cur) {
            if (first_run && starts_before) store_xyzz(head + t, acc);
            else store_xyzz(buckets + cur, acc);
            first_run = false;
            xyzz_set_inf(acc);
            cur = key;
        }
        fp x, y;
        const Row r = list.row(i);
        row_x<SrcList>(r, x);
        row_y<SrcList>(r, y);
        if (!(fp_is_zero_raw(x) && fp_is_zero_raw(y))) xyzz_madd(acc, x, y);
    }
    const bool continues_after = end < E && sorted_key[end] == cur;
    if (first_run && starts_before) store_xyzz(head + t, acc);
    else if (continues_after) store_xyzz(tail + t, acc);
    else store_xyzz(buckets + cur, acc);
}

struct AffArgs {
    const affine* pts;            // signed GLV points (round 1 items, through sorted_pt)
    const uint32_t* sorted_pt;
    const uint32_t* sorted_key;
    const uint32_t* total_ptr;    // E, the number of sorted entries
    uint32_t L, H;                // chunk length, pair slots per thread (ceil(L / 2))
    size_t T;                     // threads of the whole grid (both halves): the slot-major stride
    affine* list_pts[2];          // per-thread lists: slot i of thread t at i T + t
    uint32_t* list_key[2];
    uint32_t* meta;               // per thread: pairs | output items << 16 of the round in flight
    uint32_t* pairpos;            // pair j of thread t at j T + t: input position << 16 | output slot
    fp* prefix;                   // pair j of thread t at j T + t: its prefix product
    fp* ttot;                     // per thread: product of its denominators
    fp* btot;                     // per block: product of its threads' products, then its inverse
    xyzz* buckets;
    xyzz* head;
    xyzz* tail;
    uint32_t block0;              // first block of this launch (the rounds run as two halves)
};

// Round 1's forward pass, over the sorted entries.
__global__ void __launch_bounds__(kAffThreads, CATMSM_AFF_MIN_BLOCKS) k_aff_first(AffArgs A)
{
    __shared__ fp nd[2 * kAffThreads];
    const uint32_t blk = A.block0 + blockIdx.x;
    const uint32_t t = blk * blockDim.x + threadIdx.x;
    const uint32_t E = *A.total_ptr;
    const size_t start = (size_t)t * A.L;
    const uint32_t cnt = start < E ? (uint32_t)min((size_t)A.L, (size_t)E - start) : 0;
    const SrcSorted src{A.pts, A.sorted_pt, A.sorted_key, start};
    uint32_t np = 0, co = 0;
    const Slots sl{t, A.T};
    const fp tot = aff_forward(src, cnt, A.list_pts[0], A.list_key[0], sl, A.pairpos, A.prefix, sl, &np, &co);
    A.meta[t] = np | (co << 16);
    stg_fp(A.ttot + t, tot);
    const fp root = block_product(nd, tot);
    if (threadIdx.x == 0) stg_fp(A.btot + blk, root);
}

// One thread per block product: its inverse, in place (one inversion's
// latency for the whole launch).
__global__ void k_aff_invert(fp* __restrict__ btot, uint32_t nb)
{
    const uint32_t b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b < nb) {
        fp r;
        fp_inv_vartime(r, ldg_fp<true>(btot + b));   // overwritten below
        stg_fp(btot + b, r);
    }
}

// Backward pass of round r (inputs: the sorted entries if First, else list
// (r % 2); outputs: list ((r - 1) % 2)), then round r + 1's forward pass into
// list (r % 2), or, if Last, the fold into buckets / head / tail.
template <bool First, bool Last>
__global__ void __launch_bounds__(kAffThreads, CATMSM_AFF_MIN_BLOCKS) k_aff_round(AffArgs A, uint32_t r)
{
    __shared__ fp nd[2 * kAffThreads];
    const uint32_t blk = A.block0 + blockIdx.x;
    const uint32_t t = blk * blockDim.x + threadIdx.x;
    const uint32_t E = *A.total_ptr;
    const size_t start = (size_t)t * A.L;
    const Slots sl{t, A.T};
    const uint32_t m = A.meta[t];
    const uint32_t np = m & 0xffffu, co = m >> 16;
    block_product(nd, ldg_fp<true>(A.ttot + t));                  // both rewritten at the end of this launch
    const fp I = block_leaf_inverse(nd, ldg_fp<true>(A.btot + blk));
    const uint32_t out = (r - 1) & 1, in = r & 1;
    if (First) {
        const SrcSorted src{A.pts, A.sorted_pt, A.sorted_key, start};
        aff_backward(src, np, A.list_pts[out], sl, A.pairpos, A.prefix, sl, I);
    } else {
        const SrcList src{A.list_pts[in], A.list_key[in], sl};
        aff_backward(src, np, A.list_pts[out], sl, A.pairpos, A.prefix, sl, I);
    }
    const SrcList list{A.list_pts[out], A.list_key[out], sl};
    if (Last) {
        aff_fold(list, co, A.sorted_key, start, E, A.L, t, A.buckets, A.head, A.tail);
    } else {
        uint32_t np2 = 0, co2 = 0;
        const fp tot = aff_forward(list, co, A.list_pts[in], A.list_key[in], sl, A.pairpos, A.prefix, sl, &np2,
                                   &co2);
        A.meta[t] = np2 | (co2 << 16);
        stg_fp(A.ttot + t, tot);
        __syncthreads();                      // every leaf inverse of this round is read
        const fp root = block_product(nd, tot);
        if (threadIdx.x == 0) stg_fp(A.btot + blk, root);
    }
}

__global__ void k_fp_inv_test(const fp* __restrict__ a, fp* __restrict__ o, uint32_t n)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    fp r;
    fp_inv_vartime(r, a[i]);
    fp_canon(r, r);
    o[i] = r;
}

cudaError_t fp_inv_test_device(Ctx* ctx, const uint64_t* d_a, uint64_t* d_out, size_t n)
{
    k_fp_inv_test<<<div_up(n, 64), 64, 0, ctx->stream>>>((const fp*)d_a, (fp*)d_out, (uint32_t)n);
    g_stats.launches++;
    return cudaGetLastError();
}

// Rounds of batch-affine additions over the sorted entries, then the fold
// into the chunk's bucket / head / tail (the output contract of
// k_accumulate: the fixup stage joins chunk carries unchanged).  rounds >= 1.
// The blocks run as two independent halves, the first on st and the second
// on the context's second stream: an inversion launch (one inversion's
// latency, a few SMs busy) of one half overlaps the other half's round
// kernel instead of idling the GPU.
cudaError_t msm_accumulate_affine(Ctx* ctx, const void* pts, const uint32_t* sorted_pt, const uint32_t* sorted_key,
                                  const uint32_t* total, uint32_t L, size_t chunks, uint32_t rounds, void* buckets,
                                  void* head, void* tail, cudaStream_t st)
{
    if (rounds == 0 || L == 0 || L > 0xffffu) return cudaErrorInvalidValue;
    MsmWork& W = ctx->msm;
    const uint32_t H = (L + 1) / 2;
    const uint32_t grid = div_up(chunks, kAffThreads);
    const size_t threads = (size_t)grid * kAffThreads;
    AffArgs A;
    A.pts = (const affine*)pts;
    A.sorted_pt = sorted_pt;
    A.sorted_key = sorted_key;
    A.total_ptr = total;
    A.L = L;
    A.H = H;
    A.T = threads;
    A.list_pts[0] = (affine*)W.aff_pts0.get(threads * L * sizeof(affine));
    A.list_pts[1] = (affine*)W.aff_pts1.get(threads * L * sizeof(affine));
    A.list_key[0] = (uint32_t*)W.aff_key0.get(threads * L * 4);
    A.list_key[1] = (uint32_t*)W.aff_key1.get(threads * L * 4);
    A.meta = (uint32_t*)W.aff_meta.get(threads * 4);
    A.pairpos = (uint32_t*)W.aff_pairpos.get(threads * H * 4);
    A.prefix = (fp*)W.aff_prefix.get(threads * H * sizeof(fp));
    A.ttot = (fp*)W.aff_ttot.get(threads * sizeof(fp));
    A.btot = (fp*)W.aff_btot.get((size_t)grid * sizeof(fp));
    A.buckets = (xyzz*)buckets;
    A.head = (xyzz*)head;
    A.tail = (xyzz*)tail;
    if (!A.list_pts[0] || !A.list_pts[1] || !A.list_key[0] || !A.list_key[1] || !A.meta || !A.pairpos ||
        !A.prefix || !A.ttot || !A.btot)
        return cudaErrorMemoryAllocation;
    if (!ctx->aff_stream) {
        int prio = 0;
        CATMSM_CHECK(cudaStreamGetPriority(st, &prio));     // the second half runs at the pipeline stream's priority
        CATMSM_CHECK(cudaStreamCreateWithPriority(&ctx->aff_stream, cudaStreamNonBlocking, prio));
        CATMSM_CHECK(cudaEventCreateWithFlags(&ctx->aff_fork, cudaEventDisableTiming));
        CATMSM_CHECK(cudaEventCreateWithFlags(&ctx->aff_join, cudaEventDisableTiming));
    }
    const uint32_t half0 = (grid + 1) / 2;
    const uint32_t nblk[2] = {half0, grid - half0};
    const uint32_t blk0[2] = {0, half0};
    cudaStream_t sts[2] = {st, ctx->aff_stream};
    const int halves = nblk[1] ? 2 : 1;
    if (halves == 2) {
        CATMSM_CHECK(cudaEventRecord(ctx->aff_fork, st));
        CATMSM_CHECK(cudaStreamWaitEvent(sts[1], ctx->aff_fork, 0));
    }
    for (int h = 0; h < halves; h++) {
        A.block0 = blk0[h];
        k_aff_first<<<nblk[h], kAffThreads, 0, sts[h]>>>(A);
    }
    for (uint32_t r = 1; r <= rounds; r++) {
        const bool first = r == 1, last = r == rounds;
        for (int h = 0; h < halves; h++)
            k_aff_invert<<<div_up(nblk[h], 32), 32, 0, sts[h]>>>(A.btot + blk0[h], nblk[h]);
        for (int h = 0; h < halves; h++) {
            A.block0 = blk0[h];
            if (first && last) k_aff_round<true, true><<<nblk[h], kAffThreads, 0, sts[h]>>>(A, r);
            else if (first) k_aff_round<true, false><<<nblk[h], kAffThreads, 0, sts[h]>>>(A, r);
            else if (last) k_aff_round<false, true><<<nblk[h], kAffThreads, 0, sts[h]>>>(A, r);
            else k_aff_round<false, false><<<nblk[h], kAffThreads, 0, sts[h]>>>(A, r);
        }
        g_stats.launches += 2 * halves;
    }
    g_stats.launches += halves;
    CATMSM_CHECK(cudaGetLastError());
    if (halves == 2) {
        CATMSM_CHECK(cudaEventRecord(ctx->aff_join, sts[1]));
        CATMSM_CHECK(cudaStreamWaitEvent(st, ctx->aff_join, 0));
    }
    return cudaSuccess;
}

}  // namespace catmsm
