// The reference's fixed-table MSM API on the GPU (blst/c_api.cpp:1310-1369;
// scalar/curve/multi_scalar.h:245-315; multi_scalar.cpp:297-720).
//
// blst_p1s_mult_wbits_precompute writes the reference's table: per point i a
// row of the 2^(wbits-1) affine multiples [P_i, 2 P_i, ..., 2^(wbits-1) P_i]
// (Montgomery, reduced; infinity rows all-zero).  On the GPU every thread
// builds 64 consecutive entries of the flat table and normalises them with one
// inversion; the rows go back to the caller's table slab by slab.
//
// blst_p1s_mult_wbits evaluates sum_i k_i P_i.  Its result is a group element,
// so the GPU runs its Pippenger pipeline over the rows' first entries (the
// points themselves): only n x 96 bytes of the table cross the bus, and the
// output equals the reference's table method.
#include "common.cuh"
#include "curve.cuh"
#include "catmsm_internal.h"
#include "catmsm_gpu.h"

#include <algorithm>

namespace catmsm {

constexpr uint32_t kRowChunk = 64;            // table entries per thread (one inversion)
constexpr size_t kSlabEntries = size_t(1) << 22;  // table entries per launch (384 MB of rows)

// Thread t writes the flat table entries e = 64 t .. 64 t + 63 of rows
// row0 .. row0 + rows - 1; entry e is (e % m + 1) * P[e / m].  m is a power of
// two, so a thread's entries lie in one row (m >= 64) or cover whole rows.
// The multiples are built in XYZZ (a double-and-add to the first one, then one
// mixed addition per entry) and normalised with one inversion per thread.
__global__ void __launch_bounds__(64) k_wbits_rows(const affine* __restrict__ pts, uint32_t row0, uint32_t rows,
                                                   uint32_t m, affine* __restrict__ out, xyzz* __restrict__ tmp,
                                                   fp* __restrict__ pre_buf)
{
    const uint32_t total = rows * m;
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t e0 = t * kRowChunk;
    if (e0 >= total) return;
    const uint32_t cnt = min(kRowChunk, total - e0);
    xyzz* q = tmp + (size_t)t * kRowChunk;
    fp* pre = pre_buf + (size_t)t * kRowChunk;
    xyzz acc;
    affine p;
    bool pinf = true;
    fp prod;
    fp_set_one(prod);
    for (uint32_t k = 0; k < cnt; k++) {
        const uint32_t e = e0 + k;
        const uint32_t j = e & (m - 1);
        if (k == 0 || j == 0) {
            p = pts[row0 + e / m];
            pinf = aff_is_inf(p);
            xyzz_set_inf(acc);
            if (!pinf) {
                for (int bit = 31 - __clz(j + 1); bit >= 0; bit--) {   // acc = (j + 1) P
                    xyzz_dbl(acc);
                    if (((j + 1) >> bit) & 1) xyzz_madd(acc, p.x, p.y);
                }
            }
        } else if (!pinf) {
            xyzz_madd(acc, p.x, p.y);
        }
        q[k] = acc;
        pre[k] = prod;
        if (!xyzz_is_inf(acc)) {
            fp s;
            fp_mul(s, acc.zz, acc.zzz);
            fp_mul(prod, prod, s);
        }
    }
    fp inv;
    fp_inv(inv, prod);
    for (int k = (int)cnt - 1; k >= 0; k--) {
        const xyzz v = q[k];
        affine o;
        if (xyzz_is_inf(v)) {
            fp_zero(o.x);
            fp_zero(o.y);
        } else {
            fp s, iv, u;
            fp_mul(s, v.zz, v.zzz);
            fp_mul(iv, inv, pre[k]);       // 1 / (zz zzz) of entry k
            fp_mul(inv, inv, s);
            fp_mul(u, iv, v.zzz);          // 1 / zz
            fp_mul(o.x, v.x, u);
            fp_mul(u, iv, v.zz);           // 1 / zzz
            fp_mul(o.y, v.y, u);
            fp_canon(o.x, o.x);
            fp_canon(o.y, o.y);
        }
        out[e0 + k] = o;
    }
}

static bool valid_wbits(size_t w) { return w >= 2 && w <= 14; }

// 96 * n * 2^(w-1) with the reference's overflow rules
static size_t table_bytes(size_t wbits, size_t n)
{
    if (!valid_wbits(wbits)) return 0;
    if (n != 0 && 96 > SIZE_MAX / n) return 0;
    const size_t b = 96 * n;
    if (b > (SIZE_MAX >> (wbits - 1))) return 0;
    return b << (wbits - 1);
}

}  // namespace catmsm

using namespace catmsm;

extern "C" {

size_t blst_p1s_mult_wbits_precompute_sizeof(size_t wbits, size_t npoints) { return table_bytes(wbits, npoints); }

void blst_p1s_mult_wbits_precompute(blst_p1_affine table[], size_t wbits, const blst_p1_affine* const points[],
                                    size_t npoints)
{
    try {
        if (!valid_wbits(wbits) || (npoints != 0 && !table) ||
            (npoints != 0 && (!points || !points[0])))
            return;
        if (npoints == 0) return;
        const size_t m = (size_t)1 << (wbits - 1);
        if (table_bytes(wbits, npoints) == 0 || npoints > 0x7fffffffu) return;
        Ctx* ctx = get_ctx();
        if (!ctx) return;
        cudaStream_t st = ctx->stream;
        // The descriptor walk is read (and copied to the device, in stream
        // order) before the table is written: packed points may share storage
        // with the table's tail.
        bool gerr;
        const uint8_t* hp = gather(points, npoints, sizeof(blst_p1_affine), ctx->h_points, gerr);
        if (gerr) return;
        const size_t slab_rows = m >= kSlabEntries ? 1 : std::min(npoints, kSlabEntries / m);
        const size_t slab_entries = slab_rows * m;
        const size_t slab_threads = (slab_entries + kRowChunk - 1) / kRowChunk;
        affine* dp = (affine*)ctx->msm.points.get(npoints * sizeof(affine));
        affine* dt = (affine*)ctx->msm.buckets.get(slab_entries * sizeof(affine));
        xyzz* tmp = (xyzz*)ctx->msm.seg.get(slab_threads * kRowChunk * (sizeof(xyzz) + sizeof(fp)));
        if (!dp || !dt || !tmp) return;
        fp* pre = (fp*)(tmp + slab_threads * kRowChunk);
        cudaError_t err = cudaMemcpyAsync(dp, hp, npoints * sizeof(affine), cudaMemcpyHostToDevice, st);
        for (size_t r0 = 0; r0 < npoints && err == cudaSuccess; r0 += slab_rows) {
            const size_t rows = std::min(slab_rows, npoints - r0);
            const size_t threads = (rows * m + kRowChunk - 1) / kRowChunk;
            k_wbits_rows<<<div_up(threads, 64), 64, 0, st>>>(dp, (uint32_t)r0, (uint32_t)rows, (uint32_t)m, dt,
                                                            tmp, pre);
            g_stats.launches++;
            err = cudaGetLastError();
            if (err == cudaSuccess)
                err = cudaMemcpyAsync(table + r0 * m, dt, rows * m * sizeof(affine), cudaMemcpyDeviceToHost, st);
        }
        if (err == cudaSuccess) err = cudaStreamSynchronize(st);
    } catch (...) {
    }
}

size_t blst_p1s_mult_wbits_scratch_sizeof(size_t npoints) { return 144 * (npoints < 8192 ? npoints : 8192); }

void blst_p1s_mult_wbits(blst_p1* ret, const blst_p1_affine table[], size_t wbits, size_t npoints,
                         const blst_byte* const scalars[], size_t nbits, blst_limb_t* scratch)
{
    try {
        if (!ret) return;
        std::memset(ret, 0, sizeof(*ret));
        if (npoints == 0 || nbits == 0) return;
        if (nbits > 256 || !valid_wbits(wbits) || !table || !scalars || !scalars[0] || !scratch) return;
        if (npoints > (SIZE_MAX >> (wbits - 1)) || npoints > 0x7fffffffu) return;
        const size_t m = (size_t)1 << (wbits - 1);
        Ctx* ctx = get_ctx();
        if (!ctx) return;
        cudaStream_t st = ctx->stream;
        const size_t nbytes = (nbits + 7) / 8;
        bool gerr;
        const uint8_t* hs = gather(scalars, npoints, nbytes, ctx->h_scalars, gerr);
        if (gerr) return;
        void* dp = ctx->msm.points.get(npoints * sizeof(blst_p1_affine));
        void* ds = ctx->msm.scalars.get(npoints * nbytes + 16);
        // row heads table[i * m] gathered into pinned staging: one dense copy
        blst_p1_affine* heads = (blst_p1_affine*)ctx->h_points.get(npoints * sizeof(blst_p1_affine));
        if (!dp || !ds || !heads) return;
        for (size_t i = 0; i < npoints; i++) heads[i] = table[i * m];
        cudaError_t err = cudaMemcpyAsync(dp, heads, npoints * sizeof(blst_p1_affine), cudaMemcpyHostToDevice, st);
        if (err == cudaSuccess) err = cudaMemcpyAsync(ds, hs, npoints * nbytes, cudaMemcpyHostToDevice, st);
        uint64_t out[18];
        if (err == cudaSuccess)
            err = msm_device(ctx, dp, (const uint8_t*)ds, (uint32_t)nbytes, npoints, (uint32_t)nbits, 0, out);
        if (err != cudaSuccess) {
            std::memset(ret, 0, sizeof(*ret));
            return;
        }
        std::memcpy(ret, out, sizeof(*ret));
    } catch (...) {
        if (ret) std::memset(ret, 0, sizeof(*ret));
    }
}

}  // extern "C"
