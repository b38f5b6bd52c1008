// Internal declarations shared by the library's translation units.
#pragma once
#include "common.cuh"
#include "catmsm_gpu.h"

namespace catmsm {

uint32_t msm_default_window(size_t n);

// Bucket-count scan (k_scan_local / k_scan_top / k_scan_add in msm.cu): a
// block of kScanThreads threads scans a tile of kScanTile counts, so M counts
// need ceil(M / kScanTile) block sums.
constexpr int kScanThreads = 1024;
constexpr int kScanPer = 4;
constexpr int kScanTile = kScanThreads * kScanPer;

// Resident basis with fixed-base tables (batch.cu) and per-worker workspaces.
struct Basis;
struct BatchWork;
BatchWork* batch_work_new();
void batch_work_free(BatchWork* w);
// nmsm MSMs over the basis prefixes counts[j] with 32-byte scalars
// (concatenated); Jacobian results to host `out`; synchronous on stream st.
cudaError_t batch_run(Basis* b, BatchWork* w, cudaStream_t st, blst_p1* out, uint32_t nmsm,
                      const size_t* counts, const uint8_t* scalars);
size_t basis_points(const Basis* b);
uint32_t basis_window(const Basis* b);
int basis_device(const Basis* b);
// The basis points (affine, device memory) of the resident basis.
const void* basis_points_device(const Basis* b);

// Window width, window count and pipeline point count msm_device uses for
// n points of nbits-bit scalars on this context (2n points of 127 bits when
// the GLV split applies).
void msm_plan_detail(size_t n, uint32_t nbits, bool glv, uint32_t* c, uint32_t* windows, size_t* points,
                     uint32_t* chunk, uint32_t* fan_in);
void msm_plan(const Ctx* ctx, size_t n, uint32_t nbits, uint32_t* c, uint32_t* windows, size_t* points);

// Per-device set-up of the MSM kernels (shared-memory limits), run once per
// context.
cudaError_t msm_setup_device();

// The fused last reduction levels for D independent sets of m (A, Q) XYZZ
// pairs (m <= msm_reduce_tail_max(D)); roots to outQ[0..D).
uint32_t msm_reduce_tail_max(uint32_t D);
void msm_reduce_tail(const void* inA, const void* inQ, uint32_t m, uint32_t D, void* outQ, cudaStream_t st);
// Joins of buckets whose carries span more than 1024 partials, by the whole
// grid (after k_fixup_hot / k_fixup_hot_seg; seg = the segmented fixup).
void fixup_giants(const void* hot_list, const uint32_t* hot_count, const uint32_t* offsets, uint32_t L,
                  void* buckets, void* head, void* tail, bool seg, cudaStream_t st);
// One binary reduction level (fan-in 2) over D sets of m (A, Q) pairs.
void msm_reduce_pair(const void* inA, const void* inQ, uint32_t m, uint32_t D, void* outA, void* outQ,
                     cudaStream_t st);

// Bucket accumulation with `rounds` rounds of batch-affine additions
// (Montgomery batch inversion per block and round) before the XYZZ fold;
// same outputs as k_accumulate (buckets / head / tail per chunk of L sorted
// entries), so the fixup stage is unchanged.
cudaError_t msm_accumulate_affine(Ctx* ctx, const void* pts, const uint32_t* sorted_pt, const uint32_t* sorted_key,
                                  const uint32_t* total, uint32_t L, size_t chunks, uint32_t rounds, void* buckets,
                                  void* head, void* tail, cudaStream_t st);
// Rounds the plain MSM uses for nD bucket entries over M buckets (0: the
// XYZZ-only k_accumulate).
uint32_t msm_affine_rounds(size_t nD, size_t M);

// H2D of `bytes` from src to dst on the context's copy stream, after the work
// already queued on its pipeline stream; *ready is an event recorded after
// the copy (pass it to msm_device as points_ready).
cudaError_t copy_points_async(Ctx* ctx, void* dst, const void* src, size_t bytes, cudaEvent_t* ready);

cudaError_t msm_device(Ctx* ctx, const void* d_points, const uint8_t* d_scalars, uint32_t stride,
                       size_t n, uint32_t nbits, uint32_t c, uint64_t* out, cudaEvent_t points_ready = nullptr);

// One window of the reference's tile MSM (blst_p1s_tile_pippenger) over
// device-resident inputs: sum_i d_i P_i with d_i the Booth digit of bits
// [bit0, bit0 + window) of scalar i (window in [1, 24], bit0 < nbits).
cudaError_t msm_tile_device(Ctx* ctx, const void* d_points, const uint8_t* d_scalars, uint32_t stride, size_t n,
                            uint32_t nbits, uint32_t bit0, uint32_t window, uint64_t* out);

cudaError_t points_from_scalars_device(Ctx* ctx, const uint8_t* d_k32, size_t n, void* d_out);

// d_out[i] = d_a[i]^-1 (Montgomery form, canonical; 0 -> 0) by the
// variable-time inversion of the batch-affine rounds.
cudaError_t fp_inv_test_device(Ctx* ctx, const uint64_t* d_a, uint64_t* d_out, size_t n);

cudaError_t fp_mul_test_device(Ctx* ctx, const uint64_t* d_a, const uint64_t* d_b, uint64_t* d_out, size_t n,
                               bool square);

// One transform of a batch: n points, the n Montgomery roots its butterflies
// index, whether the inverse reads forward roots at n - idx, and an optional
// Montgomery scale applied to every output (all device pointers).
struct FftSpec {
    size_t n;
    const uint32_t* roots_mont;
    bool inv_from_fwd;
    const uint32_t* scale_mont;
    size_t xn = 0;          // forward transforms: inputs [xn, n) are the identity (0 = none known)
};

// Every transform of `specs` over the concatenated values in d_values.
cudaError_t fft_run_multi(Ctx* ctx, void* d_values, const FftSpec* specs, size_t count);

// G1 FFT over device-resident Jacobian values (blst_p1 layout).
// d_roots_mont: the n Montgomery-form Fr roots the butterflies index;
// inv_from_fwd: read index n - j*(n/len) (inverse from forward roots);
// d_scale_mont: optional Montgomery-form Fr applied to every output.
cudaError_t fft_run(Ctx* ctx, void* d_values, size_t n, const uint32_t* d_roots_mont, bool inv_from_fwd,
                    const uint32_t* d_scale_mont, size_t xn = 0);

// d_out[i] = w^i (Montgomery), i < n
cudaError_t fft_root_powers(Ctx* ctx, const uint32_t* d_w_mont, size_t n, uint32_t* d_out);

}  // namespace catmsm
