/*
 * catmsm-gb300: BLS12-381 G1 multi-scalar multiplication and G1 group FFT on
 * one sm_103a GPU, behind the category-blst C ABI.
 *
 * Part 1 declares the drop-in entry points.  Each has the exact name,
 * signature, argument meaning and fail-closed behaviour of the reference
 * function cited beside it (paths are within the reference project).  All
 * buffers are caller-owned HOST memory; every call is synchronous; no
 * exception or abort crosses the boundary.  Device memory, streams and
 * pinned staging are owned per calling thread inside the library.
 *
 * Part 2 declares device-resident and tooling entry points that have no
 * reference counterpart (resident inputs for serving/benchmarks, seeded
 * input generation, field self-checks).
 */
#ifndef CATMSM_GPU_H
#define CATMSM_GPU_H

#include <stdbool.h>
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Reference ABI types (bindings/blst_types.h:40-103), byte-identical. */
typedef uint8_t blst_byte;
typedef uint64_t blst_limb_t;
typedef struct { blst_limb_t l[4]; } blst_fr;             /* Montgomery, R = 2^256 */
typedef struct { blst_limb_t l[6]; } blst_fp;             /* Montgomery, R = 2^384 */
typedef struct { blst_fp x, y, z; } blst_p1;              /* Jacobian; z == 0 is infinity */
typedef struct { blst_fp x, y; } blst_p1_affine;          /* all-zero is infinity */

/* ------------------------------------------------------------------ Part 1 */

/* Replaces blst_p1s_mult_pippenger_scratch_sizeof
 * (bindings/blst_scalar.h:535, blst/c_api.cpp:1371).  Returns the reference's
 * value, 192 * 2^(c(n)-1) bytes (0 for n = 0), so callers size scratch as
 * before; the GPU path itself does not touch the scratch. */
size_t blst_p1s_mult_pippenger_scratch_sizeof(size_t npoints);

/* Replaces blst_p1s_mult_pippenger_window_scratch_sizeof
 * (bindings/blst_scalar.h:537, blst/c_api.cpp:1376): 0 for window outside [1, 24]. */
size_t blst_p1s_mult_pippenger_window_scratch_sizeof(size_t window);

/* Replaces blst_p1s_mult_pippenger (bindings/blst_scalar.h:539,
 * blst/c_api.cpp:1382-1418).  ret = sum_i k_i * P_i, k_i the low nbits bits
 * of scalars[i] (ceil(nbits/8) little-endian bytes).  Descriptor arrays:
 * a later NULL entry means contiguous continuation from the previous entry
 * (blst/scalar/curve/multi_scalar.cpp:838-841); exact n-entry arrays are read
 * without a sentinel.  npoints == 0 or nbits == 0 -> infinity; nbits > 256 or
 * a NULL head pointer -> infinity; npoints > 1 with scratch == NULL ->
 * infinity; a device failure also writes infinity.  The result is written
 * normalised (z = Montgomery one, or all-zero for infinity). */
void blst_p1s_mult_pippenger(blst_p1 *ret, const blst_p1_affine *const points[], size_t npoints,
                             const blst_byte *const scalars[], size_t nbits, blst_limb_t *scratch);

/* Replaces blst_p1s_mult_pippenger_window (bindings/blst_scalar.h:603,
 * blst/c_api.cpp:1546-1583): as above; window outside [1, 24] -> infinity.
 * The window is accepted for validation only: the GPU picks its own width,
 * which leaves the result (a group element) unchanged. */
void blst_p1s_mult_pippenger_window(blst_p1 *ret, const blst_p1_affine *const points[], size_t npoints,
                                    const blst_byte *const scalars[], size_t nbits, blst_limb_t *scratch,
                                    size_t window);

/* Replaces blst_p1s_tile_pippenger (bindings/blst_scalar.h:605,
 * blst/c_api.cpp:1585-1612 -> scalar/curve/multi_scalar.cpp:806-864): one
 * signed window of the Pippenger MSM, ret = sum_i d_i P_i with d_i the Booth
 * digit of bits [bit0, bit0 + window) of scalar i (overlap bit bit0 - 1;
 * encode size min(nbits - bit0 + 1, window)).  npoints == 0, a NULL head or
 * scratch, window outside [1, 24], nbits outside [1, 256] or bit0 >= nbits
 * -> infinity.  The result is written normalised. */
void blst_p1s_tile_pippenger(blst_p1 *ret, const blst_p1_affine *const points[], size_t npoints,
                             const blst_byte *const scalars[], size_t nbits, blst_limb_t *scratch, size_t bit0,
                             size_t window);

/* Replaces blst_fr_fft_domain_len (bindings/blst_fft.h:52, blst/fft_c_api.cpp:128):
 * n + 2 for n a power of two in [1, 2^30], else 0. */
size_t blst_fr_fft_domain_len(size_t n);

/* Replaces blst_fr_fft_domain_init (bindings/blst_fft.h:65, blst/fft_c_api.cpp:133-146):
 * domain = [w^0 .. w^(n-1), 1/n, n] in Montgomery form, w the reference's
 * primitive n-th root.  false (contents unspecified) on a bad length/size. */
bool blst_fr_fft_domain_init(blst_fr *domain, size_t domain_len, size_t n);

/* Replaces blst_p1_fft (bindings/blst_fft.h:109, blst/fft_c_api.cpp:184 -> :51-66):
 * in-place natural-order G1 DFT with powers of the primitive n-th root
 * (inverse: of its reciprocal, then scaled by 1/n).  false before writing on
 * NULL values or invalid n; false with values untouched on a device failure. */
bool blst_p1_fft(blst_p1 *values, size_t n, bool inverse);

/* Replaces blst_p1_fft_with_domain (bindings/blst_fft.h:111, blst/fft_c_api.cpp:194 ->
 * :68-103): domain_len must be n + 2 and domain[n+1] the Montgomery tag n, else
 * false before writing; inverse reads forward roots at n - idx and scales by
 * domain[n]. */
bool blst_p1_fft_with_domain(blst_p1 *values, size_t n, const blst_fr *domain, size_t domain_len,
                             bool inverse);

/* Replaces blst_p1_ifft_unscaled_with_domain (bindings/blst_fft.h:131,
 * blst/fft_c_api.cpp:208): the inverse transform without the 1/n scale. */
bool blst_p1_ifft_unscaled_with_domain(blst_p1 *values, size_t n, const blst_fr *domain, size_t domain_len);

/* Replaces blst_p1s_mult_pippenger_fr_scratch_sizeof (bindings/blst_scalar.h:541,
 * blst/c_api.cpp:1420 -> :271-296): n*32 scalar bytes plus 192 * 2^(c(n)-1)
 * bucket bytes for n > 1; 0 for n == 0 or an unrepresentable size. */
size_t blst_p1s_mult_pippenger_fr_scratch_sizeof(size_t npoints);

/* Replaces blst_p1s_mult_pippenger_fr (bindings/blst_scalar.h:549,
 * blst/c_api.cpp:1425-1435 -> :532-585): MSM of contiguous points with
 * Montgomery-form blst_fr scalars (converted to canonical integers, 255 bits).
 * NULL ret -> false; n == 0 -> infinity and true; NULL points/scalars/scratch
 * or scratch_size below the queried size -> false with ret unchanged. */
bool blst_p1s_mult_pippenger_fr(blst_p1 *ret, const blst_p1_affine points[], const blst_fr scalars[],
                                size_t npoints, blst_limb_t *scratch, size_t scratch_size);

/* Replaces blst_fr_fft (bindings/blst_fft.h:41, blst/fft_c_api.cpp:109-126):
 * in-place Fr DFT with powers of the primitive n-th root (inverse: of its
 * reciprocal, scaled by 1/n); false before writing on NULL or invalid n. */
bool blst_fr_fft(blst_fr *values, size_t n, bool inverse);

/* Replaces blst_fr_fft_with_domain (bindings/blst_fft.h:87, blst/fft_c_api.cpp:
 * 150-182): prepared-domain Fr DFT; the inverse reads forward roots at n - idx
 * and scales by domain[n]; false before writing on a bad length or tag. */
bool blst_fr_fft_with_domain(blst_fr *values, size_t n, const blst_fr *domain, size_t domain_len, bool inverse);

/* Replaces blst_p1s_mult_wbits_precompute_sizeof (bindings/blst_scalar.h:527,
 * blst/c_api.cpp:1310-1316 -> scalar/curve/multi_scalar.h:245-255):
 * 96 * npoints * 2^(wbits-1); 0 for wbits outside [2, 14] or on overflow. */
size_t blst_p1s_mult_wbits_precompute_sizeof(size_t wbits, size_t npoints);

/* Replaces blst_p1s_mult_wbits_precompute (bindings/blst_scalar.h:529,
 * blst/c_api.cpp:1318-1330 -> scalar/curve/multi_scalar.cpp:481-565): row i
 * of the table is [P_i, 2 P_i, ..., 2^(wbits-1) P_i], affine, Montgomery,
 * fully reduced, all-zero for infinity.  Invalid wbits, a NULL table or a
 * NULL head with npoints != 0 return without writing.  Packed points may sit
 * in the final npoints entries of the table: every point is read before the
 * first table entry is written. */
void blst_p1s_mult_wbits_precompute(blst_p1_affine table[], size_t wbits, const blst_p1_affine *const points[],
                                    size_t npoints);

/* Replaces blst_p1s_mult_wbits_scratch_sizeof (bindings/blst_scalar.h:531,
 * blst/c_api.cpp:1332-1335 -> scalar/curve/multi_scalar.h:310-315):
 * 144 * min(npoints, 8192); the GPU path does not touch the scratch. */
size_t blst_p1s_mult_wbits_scratch_sizeof(size_t npoints);

/* Replaces blst_p1s_mult_wbits (bindings/blst_scalar.h:533,
 * blst/c_api.cpp:1337-1369 -> scalar/curve/multi_scalar.cpp:600-720):
 * ret = sum_i k_i P_i over a table made by blst_p1s_mult_wbits_precompute;
 * scalars as for blst_p1s_mult_pippenger.  npoints == 0 or nbits == 0 ->
 * infinity; nbits > 256, wbits outside [2, 14], a NULL table, scalar head or
 * scratch -> infinity.  Only the rows' first entries (the points) are read. */
void blst_p1s_mult_wbits(blst_p1 *ret, const blst_p1_affine table[], size_t wbits, size_t npoints,
                         const blst_byte *const scalars[], size_t nbits, blst_limb_t *scratch);

/* Replaces blst_p1s_mult_fr_scratch_sizeof (bindings/blst_scalar.h:592,
 * blst/c_api.cpp:1502-1506 -> :758-807): the reference policy MSM's capacity
 * query, the larger of the Pippenger and the planned batch-affine sizes. */
size_t blst_p1s_mult_fr_scratch_sizeof(size_t max_points);

/* Replaces blst_p1s_mult_fr (bindings/blst_scalar.h:597, blst/c_api.cpp:
 * 1508-1520 -> :809-850): same contract as blst_p1s_mult_pippenger_fr with
 * the policy scratch size above. */
bool blst_p1s_mult_fr(blst_p1 *ret, const blst_p1_affine points[], const blst_fr scalars[], size_t npoints,
                      blst_limb_t *scratch, size_t scratch_size);

/* Replaces blst_p1s_mult_batch_affine_fr_scratch_sizeof (bindings/blst_scalar.h:
 * 599, blst/c_api.cpp:1522-1529 -> :593-639): 32 n + 256 * 2^(window-1) +
 * 108 * batch_size (32 for n == 1); 0 for n == 0, n >= 2^32, window outside
 * [1, 24] or batch_size not 128 or 384. */
size_t blst_p1s_mult_batch_affine_fr_scratch_sizeof(size_t npoints, size_t window, size_t batch_size);

/* Replaces blst_p1s_mult_batch_affine_fr (bindings/blst_scalar.h:601,
 * blst/c_api.cpp:1531-1545 -> :641-690): NULL ret -> false; n == 0 ->
 * infinity and true; an invalid window/batch size, NULL inputs or scratch
 * below the queried size -> false with ret unchanged.  window and batch_size
 * select the reference's CPU schedule; the GPU computes the same group
 * element with its own. */
bool blst_p1s_mult_batch_affine_fr(blst_p1 *ret, const blst_p1_affine points[], const blst_fr scalars[],
                                   size_t npoints, blst_limb_t *scratch, size_t scratch_size, size_t window,
                                   size_t batch_size);

/* ------------------------------------------------------------------ Part 2 */

/* MSM over DEVICE-resident inputs (no reference counterpart): d_points is n
 * contiguous affine points (16-byte aligned), d_scalars n scalars of `stride`
 * bytes (nbits used), all in device memory of the current device; window 0 =
 * library default.
 * Runs on the calling thread's library stream; the result lands in host *ret.
 * Returns 0 on success, else a cudaError_t value (ret set to infinity). */
int catmsm_p1s_mult_pippenger_device(blst_p1 *ret, const void *d_points, const void *d_scalars,
                                     size_t stride, size_t npoints, size_t nbits, size_t window);

/* G1 FFT over DEVICE-resident Jacobian values (16-byte aligned) with a DEVICE-resident domain
 * (n + 2 Montgomery Fr, as built by blst_fr_fft_domain_init).  mode 0:
 * forward, 1: inverse (scaled), 2: inverse unscaled.  Returns 0 on success. */
int catmsm_p1_fft_device(void *d_values, size_t n, const void *d_domain, int mode);

/* A batch of G1 FFTs in one pass (no reference counterpart): transform i is
 * blst_p1_fft_with_domain(values[i], ns[i], domains[i], ns[i] + 2, ...) with
 * modes[i] = 0 forward, 1 inverse (scaled by domain[n]), 2 inverse unscaled
 * (as blst_p1_ifft_unscaled_with_domain).  Sizes may differ; every stage
 * level runs as one launch over all transforms that have it.  Any invalid
 * entry (NULL values, bad size, domain length or tag, bad mode) returns
 * cudaErrorInvalidValue before anything is written.  Host buffers; returns 0
 * on success or a cudaError_t value (values untouched on failure). */
int catmsm_p1_fft_batch(blst_p1 *const values[], const size_t ns[], const blst_fr *const domains[],
                        const int modes[], size_t count);

/* Forward G1 FFT of an input whose elements [xn, n) are the identity: the
 * C-ABI form of the reference's fft_forward_truncated_prefix<G1Point, Fr,
 * G1CoeffCtx> (blst/fft/ctFft.h:132-150, :384-460, :575-646; a C++ template
 * there, used by the middle product, with no C entry of its own).  All n
 * outputs equal blst_p1_fft_with_domain(values, n, domain, domain_len, false)
 * on the same input; stage s runs only the butterflies of the min(xn, n / 2^s)
 * groups that hold a non-identity input (the reference's plan).  Returns
 * false before writing on: NULL values, an invalid size, domain length or
 * tag (as blst_p1_fft_with_domain), xn == 0 or xn > n, or a non-identity
 * element (z != 0) in [xn, n) (the reference leaves that case unspecified). */
bool catmsm_p1_fft_truncated_prefix(blst_p1 *values, size_t n, size_t xn, const blst_fr *domain,
                                    size_t domain_len);

/* The calling thread's library CUDA stream (cudaStream_t), for event timing. */
void *catmsm_stream(void);

/* Number of kernels this thread launched through the library so far. */
long catmsm_launch_count(void);

/* The window width the GPU MSM uses for n points of scalars of at most 128
 * bits (no GLV split). */
size_t catmsm_msm_window(size_t npoints);

/* The plan of the calling thread's next MSM of n points with nbits-bit
 * scalars: window width, number of windows, and the number of points the
 * pipeline runs over (2n when the GLV split applies: nbits > 128 and the
 * split enabled).  Returns 0, or -1 on invalid arguments. */
int catmsm_msm_plan(size_t npoints, size_t nbits, size_t *window, size_t *windows, size_t *points);

/* The same plan without a context (host arithmetic only, no GPU needed):
 * glv = 1 applies the GLV split as the library does by default.  Also
 * reports the bucket-accumulation chunk length (entries per thread) and the
 * reduction's level-1 fan-in (2, 8 or 16).  Off a GPU the chunk model uses
 * the GB300's 152 SMs x 4 resident blocks.  Returns 0, or -1 on invalid
 * arguments. */
int catmsm_msm_plan_detail(size_t npoints, size_t nbits, int glv, size_t *window, size_t *windows, size_t *points,
                           size_t *chunk, size_t *fan_in);

/* Enables (1) or disables (0) the GLV split for the calling thread's MSMs
 * (on by default; -1 only queries).  Returns the previous setting, or -1
 * without a device context.  Both settings give the same group element for
 * subgroup points, the reference's precondition. */
int catmsm_msm_glv(int enable);
/* Batch-affine accumulation rounds of this thread's MSMs (no reference
 * counterpart): 0 = XYZZ mixed additions only, 1..8 = that many rounds of
 * affine additions behind Montgomery batch inversions before the XYZZ fold,
 * -1 = chosen by size (the default).  Returns the previous setting (-2 if no
 * device context); values outside -1..8 only query. */
int catmsm_msm_affine_rounds(int rounds);
/* The batch-affine rounds this thread's next MSM of npoints nbits-bit scalars
 * would run (the setting above, or the size rule); -1 on invalid input. */
int catmsm_msm_affine_rounds_for(size_t npoints, size_t nbits);

/* Seeded-input support: out[i] = k_i * G (affine, canonical) for n 32-byte
 * little-endian scalars.  Host buffers; returns 0 on success. */
int catmsm_p1_affines_from_scalars(blst_p1_affine *out, const blst_byte *k32, size_t n);
/* Same with device buffers on the library stream. */
int catmsm_p1_affines_from_scalars_device(void *d_out, const void *d_k32, size_t n);

/* Measured integer multiply-add throughput of the current device in
 * tera-IMAD/s: independent 32-bit chains on every SM, the better of the
 * mad.lo.u32 form and the mad.wide.u32 form (one instruction yielding both
 * product halves, counted as two); negative on failure.  _form measures one
 * form only (wide = 0: mad.lo, 1: mad.wide). */
double catmsm_imad_peak(void);
double catmsm_imad_peak_form(int wide);

/* Per-stage CUDA-event timing of this thread's MSM pipeline.  Stages:
 * 0 memset, 1 digits, 2 scan, 3 scatter, 4 accumulate, 5 fixup,
 * 6 reduce (segments + windows + result copy), 7 host fold.  read returns the
 * stage count and fills min(max, count) accumulated milliseconds. */
void catmsm_profile(int enable);
void catmsm_profile_reset(void);
int catmsm_profile_read(double *ms, int max, long *calls);
/* Total bucket entries (nonzero window digits) of the profiled MSM calls. */
double catmsm_profile_entries(void);

/* MSM that allocates nothing -- no counterpart in the reference library.
 * For callers that must not allocate device memory at call time (for example
 * when another framework has reserved nearly all GPU memory in its own pool,
 * or on latency-critical paths where cudaMalloc/cudaFree could synchronise the
 * device).  ret = sum_i k_i * P_i for CONTIGUOUS host arrays: npoints affine
 * points and npoints scalars of ceil(nbits/8) little-endian bytes each.  All
 * device work uses one fixed scratch array (7,167,488 bytes) that every GPU
 * loading the library holds until the process exits; no cudaMalloc, cudaFree,
 * pinned buffer, stream creation or heap allocation happens in the call.
 * Limits: npoints <= CATMSM_NOALLOC_MAX_POINTS and nbits <= 256, else the call
 * returns CATMSM_NOALLOC_TOO_LARGE and writes infinity.  Returns 0 on success
 * (npoints == 0 or nbits == 0 give infinity), CATMSM_NOALLOC_BAD_ARGUMENT for
 * NULL pointers, or a cudaError_t value.  Runs on the per-thread default
 * stream and returns when the result is in *ret.  All calls share the one
 * scratch array, so calls that overlap on the GPU race: serialise them; a call
 * that fails after queueing work waits for that work before it returns.  The
 * first call on a device looks up the array's address there, and with the
 * CUDA runtime's default lazy module loading that is when the device reserves
 * the array: make the first call on each device before another framework
 * claims the GPU's memory and before any stream capture.  Devices 0..63. */
#define CATMSM_NOALLOC_MAX_POINTS 4096
#define CATMSM_NOALLOC_BAD_ARGUMENT (-1)
#define CATMSM_NOALLOC_TOO_LARGE (-2)
int catmsm_p1s_mult_pippenger_noalloc(blst_p1 *ret, const blst_p1_affine *points, size_t npoints,
                                      const blst_byte *scalars, size_t nbits);

/* ---- Batched commitments over a resident basis (no reference counterpart;
 * the nearest reference API is the fixed-base wbits MSM, blst/c_api.cpp:1310-1369).
 * catmsm_basis_create uploads n affine points (host) to the current device
 * and builds fixed-base tables T[w][i] = 2^(c w) P_i (window c: 0 = 11); NULL
 * on failure.  catmsm_basis_msm_batch computes nmsm MSMs in one pass:
 * out[j] = sum_{i < counts[j]} k_{j,i} P_i, where the k_{j,i} are 32-byte
 * little-endian 256-bit scalars, concatenated MSM by MSM; counts[j] <= n.
 * Results are Jacobian blst_p1 (not normalised; z = 0 for infinity), as the
 * reference MSM returns them.  use_graph != 0 replays the batch's device
 * sequence as one CUDA graph launch (captured on first use per batch size).
 * A basis has one stream and one workspace: calls on it from several host
 * threads (batches, set_config, config, autotune) are serialised by the
 * library and must be made with the basis's device current
 * (cudaErrorInvalidDevice otherwise).
 * catmsm_basis_autotune times (window, chunk) candidates on a caller batch,
 * keeps the fastest, and remembers it per (GPU, n, nmsm, points-per-MSM
 * class) in the text file $CATMSM_TUNE_CACHE (default ~/.cache/catmsm_tune.txt);
 * force != 0 re-tunes.  All return 0 or a cudaError_t value. */
void *catmsm_basis_create(const blst_p1_affine *points, size_t n, size_t window);
void catmsm_basis_destroy(void *basis);
int catmsm_basis_config(void *basis, size_t *window, size_t *chunk);
int catmsm_basis_set_config(void *basis, size_t window, size_t chunk);
int catmsm_basis_msm_batch(void *basis, blst_p1 *out, size_t nmsm, const size_t *counts,
                           const blst_byte *scalars, int use_graph);
int catmsm_basis_autotune(void *basis, size_t nmsm, const size_t *counts, const blst_byte *scalars, int force);

/* ---- Serving engine (no reference counterpart): continuous batching of MSM
 * and FFT requests over a resident basis (catmsm_basis_create) on one GPU.
 * `workers` threads each own a stream and a workspace; a free worker takes
 * the oldest queued request and, as one batch, every other queued request of
 * its size class (MSMs: k in the same power-of-four band; FFTs: the same n),
 * up to a point cap, so requests that arrive while other batches run join at
 * the next batch boundary and batches of different workers overlap on the
 * device.  Worker 0 runs on the highest-priority stream and takes the oldest
 * large request (an MSM of >= 2^20 points, an FFT of >= 2^14) first; MSMs of
 * >= 2^18 points and a batch of one MSM run through the plain pipeline over
 * the basis points, smaller batched MSMs over its fixed-base tables.  A batch
 * starts only while the estimated device memory of all in-flight batches
 * stays within hbm_budget_bytes (0 = 64 GiB; a single request above the
 * budget runs alone).
 * submit_msm: MSM over the first k basis points with k 32-byte scalars;
 * submit_fft: blst_p1_fft_with_domain semantics with mode 0 forward, 1 inverse,
 * 2 inverse unscaled, in place on `values`.  Input buffers must stay valid
 * until wait returns.  Both return a ticket (> 0) or -1 on invalid input.
 * wait blocks until the ticket completes, writes the MSM result (Jacobian) to
 * msm_out if not NULL and times_ms[0..1] = queueing and total latency in ms
 * (host steady clock) if not NULL, and returns 0 or a cudaError_t value.  A
 * ticket is waited once: an unknown ticket, or one another wait call already
 * holds or has returned, gives cudaErrorInvalidValue.  destroy runs every
 * queued request to completion and frees the ones never waited; no wait may
 * be in progress when it is called, nor follow it.
 * The basis must not be reconfigured or destroyed while a server uses it. */
void *catmsm_server_create(void *basis, size_t workers, size_t hbm_budget_bytes);
void catmsm_server_destroy(void *server);
int64_t catmsm_server_submit_msm(void *server, const blst_byte *scalars, size_t k);
int64_t catmsm_server_submit_fft(void *server, blst_p1 *values, size_t n, const blst_fr *domain, int mode);
int catmsm_server_wait(void *server, int64_t ticket, blst_p1 *msm_out, double *times_ms);
/* Engine statistics so far: batches run, requests they held, the largest
 * batch, and the most batches that were executing at the same time. */
int catmsm_server_stats(void *server, long *batches, long *batched_requests, long *max_batch,
                        long *max_concurrent);

/* ---- Batched point decoding and validation (no single reference call; each
 * element has exactly the semantics of the reference call cited):
 * catmsm_p1s_uncompress  = blst_p1_uncompress (bindings/blst_scalar.h:623) on
 *                          48-byte element i of in48;
 * catmsm_p1s_deserialize = blst_p1_deserialize (bindings/blst_scalar.h:631) on
 *                          96-byte element i of in96;
 * errs[i] receives the BLST_ERROR value (0 success, 1 bad encoding, 2 not on
 * curve, 3 not in group); out[i] is written only on success.  check_group != 0
 * adds blst_p1_affine_in_g1 to every successful decode (POINT_NOT_IN_GROUP on
 * failure).  catmsm_p1s_affine_in_g1 = blst_p1_affine_in_g1
 * (bindings/blst_scalar.h:507) per point: results[i] = 1 member, 0 not.
 * Host buffers; return 0 or a cudaError_t value. */
int catmsm_p1s_uncompress(blst_p1_affine *out, const blst_byte *in48, size_t n, int *errs, int check_group);
int catmsm_p1s_deserialize(blst_p1_affine *out, const blst_byte *in96, size_t n, int *errs, int check_group);
int catmsm_p1s_affine_in_g1(const blst_p1_affine *points, size_t n, int *results);

/* Field self-check: out[i] = a[i] * b[i] * R^-1 mod p (canonical), host
 * buffers of n blst_fp with inputs below 2p; a == b (the same pointer)
 * selects the dedicated squaring.  Returns 0 on success. */
int catmsm_fp_mul(blst_fp *out, const blst_fp *a, const blst_fp *b, size_t n);
/* Field self-check of the batch-affine rounds' inversion: out[i] = a[i]^-1
 * in Montgomery form (canonical; zero maps to zero), host buffers of n
 * blst_fp with inputs below 2p.  Returns 0 on success. */
int catmsm_fp_inv(blst_fp *out, const blst_fp *a, size_t n);
/* Self-checks of the host arithmetic that folds the MSM window sums (no GPU
 * needed): out[i] = a[i]^-1, a[i]^2 and a[i] b[i], Montgomery form, canonical
 * outputs, inputs below 2^384 (reduced first).  Return 0. */
int catmsm_host_fp_inv(blst_fp *out, const blst_fp *a, size_t n);
int catmsm_host_fp_sqr(blst_fp *out, const blst_fp *a, size_t n);
int catmsm_host_fp_mul(blst_fp *out, const blst_fp *a, const blst_fp *b, size_t n);

#ifdef __cplusplus
}
#endif
#endif
