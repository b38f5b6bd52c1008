/*
 * Oracle Pippenger MSM (test infrastructure only; see oracle.h).
 *
 * Restates the reference's plain C-ABI MSM:
 *   blst_p1s_mult_pippenger            c_api.cpp:1382-1418 (argument checks,
 *                                      one-point fallback, null scratch)
 *   blst_p1s_mult_pippenger_scratch_sizeof  c_api.cpp:1371 ->
 *                                      multi_scalar.h:459-469
 *   pippenger_window_size              multi_scalar.h:329-348
 *   WindowExtract / get_wval_limb / booth_encode
 *                                      multi_scalar.h:350-404, ec_mult.h:63-142
 *   points_tile_pippenger              multi_scalar.cpp:806-864 (descriptor
 *                                      walk: a later NULL entry means
 *                                      contiguous continuation)
 *   point_integrate_buckets            multi_scalar.cpp:730-751
 *   msm_mult_pippenger                 multi_scalar.cpp:892-923 (top window
 *                                      first, ret = 2^c (ret + tile))
 * Buckets live in the caller's scratch exactly as in the reference (XYZZ,
 * 192 bytes each, 2^(c-1) of them).
 */
#include "oracle.h"
#include <string.h>

#define MAX_WINDOW 24

size_t oracle_pippenger_window_size(size_t npoints)
{
    size_t wbits;
    for (wbits = 0; npoints >>= 1; wbits++) {}
    if (wbits > 12) wbits -= 3;
    else if (wbits > 8) wbits -= 2;
    else if (wbits > 4) wbits -= 1;
    else return wbits ? 2 : 1;
    return wbits < MAX_WINDOW ? wbits : MAX_WINDOW;
}

size_t oracle_p1s_mult_pippenger_scratch_sizeof(size_t npoints)
{
    if (npoints == 0) return 0;
    return sizeof(op1xyzz) << (oracle_pippenger_window_size(npoints) - 1);
}

static uint64_t get_wval_limb(const uint8_t *d, size_t off, size_t bits)
{
    /* bits <= 25: gather the covering bytes (never past the last covered byte) */
    size_t first = off / 8, last = (off + bits - 1) / 8;
    uint64_t ret = 0;
    for (size_t i = first; i <= last; i++) ret |= (uint64_t)d[i] << (8 * (i - first));
    return ret >> (off % 8);
}

typedef struct {
    size_t missing_overlap, extract_begin, extract_size, encode_size;
    uint64_t mask;
} wextract;

static void wextract_init(wextract *we, size_t bit0, size_t window, size_t nbits)
{
    size_t wb = bit0;
    size_t we_end = wb + window < nbits ? wb + window : nbits;
    we->missing_overlap = wb == 0 ? 1 : 0;
    we->extract_begin = wb > 0 ? wb - 1 : 0;
    we->extract_size = we_end - we->extract_begin;
    we->mask = ((uint64_t)1 << we->extract_size) - 1;
    size_t enc = nbits - wb + 1;
    we->encode_size = enc < window ? enc : window;
}

static uint64_t booth_encode(uint64_t wval, size_t w)
{
    uint64_t sign = wval >> w;
    uint64_t mask = (uint64_t)0 - sign;
    uint64_t val = (wval + 1) >> 1;
    return (val ^ mask) - mask;
}

static uint64_t wextract_digit(const wextract *we, const uint8_t *scalar)
{
    uint64_t wval = (get_wval_limb(scalar, we->extract_begin, we->extract_size) & we->mask)
                    << we->missing_overlap;
    return booth_encode(wval, we->encode_size);
}

static void point_bucket(op1xyzz *buckets, uint64_t booth_idx, size_t wbits, const op1a *p)
{
    int sign = (int)((booth_idx >> wbits) & 1);
    booth_idx &= ((uint64_t)1 << wbits) - 1;
    if (booth_idx--) oxyzz_madd(&buckets[booth_idx], &buckets[booth_idx], p, sign);
}

static void integrate_buckets(op1 *out, op1xyzz *buckets, size_t wbits)
{
    size_t n = (size_t)1 << wbits;
    op1xyzz acc = buckets[--n], ret = buckets[n];
    memset(&buckets[n], 0, sizeof(op1xyzz));
    while (n--) {
        oxyzz_add(&acc, &acc, &buckets[n]);
        oxyzz_add(&ret, &ret, &acc);
        memset(&buckets[n], 0, sizeof(op1xyzz));
    }
    oxyzz_to_jacobian(out, &ret);
}

static void tile_pippenger(op1 *ret, const op1a *const points[], size_t npoints,
                           const uint8_t *const scalars[], size_t nbits,
                           op1xyzz *buckets, size_t window_idx, size_t window)
{
    wextract we;
    wextract_init(&we, window_idx * window, window, nbits);
    size_t nbytes = (nbits + 7) / 8;
    const uint8_t *scalar = *scalars++;
    const op1a *point = *points++;
    for (size_t i = 0; i < npoints; i++) {
        if (i) {
            scalar = *scalars ? *scalars++ : scalar + nbytes;
            point = *points ? *points++ : point + 1;
        }
        point_bucket(buckets, wextract_digit(&we, scalar), we.encode_size, point);
    }
    integrate_buckets(ret, buckets, we.encode_size - 1);
}

static void msm_pippenger(op1 *ret, const op1a *const points[], size_t npoints,
                          const uint8_t *const scalars[], size_t nbits,
                          op1xyzz *buckets, size_t window)
{
    window = window ? window : oracle_pippenger_window_size(npoints);
    memset(buckets, 0, sizeof(op1xyzz) << (window - 1));
    memset(ret, 0, sizeof(*ret));
    size_t num_windows = 1 + nbits / window;
    for (size_t w = num_windows - 1; w < num_windows; --w) {
        op1 tile;
        tile_pippenger(&tile, points, npoints, scalars, nbits, buckets, w, window);
        op1_dadd(ret, ret, &tile);
        for (size_t i = 0; i < (w ? window : 0); i++) op1_double(ret, ret);
    }
}

static int valid_heads(const op1a *const points[], const uint8_t *const scalars[], size_t n)
{
    return n == 0 || (points && scalars && points[0] && scalars[0]);
}

static void mult_pippenger_common(op1 *ret, const op1a *const points[], size_t npoints,
                                  const uint8_t *const scalars[], size_t nbits,
                                  uint64_t *scratch, size_t window, int explicit_window)
{
    if (npoints == 0 || nbits == 0) { memset(ret, 0, sizeof(*ret)); return; }
    if (nbits > 256 || (explicit_window && (window < 1 || window > MAX_WINDOW)) ||
        !valid_heads(points, scalars, npoints)) {
        memset(ret, 0, sizeof(*ret));
        return;
    }
    if (npoints == 1) {
        op1 p;
        op1_from_affine(&p, points[0]);
        op1_mult_vartime(ret, &p, scalars[0], nbits);
        return;
    }
    if (scratch == NULL) { memset(ret, 0, sizeof(*ret)); return; }
    msm_pippenger(ret, points, npoints, scalars, nbits, (op1xyzz *)scratch, window);
}

/* c_api.cpp:1546-1583 (explicit window in [1, 24]) */
void oracle_p1s_mult_pippenger_window(op1 *ret, const op1a *const points[], size_t npoints,
                                      const uint8_t *const scalars[], size_t nbits,
                                      uint64_t *scratch, size_t window)
{
    mult_pippenger_common(ret, points, npoints, scalars, nbits, scratch, window, 1);
}

/* c_api.cpp:1382-1418 */
void oracle_p1s_mult_pippenger(op1 *ret, const op1a *const points[], size_t npoints,
                               const uint8_t *const scalars[], size_t nbits,
                               uint64_t *scratch)
{
    mult_pippenger_common(ret, points, npoints, scalars, nbits, scratch, 0, 0);
}

/* blst_p1s_tile_pippenger (c_api.cpp:1585-1612 -> :883-936): one window's
 * bucket fill + running-sum reduction starting at bit bit0.  Used as the
 * bounded CPU-baseline sample: a full MSM is D such tiles plus a short fold. */
void oracle_p1s_tile_pippenger(op1 *ret, const op1a *const points[], size_t npoints,
                               const uint8_t *const scalars[], size_t nbits,
                               uint64_t *scratch, size_t bit0, size_t window)
{
    memset(ret, 0, sizeof(*ret));
    if (npoints == 0 || !valid_heads(points, scalars, npoints) || scratch == NULL ||
        window < 1 || window > MAX_WINDOW || nbits == 0 || nbits > 256 || bit0 >= nbits)
        return;
    wextract we;
    wextract_init(&we, bit0, window, nbits);
    op1xyzz *buckets = (op1xyzz *)scratch;
    memset(buckets, 0, sizeof(op1xyzz) << (we.encode_size - 1));
    size_t nbytes = (nbits + 7) / 8;
    const uint8_t *scalar = *scalars++;
    const op1a *point = *points++;
    for (size_t i = 0; i < npoints; i++) {
        if (i) {
            scalar = *scalars ? *scalars++ : scalar + nbytes;
            point = *points ? *points++ : point + 1;
        }
        point_bucket(buckets, wextract_digit(&we, scalar), we.encode_size, point);
    }
    integrate_buckets(ret, buckets, we.encode_size - 1);
}

void oracle_p1s_mult_naive(op1 *ret, const op1a *points, size_t npoints,
                           const uint8_t *scalars, size_t nbits)
{
    size_t nbytes = (nbits + 7) / 8;
    memset(ret, 0, sizeof(*ret));
    for (size_t i = 0; i < npoints; i++) {
        op1 p, t;
        op1_from_affine(&p, &points[i]);
        op1_mult_vartime(&t, &p, scalars + i * nbytes, nbits);
        op1_dadd(ret, ret, &t);
    }
}
