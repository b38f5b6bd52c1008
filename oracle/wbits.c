/*
 * Oracle fixed-table (wbits) MSM (test infrastructure only; see oracle.h).
 *
 * Restates:
 *   blst_p1s_mult_wbits_precompute_sizeof  c_api.cpp:1310-1316 ->
 *                                  multi_scalar.h:245-255 (96 n 2^(w-1),
 *                                  0 for w outside [2, 14] or on overflow)
 *   blst_p1s_mult_wbits_precompute  c_api.cpp:1318-1330 ->
 *                                  multi_scalar.cpp:481-565 (row i =
 *                                  [P_i, 2 P_i, ..., 2^(w-1) P_i], affine;
 *                                  descriptor walk as for the MSM)
 *   blst_p1s_mult_wbits_scratch_sizeof  c_api.cpp:1332-1335 ->
 *                                  multi_scalar.h:310-315 (144 min(n, 8192))
 *   blst_p1s_mult_wbits            c_api.cpp:1337-1369 ->
 *                                  multi_scalar.cpp:600-720: the top window of
 *                                  nbits % w bits first, then full w-bit
 *                                  windows, Booth digits with the overlap bit
 *                                  below each window; a digit d selects row
 *                                  entry |d| - 1, negated for d < 0; w
 *                                  doublings between windows.
 * The reference batches the gathered entries in affine form before adding
 * them; the sum is the same group element, so this restatement adds them one
 * by one.
 */
#include "oracle.h"
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

static int valid_wbits(size_t w) { return w >= 2 && w <= 14; }

size_t oracle_p1s_mult_wbits_precompute_sizeof(size_t wbits, size_t npoints)
{
    if (!valid_wbits(wbits)) return 0;
    if (npoints != 0 && sizeof(op1a) > SIZE_MAX / npoints) return 0;
    size_t b = sizeof(op1a) * npoints;
    if (b > (SIZE_MAX >> (wbits - 1))) return 0;
    return b << (wbits - 1);
}

size_t oracle_p1s_mult_wbits_scratch_sizeof(size_t npoints)
{
    return 144 * (npoints < 8192 ? npoints : 8192);
}

void oracle_p1s_mult_wbits_precompute(op1a *table, size_t wbits, const op1a *const points[], size_t npoints)
{
    if (!valid_wbits(wbits) || npoints == 0 || !table || !points || !points[0]) return;
    if (npoints > (SIZE_MAX >> (wbits - 1))) return;
    size_t m = (size_t)1 << (wbits - 1);
    /* read every point first: packed input may occupy the table's tail */
    op1a *pts = (op1a *)malloc(npoints * sizeof(op1a));
    if (!pts) return;
    const op1a *point = NULL;
    for (size_t i = 0; i < npoints; i++) {
        point = (i == 0 || *points) ? *points++ : point + 1;
        pts[i] = *point;
    }
    for (size_t i = 0; i < npoints; i++) {
        op1 p, acc;
        op1_from_affine(&p, &pts[i]);
        acc = p;
        for (size_t j = 0; j < m; j++) {
            if (j) op1_dadd(&acc, &acc, &p);
            op1_to_affine(&table[i * m + j], &acc);
        }
    }
    free(pts);
}

/* bits [off, off + bits) of a little-endian scalar, bits <= 15 */
static uint64_t wval(const uint8_t *s, size_t off, size_t bits)
{
    size_t first = off / 8, last = (off + bits - 1) / 8;
    uint64_t r = 0;
    for (size_t i = first; i <= last; i++) r |= (uint64_t)s[i] << (8 * (i - first));
    return r >> (off % 8);
}

/* |digit| and sign of a (w+1)-bit window value with its overlap bit as bit 0 */
static void booth(uint64_t v, size_t w, size_t *mag, int *neg)
{
    int sign = (int)((v >> w) & 1);
    uint64_t d = (v + 1) >> 1;
    if (sign) d = ((uint64_t)1 << w) - d;
    *mag = (size_t)d;
    *neg = sign;
}

static void add_entry(op1 *ret, const op1a *row, size_t mag, int neg)
{
    if (mag == 0) return;
    op1 t;
    op1_from_affine(&t, &row[mag - 1]);
    if (neg) op1_neg(&t, &t);
    op1_dadd(ret, ret, &t);
}

void oracle_p1s_mult_wbits(op1 *ret, const op1a *table, size_t wbits, size_t npoints,
                           const uint8_t *const scalars[], size_t nbits, uint64_t *scratch)
{
    memset(ret, 0, sizeof(*ret));
    if (npoints == 0 || nbits == 0) return;
    if (nbits > 256 || !valid_wbits(wbits) || !table || !scalars || !scalars[0] || !scratch) return;
    if (npoints > (SIZE_MAX >> (wbits - 1))) return;
    size_t m = (size_t)1 << (wbits - 1), nbytes = (nbits + 7) / 8;
    const uint8_t **sc = (const uint8_t **)malloc(npoints * sizeof(*sc));
    if (!sc) return;
    const uint8_t *const *ss = scalars;
    const uint8_t *s = NULL;
    for (size_t i = 0; i < npoints; i++) {
        s = (i == 0 || *ss) ? *ss++ : s + nbytes;
        sc[i] = s;
    }
    size_t top = nbits % wbits;          /* may be zero */
    size_t rem = nbits - top;             /* bits below the current window */
    size_t width = top;                   /* current window width */
    for (;;) {
        uint64_t mask = ((uint64_t)1 << (width + 1)) - 1;
        for (size_t i = 0; i < npoints; i++) {
            uint64_t v;
            if (rem > 0) v = wval(sc[i], rem - 1, width + 1) & mask;
            else v = (wval(sc[i], 0, width) << 1) & mask;
            size_t mag;
            int neg;
            booth(v, wbits, &mag, &neg);
            add_entry(ret, table + i * m, mag, neg);
        }
        if (rem == 0) break;
        for (size_t j = 0; j < wbits; j++) op1_double(ret, ret);
        width = wbits;
        rem -= wbits;
    }
    free(sc);
}
