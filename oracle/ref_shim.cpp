/*
 * Test infrastructure only (linked into oracle/_ref/libblst_ref.so, the
 * reference compiled from its own sources; never into the product library).
 *
 * The reference's truncated-prefix forward G1 FFT is a C++ template
 * (blst/fft/ctFft.h:132-150, :384-460, :575-646) with no C entry of its own.
 * This instantiates it the way blst/fft_c_api.cpp:66-103 instantiates the full
 * transform (group = blst_p1, coefficient context GroupFftCoeffCtx) so that
 * tests/golden/make_golden.py can record its outputs as golden vectors.
 * roots: the first n entries of a blst_fr_fft_domain_init domain.
 */
#include "bindings/blst_fft.h"
#include "blst/fft/context.h"
#include "blst/fft/ctFft.h"

#include <span>

extern "C" bool refshim_p1_fft_truncated_prefix(blst_p1* values, size_t n, size_t xn, const blst_fr* roots)
{
    if (values == nullptr || roots == nullptr) return false;
    try {
        fft_forward_truncated_prefix<blst_p1, blst::Fr, blst::detail::GroupFftCoeffCtx<blst_p1>>(
            std::span<blst_p1>(values, n), std::span<const blst::Fr>(roots, n), xn);
        return true;
    } catch (...) {
        return false;
    }
}
