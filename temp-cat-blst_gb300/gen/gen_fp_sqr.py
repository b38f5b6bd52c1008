"""Generator of fp_sqr_impl (csrc/field.cuh): the unrolled 12-limb Montgomery
squaring.

Step i of the CIOS schedule adds a_i * V_i with
    V_i = a_i 2^(32 i) + 2 sum_{j > i} a_j 2^(32 j),
whose limb j is a_i (j = i), a_{i+1} << 1 (j = i + 1; the bit shifted out
goes to the next limb) or (2a)_j = d[j] (j >= i + 2), and 0 below i.  As in
fp_mul_impl, the products of even limbs go to the E accumulator (low word at
e[j], high at e[j + 1]) and those of odd limbs to O (at o[j - 1], o[j]):
step 0 assigns E, later steps add into E = t with one carry chain, and O is
assigned afresh every step.  The Montgomery step and the merge
t = (E + O 2^32) / 2^32 are fp_mul_impl's, unchanged.

Run `python gen_fp_sqr.py` to print the function; the CPU test
tests/test_field_gen.py checks that field.cuh holds exactly this text.
"""

MUL_HEAD = ("mad.lo.cc.u32  ", "madc.hi.cc.u32 ")
MADC = ("madc.lo.cc.u32 ", "madc.hi.cc.u32 ")


def operand(i: int, j: int) -> str:
    """Limb j of V_i (j >= i)."""
    if j == i:
        return "a.v[%d]" % j
    if j == i + 1:
        return "(a.v[%d] << 1)" % j
    return "d[%d]" % j


def e_chain(i: int, even: list) -> list:
    """E += bi * (the even limbs of V_i), one carry chain into e[j0 .. 12]."""
    m = len(even)
    src = ["%%%d" % (2 * m + 1 + k) for k in range(m)]
    b = "%%%d" % (3 * m + 1)
    body = []
    for k in range(m):
        lo, hi = (MUL_HEAD if k == 0 else MADC)
        body.append('%s%%%d, %s, %s, %%%d;\\n\\t' % (lo, 2 * k, src[k], b, 2 * k))
        body.append('%s%%%d, %s, %s, %%%d;\\n\\t' % (hi, 2 * k + 1, src[k], b, 2 * k + 1))
    body.append('addc.u32       %%%d, 0, 0;' % (2 * m))
    out = ['"+r"(e[%d])' % k for k in range(even[0], 12)] + ['"=r"(e[12])']
    ins = ['"r"(%s)' % operand(i, j) for j in even] + ['"r"(bi)']
    lines = ['        asm("%s"' % body[0]]
    lines += ['            "%s"' % x for x in body[1:]]
    lines.append('            : %s' % ", ".join(out))
    lines.append('            : %s);' % ", ".join(ins))
    return lines


# The Montgomery step (E += m p_even, O += m p_odd) and the merge, as in fp_mul_impl.
MONT = r'''        const uint32_t m = e[0] * CATMSM_N0;
        asm("mad.lo.cc.u32  %0, %13, %14, %0;\n\t"
            "madc.hi.cc.u32 %1, %13, %14, %1;\n\t"
            "madc.lo.cc.u32 %2, %13, %15, %2;\n\t"
            "madc.hi.cc.u32 %3, %13, %15, %3;\n\t"
            "madc.lo.cc.u32 %4, %13, %16, %4;\n\t"
            "madc.hi.cc.u32 %5, %13, %16, %5;\n\t"
            "madc.lo.cc.u32 %6, %13, %17, %6;\n\t"
            "madc.hi.cc.u32 %7, %13, %17, %7;\n\t"
            "madc.lo.cc.u32 %8, %13, %18, %8;\n\t"
            "madc.hi.cc.u32 %9, %13, %18, %9;\n\t"
            "madc.lo.cc.u32 %10, %13, %19, %10;\n\t"
            "madc.hi.cc.u32 %11, %13, %19, %11;\n\t"
            "addc.u32       %12, %12, 0;"
            : "+r"(e[0]), "+r"(e[1]), "+r"(e[2]), "+r"(e[3]), "+r"(e[4]), "+r"(e[5]),
              "+r"(e[6]), "+r"(e[7]), "+r"(e[8]), "+r"(e[9]), "+r"(e[10]), "+r"(e[11]),
              "+r"(e[12])
            : "r"(m), "n"(CATMSM_P0), "n"(CATMSM_P2), "n"(CATMSM_P4), "n"(CATMSM_P6),
              "n"(CATMSM_P8), "n"(CATMSM_P10));
        asm("mad.lo.cc.u32  %0, %13, %14, %0;\n\t"
            "madc.hi.cc.u32 %1, %13, %14, %1;\n\t"
            "madc.lo.cc.u32 %2, %13, %15, %2;\n\t"
            "madc.hi.cc.u32 %3, %13, %15, %3;\n\t"
            "madc.lo.cc.u32 %4, %13, %16, %4;\n\t"
            "madc.hi.cc.u32 %5, %13, %16, %5;\n\t"
            "madc.lo.cc.u32 %6, %13, %17, %6;\n\t"
            "madc.hi.cc.u32 %7, %13, %17, %7;\n\t"
            "madc.lo.cc.u32 %8, %13, %18, %8;\n\t"
            "madc.hi.cc.u32 %9, %13, %18, %9;\n\t"
            "madc.lo.cc.u32 %10, %13, %19, %10;\n\t"
            "madc.hi.cc.u32 %11, %13, %19, %11;\n\t"
            "addc.u32       %12, 0, 0;"
            : "+r"(o[0]), "+r"(o[1]), "+r"(o[2]), "+r"(o[3]), "+r"(o[4]), "+r"(o[5]),
              "+r"(o[6]), "+r"(o[7]), "+r"(o[8]), "+r"(o[9]), "+r"(o[10]), "+r"(o[11]),
              "=r"(o[12])
            : "r"(m), "n"(CATMSM_P1), "n"(CATMSM_P3), "n"(CATMSM_P5), "n"(CATMSM_P7),
              "n"(CATMSM_P9), "n"(CATMSM_P11));
        asm("add.cc.u32  %0, %0, %12;\n\t"
            "addc.cc.u32 %1, %1, %13;\n\t"
            "addc.cc.u32 %2, %2, %14;\n\t"
            "addc.cc.u32 %3, %3, %15;\n\t"
            "addc.cc.u32 %4, %4, %16;\n\t"
            "addc.cc.u32 %5, %5, %17;\n\t"
            "addc.cc.u32 %6, %6, %18;\n\t"
            "addc.cc.u32 %7, %7, %19;\n\t"
            "addc.cc.u32 %8, %8, %20;\n\t"
            "addc.cc.u32 %9, %9, %21;\n\t"
            "addc.cc.u32 %10, %10, %22;\n\t"
            "addc.u32    %11, %11, %23;"
            : "+r"(o[0]), "+r"(o[1]), "+r"(o[2]), "+r"(o[3]), "+r"(o[4]), "+r"(o[5]),
              "+r"(o[6]), "+r"(o[7]), "+r"(o[8]), "+r"(o[9]), "+r"(o[10]), "+r"(o[11])
            : "r"(e[1]), "r"(e[2]), "r"(e[3]), "r"(e[4]), "r"(e[5]), "r"(e[6]),
              "r"(e[7]), "r"(e[8]), "r"(e[9]), "r"(e[10]), "r"(e[11]), "r"(e[12]));
#pragma unroll
        for (int k = 0; k < 12; k++) t[k] = o[k];'''


def generate() -> str:
    L = ["__device__ __forceinline__ void fp_sqr_impl(fp& r, const fp& a)",
         "{",
         "    uint32_t t[12], e[13], o[13], d[12];",
         "#pragma unroll",
         "    for (int j = 1; j < 12; j++) d[j] = __funnelshift_l(a.v[j - 1], a.v[j], 1);   // (2a)_j"]
    for i in range(12):
        even = [j for j in range(i, 12) if j % 2 == 0]
        odd = [j for j in range(i, 12) if j % 2 == 1]
        L.append("    {   // step %d" % i)
        L.append("        const uint32_t bi = a.v[%d];" % i)
        L.append("#pragma unroll")
        if i == 0:
            L.append("        for (int k = 0; k < 13; k++) e[k] = 0;")
            for j in even:
                L.append("        e[%d] = %s * bi;" % (j, operand(i, j)))
                L.append("        e[%d] = __umulhi(%s, bi);" % (j + 1, operand(i, j)))
        else:
            L.append("        for (int k = 0; k < 12; k++) e[k] = t[k];")
            if even:
                L += e_chain(i, even)
            else:
                L.append("        e[12] = 0;")
        L.append("#pragma unroll")
        L.append("        for (int k = 0; k < 13; k++) o[k] = 0;")
        for j in odd:
            L.append("        o[%d] = %s * bi;" % (j - 1, operand(i, j)))
            L.append("        o[%d] = __umulhi(%s, bi);" % (j, operand(i, j)))
        L += MONT.split("\n")
        L.append("    }")
    L += ["#pragma unroll", "    for (int k = 0; k < 12; k++) r.v[k] = t[k];", "}"]
    return "\n".join(L) + "\n"


if __name__ == "__main__":
    print(generate(), end="")
