"""The unrolled squaring in csrc/field.cuh is the output of its generator
(temp-cat-blst_gb300/gen/gen_fp_sqr.py): regenerate and compare the text.
No GPU; the arithmetic itself is checked on the GPU by test_gpu_msm.py
(test_fp_sqr_matches_bigint)."""
import importlib.util
import os

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "temp-cat-blst_gb300")


def _gen():
    spec = importlib.util.spec_from_file_location("gen_fp_sqr", os.path.join(PKG, "gen", "gen_fp_sqr.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def test_fp_sqr_impl_is_generated():
    text = open(os.path.join(PKG, "csrc", "field.cuh")).read()
    gen = _gen().generate()
    assert gen.startswith("__device__ __forceinline__ void fp_sqr_impl(")
    assert gen in text


def test_fp_sqr_schedule_counts():
    """Step i multiplies 12 - i limbs of V_i: 78 limb products (156 IMAD with
    high words) against 144 for a general product."""
    g = _gen()
    gen = g.generate()
    products = gen.count("* bi;") + sum(2 * len([j for j in range(i, 12) if j % 2 == 0])
                                        for i in range(1, 12)) // 2
    assert products == sum(12 - i for i in range(12)) == 78
    assert g.operand(3, 3) == "a.v[3]" and g.operand(3, 4) == "(a.v[4] << 1)" and g.operand(3, 7) == "d[7]"
