"""CPU check: the C-ABI library builds for sm_103a, loads, and exports every
function declared in include/*.h (no GPU call is made)."""
import ctypes as C
import glob
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared_functions():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        src = open(h).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        for m in re.finditer(r"^[A-Za-z_][\w \*]*?\b([a-z_][a-z0-9_]*)\s*\(", src, flags=re.M):
            name = m.group(1)
            if name not in ("defined", "if", "sizeof"):
                names.add(name)
    return names


def test_header_declares_drop_in_entry_points():
    names = _declared_functions()
    for must in ("blst_p1s_mult_pippenger", "blst_p1s_mult_pippenger_scratch_sizeof",
                 "blst_p1_fft", "blst_p1_fft_with_domain", "blst_p1_ifft_unscaled_with_domain",
                 "blst_fr_fft_domain_len", "blst_fr_fft_domain_init"):
        assert must in names


def test_library_exports_every_declared_symbol(gpu_binding):
    gpu_binding.load()                       # builds with nvcc if needed; raises on failure
    lib = C.CDLL(gpu_binding.LIB_PATH)
    missing = [n for n in sorted(_declared_functions()) if not hasattr(lib, n)]
    assert not missing, missing


def test_scratch_sizeof_matches_reference_contract(gpu_binding, oracle):
    # pure host functions: no device call
    for n in (0, 1, 2, 5, 17, 256, 4096, 1 << 16, 1 << 20, 1 << 22):
        assert gpu_binding.scratch_sizeof(n) == oracle.scratch_sizeof(n), n
    assert gpu_binding.scratch_sizeof(4096) == 98304
    assert gpu_binding.scratch_sizeof(1 << 16) == 786432
    for w in (0, 1, 5, 24, 25):
        exp = 0 if w < 1 or w > 24 else 192 << (w - 1)
        assert gpu_binding.window_scratch_sizeof(w) == exp
    for n in (0, 3, 6, 1 << 31):
        assert gpu_binding.fr_fft_domain_len(n) == 0
    for k in (0, 1, 10, 30):
        assert gpu_binding.fr_fft_domain_len(1 << k) == (1 << k) + 2


def test_wbits_sizes_match_reference_contract(gpu_binding, oracle):
    # pure host functions: no device call; values probed from the reference
    for w in (0, 1, 2, 3, 8, 14, 15, 16, 64):
        for n in (0, 1, 10, 4096, 1 << 40, 1 << 60):
            assert gpu_binding.p1s_mult_wbits_precompute_sizeof(w, n) == oracle.wbits_table_sizeof(w, n), (w, n)
    assert gpu_binding.p1s_mult_wbits_precompute_sizeof(2, 10) == 1920
    assert gpu_binding.p1s_mult_wbits_precompute_sizeof(14, 10) == 96 * 10 * 8192
    assert gpu_binding.p1s_mult_wbits_precompute_sizeof(15, 10) == 0
    for n in (0, 1, 4096, 8191, 8192, 8193, 1 << 20):
        assert gpu_binding.p1s_mult_wbits_scratch_sizeof(n) == oracle.wbits_scratch_sizeof(n) == 144 * min(n, 8192)


def test_fr_msm_variant_sizes_match_reference(gpu_binding, golden):
    # pure host functions: no device call; values recorded from the reference
    g = golden["msm_fr_variants"]
    for n, exp in g["mult_fr_scratch"]:
        assert gpu_binding.p1s_mult_fr_scratch_sizeof(n) == exp, n
    for n, w, b, exp in g["batch_affine_scratch"]:
        assert gpu_binding.p1s_mult_batch_affine_fr_scratch_sizeof(n, w, b) == exp, (n, w, b)


def test_msm_plan_heuristics(gpu_binding):
    """Host arithmetic only: the window model, the bucket-accumulation chunk
    length (partial-wave model below ~one wave, whole waves above) and the
    reduction's level-1 fan-in, pinned at the sizes they were measured and
    tuned at on a GB300 (152 SMs x 4 resident blocks).  A change here changes
    the GPU schedule and must be re-measured."""
    # n: (window, windows, pipeline points, chunk, level-1 fan-in), GLV on
    expected = {
        1 << 10: (8, 16, 1 << 11, 4, 2),
        1 << 12: (8, 16, 1 << 13, 7, 2),
        1 << 14: (10, 13, 1 << 15, 11, 2),
        1 << 16: (13, 10, 1 << 17, 34, 2),
        1 << 17: (13, 10, 1 << 18, 45, 2),
        1 << 18: (16, 8, 1 << 19, 54, 8),
        1 << 20: (16, 8, 1 << 21, 72, 8),
        1 << 22: (19, 7, 1 << 23, 84, 16),
    }
    for n, exp in expected.items():
        assert gpu_binding.msm_plan_detail(n) == exp, n
    # no GLV split: 255-bit windows over n points; 64-bit scalars skip the split
    assert gpu_binding.msm_plan_detail(1 << 20, 255, 0)[:3] == (16, 16, 1 << 20)
    assert gpu_binding.msm_plan_detail(1 << 16, 64)[:3] == (12, 6, 1 << 16)


def test_fft_truncated_prefix_rejects_on_the_host(gpu_binding, oracle):
    """catmsm_p1_fft_truncated_prefix checks its arguments on the host before
    any device work: a bad size, domain length or tag, xn = 0 or xn > n, or a
    non-identity element past xn returns false with the values untouched."""
    n = 16
    d = oracle.domain(n)
    jac = bytearray(oracle.jacobian_randomize(7, n, oracle.gen_points(7, n)))
    jac[144 * 6:] = bytes(144 * (n - 6))
    jac = bytes(jac)
    bad_tag = bytearray(d)
    bad_tag[-32] ^= 1
    for args in ((jac, n, 0, d, n + 2), (jac, n, n + 1, d, n + 2), (jac, n, 6, d, n + 1),
                 (jac, n, 6, bytes(bad_tag), n + 2), (jac, 12, 6, d, 14), (jac, n, 5, d, n + 2)):
        ok, out = gpu_binding.p1_fft_truncated_prefix(*args)
        assert not ok and out == jac



def test_inversion_correction_tables():
    """fpinv.cuh's KINV_T1[a] = R^3 2^(-32a) mod p and KINV_T2[b] = R 2^(-b)
    mod p (R = 2^384), recomputed with Python integers."""
    import re
    P = 0x1a0111ea397fe69a4b1ba7b6434bacd764774b84f38512bf6730d2a0f6b0f6241eabfffeb153ffffb9feffffffffaaab
    R = (1 << 384) % P
    src = open(os.path.join(ROOT, "temp-cat-blst_gb300", "csrc", "fpinv.cuh")).read()

    def table(name):
        body = src[src.index(name + "["):]          # the declaration, not a comment's mention
        body = body[body.index("= {") + 3:body.index("};")]
        rows = re.findall(r"\{([^}]*)\}", body)
        return [sum(int(w.strip().rstrip("u"), 16) << (32 * i) for i, w in enumerate(r.split(",")) if w.strip())
                for r in rows]
    t1, t2 = table("uint32_t KINV_T1"), table("uint32_t KINV_T2")
    assert len(t1) == 25 and len(t2) == 32
    assert all(t1[a] == R ** 3 * pow(2, -32 * a, P) % P for a in range(25))
    assert all(t2[b] == R * pow(2, -b, P) % P for b in range(32))


def test_host_fold_arithmetic(gpu_binding):
    """The host arithmetic that folds the MSM window sums and normalises the
    result (no GPU involved): the multiplication, the squaring and the
    variable-time inversion against Python integers, including 0, 1, p - 1, R
    and non-canonical inputs in [p, 2^384)."""
    import random
    P = 0x1a0111ea397fe69a4b1ba7b6434bacd764774b84f38512bf6730d2a0f6b0f6241eabfffeb153ffffb9feffffffffaaab
    RM = (1 << 384) % P
    lib = C.CDLL(gpu_binding.LIB_PATH)
    rnd = random.Random(21)
    vals = [0, 1, 2, P - 1, P, P + 1, 2 * P - 1, RM, (1 << 381) - 1, (1 << 384) - 1, 1 << 64, (1 << 64) - 1]
    vals += [rnd.randrange(1 << 384) for _ in range(3000)]
    vals += [rnd.randrange(1 << rnd.randrange(1, 381)) for _ in range(1000)]
    n = len(vals)
    buf = (C.c_char * (48 * n)).from_buffer(bytearray(b"".join(v.to_bytes(48, "little") for v in vals)))
    inv_out = (C.c_char * (48 * n))()
    sqr_out = (C.c_char * (48 * n))()
    assert lib.catmsm_host_fp_inv(inv_out, buf, C.c_size_t(n)) == 0
    assert lib.catmsm_host_fp_sqr(sqr_out, buf, C.c_size_t(n)) == 0
    others = vals[1:] + vals[:1]                 # b[i] = a[i + 1]: every edge value meets others
    buf_b = (C.c_char * (48 * n)).from_buffer(bytearray(b"".join(v.to_bytes(48, "little") for v in others)))
    mul_out = (C.c_char * (48 * n))()
    assert lib.catmsm_host_fp_mul(mul_out, buf, buf_b, C.c_size_t(n)) == 0
    rinv = pow(RM, -1, P)
    for i, v in enumerate(vals):
        a = v % P * rinv % P                    # the field element v represents
        exp_inv = 0 if a == 0 else pow(a, -1, P) * RM % P
        assert int.from_bytes(bytes(inv_out[48 * i:48 * i + 48]), "little") == exp_inv, hex(v)
        assert int.from_bytes(bytes(sqr_out[48 * i:48 * i + 48]), "little") == (v % P) ** 2 * rinv % P, hex(v)
        assert int.from_bytes(bytes(mul_out[48 * i:48 * i + 48]), "little") == \
            (v % P) * (others[i] % P) * rinv % P, (hex(v), hex(others[i]))
