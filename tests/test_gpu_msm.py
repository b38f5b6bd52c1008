"""GPU parity for the MSM through the C ABI: bit-exact 48-byte compressed
results against the reference's golden vectors and the oracle, the
reference's fail-closed edge cases, descriptor arrays, and a full-size
linearity property.  Integer arithmetic: the bar is byte equality."""
import ctypes as C

import pytest

pytestmark = pytest.mark.gpu

R = 0x73eda753299d7d483339d80809a1d80553bda402fffe5bfeffffffff00000001
INF48 = bytes([0xC0]) + bytes(47)


def _msm_inputs(oracle, gpu, synth, c, use_gpu_points=False):
    n, nbits = c["n"], c["nbits"]
    if use_gpu_points:
        pts = gpu.points_from_scalars(synth.point_scalars(c["seed"], n), n)
        if c["dup"]:
            pts = bytes(synth.apply_duplicates(bytearray(pts), c["seed"], n))
    else:
        pts = oracle.gen_points(c["seed"], n)
        if c["dup"]:
            pts = oracle.duplicate_points(c["seed"], n, pts)
    sc = synth.scalars(c["seed"] + 1000, n, c["kind"])
    nb = (nbits + 7) // 8
    if nb != 32:
        sc = b"".join(sc[32 * i:32 * i + nb] for i in range(n))
    return pts, sc


def test_fp_mul_matches_oracle(gpu, oracle, synth):
    import random
    rnd = random.Random(5)
    p = 0x1a0111ea397fe69a4b1ba7b6434bacd764774b84f38512bf6730d2a0f6b0f6241eabfffeb153ffffb9feffffffffaaab
    vals = [0, 1, 2, p - 1, p - 2, (1 << 383) % p, (1 << 384) % p, (p + 1) // 2]
    vals += [rnd.randrange(p) for _ in range(2000)]
    a = [vals[i] for i in range(len(vals))]
    b = [vals[(7 * i + 3) % len(vals)] for i in range(len(vals))]
    n = len(a)
    ab = b"".join(x.to_bytes(48, "little") for x in a)
    bb = b"".join(x.to_bytes(48, "little") for x in b)
    got = gpu.fp_mul(ab, bb, n)
    rinv = pow(1 << 384, -1, p)
    for i in range(n):
        exp = a[i] * b[i] * rinv % p
        assert int.from_bytes(got[48 * i:48 * i + 48], "little") == exp, i


def test_fp_sqr_matches_bigint(gpu):
    """The dedicated squaring (catmsm_fp_mul with a == b) on lazily reduced
    inputs in [0, 2p), including the boundary values."""
    import random
    rnd = random.Random(6)
    p = 0x1a0111ea397fe69a4b1ba7b6434bacd764774b84f38512bf6730d2a0f6b0f6241eabfffeb153ffffb9feffffffffaaab
    vals = [0, 1, 2, p - 1, p, p + 1, 2 * p - 1, 2 * p - 2, (p + 1) // 2, (1 << 381) - 1, (1 << 32) - 1,
            sum(0xffffffff << (64 * k) for k in range(6)) % (2 * p)]
    vals += [rnd.randrange(2 * p) for _ in range(4000)]
    n = len(vals)
    buf = b"".join(x.to_bytes(48, "little") for x in vals)
    out = bytearray(48 * n)
    import ctypes as C
    L = gpu.load()
    ab = (C.c_char * len(buf)).from_buffer(bytearray(buf))
    assert L.catmsm_fp_mul((C.c_char * len(out)).from_buffer(out), ab, ab, n) == 0
    rinv = pow(1 << 384, -1, p)
    for i, x in enumerate(vals):
        assert int.from_bytes(out[48 * i:48 * i + 48], "little") == x * x * rinv % p, i


def test_points_from_scalars_matches_oracle(gpu, oracle, synth):
    n = 3000
    k = synth.point_scalars(77, n)
    assert gpu.points_from_scalars(k, n) == oracle.points_from_scalars(k, n)


def test_msm_golden_small(gpu, oracle, synth, golden):
    for c in golden["msm"]:
        if c["n"] > (1 << 16):
            continue
        pts, sc = _msm_inputs(oracle, gpu, synth, c)
        got = oracle.compress(gpu.p1s_mult_pippenger(pts, sc, c["n"], c["nbits"]))
        assert got.hex() == c["compressed"], c


def test_msm_golden_large(gpu, oracle, synth, golden):
    big = [c for c in golden["msm"] if c["n"] > (1 << 16)]
    if not big:
        pytest.skip("no large golden cases")
    for c in big:
        pts, sc = _msm_inputs(oracle, gpu, synth, c, use_gpu_points=True)
        got = oracle.compress(gpu.p1s_mult_pippenger(pts, sc, c["n"], c["nbits"]))
        assert got.hex() == c["compressed"], (c["seed"], c["n"])


@pytest.mark.parametrize("n,nbits,kind", [(2, 255, 0), (5, 256, 0), (31, 64, 1), (64, 9, 0),
                                          (333, 255, 2), (1023, 130, 0), (5000, 255, 0),
                                          (1 << 13, 64, 1), (12345, 255, 2)])
def test_msm_matches_oracle(gpu, oracle, synth, n, nbits, kind):
    pts = oracle.gen_points(900 + n, n)
    sc = synth.scalars(901 + n, n, kind)
    nb = (nbits + 7) // 8
    if nb != 32:
        sc = b"".join(sc[32 * i:32 * i + nb] for i in range(n))
    assert oracle.compress(gpu.p1s_mult_pippenger(pts, sc, n, nbits)) == oracle.msm(pts, sc, n, nbits)


def test_msm_fail_closed_edge_cases(gpu, oracle, synth):
    n = 8
    pts = oracle.gen_points(3, n)
    sc = synth.scalars(4, n, 0)
    # n == 0 and nbits == 0 -> infinity
    assert oracle.compress(gpu.p1s_mult_pippenger(pts, sc, 0, 255)) == INF48
    assert oracle.compress(gpu.p1s_mult_pippenger(pts, sc, n, 0)) == INF48
    # nbits > 256 -> infinity
    assert oracle.compress(gpu.p1s_mult_pippenger(pts, sc + bytes(64), n, 257)) == INF48
    # n > 1 with null scratch -> infinity; n == 1 needs no scratch
    assert oracle.compress(gpu.p1s_mult_pippenger(pts, sc, n, 255, scratch=False)) == INF48
    one = gpu.p1s_mult_pippenger(pts[:96], sc[:32], 1, 255, scratch=False)
    assert oracle.compress(one) == oracle.msm(pts[:96], sc[:32], 1, 255)
    # null head pointers -> infinity
    assert oracle.compress(gpu.p1s_mult_pippenger_descriptors([None, None], [None, None], n, 255)) == INF48
    # explicit window out of range -> infinity; in range -> same as default
    pb = (C.c_char * len(pts)).from_buffer(bytearray(pts))
    sb = (C.c_char * len(sc)).from_buffer(bytearray(sc))
    parr = [C.addressof(pb), None]
    sarr = [C.addressof(sb), None]
    assert oracle.compress(gpu.p1s_mult_pippenger_descriptors(parr, sarr, n, 255, window=0)) == INF48
    assert oracle.compress(gpu.p1s_mult_pippenger_descriptors(parr, sarr, n, 255, window=25)) == INF48
    assert oracle.compress(gpu.p1s_mult_pippenger_descriptors(parr, sarr, n, 255, window=3)) == \
        oracle.msm(pts, sc, n, 255)
    # all-zero scalars -> infinity
    assert oracle.compress(gpu.p1s_mult_pippenger(pts, bytes(32 * n), n, 255)) == INF48
    # infinity points are skipped
    pts_inf = bytearray(pts)
    pts_inf[96 * 2:96 * 3] = bytes(96)
    pts_inf[96 * 5:96 * 6] = bytes(96)
    assert oracle.compress(gpu.p1s_mult_pippenger(bytes(pts_inf), sc, n, 255)) == \
        oracle.msm(bytes(pts_inf), sc, n, 255)
    # equal points double inside a bucket; k P + (r - k) P cancels to infinity
    P = pts[:96]
    k = (5).to_bytes(32, "little")
    twice = gpu.p1s_mult_pippenger(P + P, k + k, 2, 255)
    assert oracle.compress(twice) == oracle.msm(P + P, k + k, 2, 255)
    kk = int.from_bytes(sc[:32], "little")
    cancel = sc[:32] + (R - kk).to_bytes(32, "little")
    assert oracle.compress(gpu.p1s_mult_pippenger(P + P, cancel, 2, 255)) == INF48


def test_msm_descriptor_arrays(gpu, oracle, synth):
    n = 9
    pts = bytearray(oracle.gen_points(55, n))
    sc = bytearray(synth.scalars(56, n, 0))
    pb = (C.c_char * len(pts)).from_buffer(pts)
    sb = (C.c_char * len(sc)).from_buffer(sc)
    bp, bs = C.addressof(pb), C.addressof(sb)
    order = [3, 0, 5, 1, 8, 2, 7, 4, 6]
    perm_p = b"".join(bytes(pts[96 * i:96 * i + 96]) for i in order)
    perm_s = b"".join(bytes(sc[32 * i:32 * i + 32]) for i in order)
    exp = oracle.msm(perm_p, perm_s, n, 255)
    got = gpu.p1s_mult_pippenger_descriptors([bp + 96 * i for i in order], [bs + 32 * i for i in order], n, 255)
    assert oracle.compress(got) == exp
    # two explicit heads then NULL continuation
    got2 = gpu.p1s_mult_pippenger_descriptors([bp, bp + 96, None], [bs, bs + 32, None], n, 255)
    assert oracle.compress(got2) == oracle.msm(bytes(pts), bytes(sc), n, 255)


def test_msm_output_is_normalised(gpu, oracle, synth):
    n = 100
    pts = oracle.gen_points(8, n)
    sc = synth.scalars(9, n, 0)
    out = gpu.p1s_mult_pippenger(pts, sc, n, 255)
    one_mont = ((1 << 384) % 0x1a0111ea397fe69a4b1ba7b6434bacd764774b84f38512bf6730d2a0f6b0f6241eabfffeb153ffffb9feffffffffaaab)
    assert int.from_bytes(out[96:144], "little") == one_mont
    assert oracle.on_curve(out)


def test_msm_linearity_full_size(gpu, oracle, synth):
    """n = 2^20, P_i = s_i G:  sum k_i P_i == (sum k_i s_i mod r) G."""
    n = 1 << 20
    s = synth.point_scalars(4242, n)
    k = synth.scalars(4343, n, 0)
    pts = gpu.points_from_scalars(s, n)
    got = oracle.compress(gpu.p1s_mult_pippenger(pts, k, n, 255))
    import numpy as np
    sv = np.frombuffer(s, dtype=np.uint64).reshape(n, 4)
    kv = np.frombuffer(k, dtype=np.uint64).reshape(n, 4)
    acc = 0
    for i in range(0, n, 4096):
        for a, b in zip(sv[i:i + 4096].tolist(), kv[i:i + 4096].tolist()):
            acc += (a[0] | a[1] << 64 | a[2] << 128 | a[3] << 192) * (b[0] | b[1] << 64 | b[2] << 128 | b[3] << 192)
        acc %= R
    exp = oracle.compress(oracle.mult(oracle.generator(), acc.to_bytes(32, "little"), 256))
    assert got == exp


def test_msm_linearity_max_size(gpu, oracle, synth):
    """n = 2^24 (the pipeline at 2^25 GLV points, ~12 GB of device working
    set) through the device-resident entry: sum k_i P_i == (sum k_i s_i mod
    r) G, the sums of products taken with numpy in 32-bit limbs."""
    import numpy as np
    import torch
    n = 1 << 24
    s = synth.point_scalars(4444, n)
    k = synth.scalars(4545, n, 0)
    ks = torch.frombuffer(bytearray(s), dtype=torch.uint8).cuda()
    dp = torch.empty(n * 96, dtype=torch.uint8, device="cuda")
    torch.cuda.synchronize()
    assert gpu.load().catmsm_p1_affines_from_scalars_device(dp.data_ptr(), ks.data_ptr(), n) == 0
    del ks
    dk = torch.frombuffer(bytearray(k), dtype=torch.uint8).cuda()
    torch.cuda.synchronize()
    got = oracle.compress(gpu.msm_device(dp.data_ptr(), dk.data_ptr(), 32, n, 255, 0))
    # sum_i s_i k_i from the 64 limb-pair columns: the low and high 32-bit
    # halves of the 64-bit products are summed separately (each sum < 2^56)
    sv = np.frombuffer(s, dtype=np.uint32).reshape(n, 8).astype(np.uint64)
    kv = np.frombuffer(k, dtype=np.uint32).reshape(n, 8).astype(np.uint64)
    total = 0
    for i in range(8):
        for j in range(8):
            prod = sv[:, i] * kv[:, j]                         # < 2^64, exact
            lo = int((prod & 0xffffffff).sum())
            hi = int((prod >> 32).sum())
            total += (lo + (hi << 32)) << (32 * (i + j))
    exp = oracle.compress(oracle.mult(oracle.generator(), (total % R).to_bytes(32, "little"), 256))
    assert got == exp


def test_msm_hot_buckets(gpu, oracle, synth):
    """Every window puts all points in one bucket (equal scalars): the
    chunk-spanning fixup must stay parallel and exact (spans of ~1.9k
    chunks: the grid-wide join of the serial fixup, k_fixup_giant<false>)."""
    n = 1 << 16
    pts = oracle.gen_points(31, n)
    k = synth.scalars(32, 1, 0)
    sc = k * n
    assert oracle.compress(gpu.p1s_mult_pippenger(pts, sc, n, 255)) == oracle.msm(pts, sc, n, 255)


def test_msm_hot_buckets_segmented_grid_join(gpu, oracle, synth):
    """n = 2^22 with one scalar repeated and window 16: buckets average more
    than two chunks (the segmented fixup), and each window's two occupied
    buckets span ~44k chunks (~1.4k warp pieces), so their joins take the
    grid-wide path (k_fixup_giant<true>).  sum k P_i == (k sum s_i mod r) G."""
    import numpy as np
    import torch
    n = 1 << 22
    s = synth.point_scalars(4646, n)
    k = synth.scalars(4747, 1, 0)
    ks = torch.frombuffer(bytearray(s), dtype=torch.uint8).cuda()
    dp = torch.empty(n * 96, dtype=torch.uint8, device="cuda")
    torch.cuda.synchronize()
    assert gpu.load().catmsm_p1_affines_from_scalars_device(dp.data_ptr(), ks.data_ptr(), n) == 0
    del ks
    dk = torch.frombuffer(bytearray(k * n), dtype=torch.uint8).cuda()
    torch.cuda.synchronize()
    got = oracle.compress(gpu.msm_device(dp.data_ptr(), dk.data_ptr(), 32, n, 255, 16))
    sv = np.frombuffer(s, dtype=np.uint32).reshape(n, 8).astype(np.uint64)
    ssum = sum(int(sv[:, i].sum()) << (32 * i) for i in range(8))
    kk = int.from_bytes(k, "little")
    exp = oracle.compress(oracle.mult(oracle.generator(), (kk * ssum % R).to_bytes(32, "little"), 256))
    assert got == exp


@pytest.mark.parametrize("glv", [0, 1])
@pytest.mark.parametrize("window", [2, 5, 8, 13, 15, 16, 17, 20])
def test_msm_device_windows(gpu, oracle, synth, window, glv):
    """Device-resident entry point over every window width class, with and
    without the GLV split; without it, 15 and 17 divide 255 (a carry-only
    top window)."""
    import torch
    n = 20000
    pts = oracle.gen_points(40 + window, n)
    sc = synth.scalars(41 + window, n, 0)
    dp = torch.frombuffer(bytearray(pts), dtype=torch.uint8).cuda()
    ds = torch.frombuffer(bytearray(sc), dtype=torch.uint8).cuda()
    torch.cuda.synchronize()
    prev = gpu.msm_glv(glv)
    try:
        got = gpu.msm_device(dp.data_ptr(), ds.data_ptr(), 32, n, 255, window)
    finally:
        gpu.msm_glv(prev)
    assert oracle.compress(got) == oracle.msm(pts, sc, n, 255)


LAMBDA = 0xac45a4010001a40200000000ffffffff


def test_msm_glv_split_edge_scalars(gpu, oracle, synth):
    """Scalars at the GLV split's boundaries (0, 1, lambda and its
    neighbours, (lambda+1)/2, multiples of lambda, r - 1, r, r + 1, values
    above 2r up to 2^256 - 1), infinity and repeated points: the GLV path
    equals the plain path and the oracle, and the plan doubles the points."""
    half = (LAMBDA + 1) // 2
    ks = [0, 1, 2, LAMBDA - 1, LAMBDA, LAMBDA + 1, half - 1, half, half + 1, R - 1, R, R + 1, 2 * R + 5,
          (1 << 256) - 1, (1 << 255), LAMBDA * LAMBDA, LAMBDA * LAMBDA + LAMBDA, half * LAMBDA,
          (half - 1) * LAMBDA + half, (LAMBDA + 1) * LAMBDA - 1, R - LAMBDA, R - half]
    ks += [int.from_bytes(synth.scalars(77, 1, 0), "little") + j * LAMBDA for j in range(10)]
    n = len(ks)
    pts = bytearray(oracle.gen_points(78, n))
    pts[96 * 3:96 * 4] = bytes(96)                      # a point at infinity
    pts[96 * 5:96 * 6] = pts[96 * 6:96 * 7]             # a repeated point
    pts = bytes(pts)
    sc = b"".join((k % (1 << 256)).to_bytes(32, "little") for k in ks)
    assert gpu.msm_plan(n, 256)[2] == 2 * n and gpu.msm_plan(n, 128)[2] == n
    exp = oracle.msm(pts, sc, n, 256)
    assert oracle.compress(gpu.p1s_mult_pippenger(pts, sc, n, 256)) == exp
    prev = gpu.msm_glv(0)
    try:
        assert gpu.msm_plan(n, 256)[2] == n
        assert oracle.compress(gpu.p1s_mult_pippenger(pts, sc, n, 256)) == exp
    finally:
        gpu.msm_glv(prev)
    # one point per scalar: every split alone
    for i, k in enumerate(ks):
        p1 = pts[96 * i:96 * i + 96]
        s1 = sc[32 * i:32 * i + 32]
        two = p1 + p1
        got = gpu.p1s_mult_pippenger(two, s1 + bytes(32), 2, 256)
        assert oracle.compress(got) == oracle.msm(two, s1 + bytes(32), 2, 256), hex(k)
