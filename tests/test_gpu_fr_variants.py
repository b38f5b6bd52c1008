"""GPU parity for blst_p1s_mult_fr and blst_p1s_mult_batch_affine_fr against
the reference's outputs (tests/golden/golden.json, generated by the
reference), and the reference's scratch and argument contract: false with
ret unchanged below the queried scratch, for an invalid window or batch size
and for NULL inputs; infinity and true for an empty MSM."""
import pytest

pytestmark = pytest.mark.gpu

INF = bytes([0xC0]) + bytes(47)


def _inputs(oracle, c):
    n = c["n"]
    pts = oracle.gen_points(c["seed"], n)
    if c["inf"]:
        k = c["seed"] % n
        pts = pts[:96 * k] + bytes(96) + pts[96 * (k + 1):]
    sc = oracle.gen_scalars(c["seed"] + 1000, n, 0)
    frs = b"".join(oracle.fr_to_mont(sc[32 * i:32 * i + 32]) for i in range(n))
    return pts, frs


def test_fr_variants_match_reference(gpu, golden, oracle):
    cases = golden["msm_fr_variants"]["cases"]
    assert len(cases) >= 12
    for c in cases:
        pts, frs = _inputs(oracle, c)
        if c["api"] == "mult_fr":
            ok, ret = gpu.p1s_mult_fr(pts, frs, c["n"])
        else:
            ok, ret = gpu.p1s_mult_batch_affine_fr(pts, frs, c["n"], c["window"], c["batch"])
        assert ok, c
        assert oracle.compress(ret) == bytes.fromhex(c["compressed"]), (c["api"], c["n"])


def test_fr_variants_fail_closed(gpu, oracle):
    n = 300
    pts = oracle.gen_points(301, n)
    frs = b"".join(oracle.fr_to_mont(oracle.gen_scalars(302, n, 0)[32 * i:32 * i + 32]) for i in range(n))
    sentinel = bytes(range(144))
    need = gpu.p1s_mult_fr_scratch_sizeof(n)
    ok, ret = gpu.p1s_mult_fr(pts, frs, n, scratch_size=need - 1, ret_init=sentinel)
    assert not ok and ret == sentinel
    ok, ret = gpu.p1s_mult_fr(None, frs, n, ret_init=sentinel)
    assert not ok and ret == sentinel
    ok, ret = gpu.p1s_mult_fr(pts, None, n, ret_init=sentinel)
    assert not ok and ret == sentinel
    ok, ret = gpu.p1s_mult_fr(pts, frs, n, scratch_size=-1, ret_init=sentinel)
    assert not ok and ret == sentinel
    ok, ret = gpu.p1s_mult_fr(pts, frs, 0, ret_init=sentinel)
    assert ok and oracle.compress(ret) == INF
    for w, b in ((0, 128), (25, 128), (10, 100), (10, 0), (10, 512)):
        ok, ret = gpu.p1s_mult_batch_affine_fr(pts, frs, n, w, b, scratch_size=1 << 20, ret_init=sentinel)
        assert not ok and ret == sentinel, (w, b)
    need = gpu.p1s_mult_batch_affine_fr_scratch_sizeof(n, 9, 384)
    ok, ret = gpu.p1s_mult_batch_affine_fr(pts, frs, n, 9, 384, scratch_size=need - 8, ret_init=sentinel)
    assert not ok and ret == sentinel
    ok, ret = gpu.p1s_mult_batch_affine_fr(pts, frs, 0, 9, 384, ret_init=sentinel)
    assert ok and oracle.compress(ret) == INF
    # the accepted calls all give the same group element
    exp = oracle.msm_fr(pts, frs, n)
    for w, b in ((1, 128), (9, 384), (16, 128)):
        ok, ret = gpu.p1s_mult_batch_affine_fr(pts, frs, n, w, b)
        assert ok and oracle.compress(ret) == exp, (w, b)
    ok, ret = gpu.p1s_mult_fr(pts, frs, n)
    assert ok and oracle.compress(ret) == exp
