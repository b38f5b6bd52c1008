"""GPU parity for blst_p1s_tile_pippenger: one signed window of the MSM at an
exact bit offset, against the reference's outputs (tests/golden/golden.json,
generated by the reference), its fail-closed rules, and the property that
the tiles of a full window decomposition fold back to the whole MSM."""
import pytest

pytestmark = pytest.mark.gpu

INF = bytes([0xC0]) + bytes(47)


def _inputs(oracle, synth, c):
    n, nbits = c["n"], c["nbits"]
    pts = oracle.gen_points(c["seed"], n)
    if c["dup"]:
        pts = oracle.duplicate_points(c["seed"], n, pts)
    sc = synth.scalars(c["seed"] + 1000, n, c["kind"])
    nb = (nbits + 7) // 8
    if nb != 32:
        sc = b"".join(sc[32 * i:32 * i + nb] for i in range(n))
    return pts, sc


def test_tile_matches_reference(gpu, golden, oracle, synth):
    for c in golden["tile"]:
        pts, sc = _inputs(oracle, synth, c)
        got = gpu.p1s_tile_pippenger(pts, sc, c["n"], c["nbits"], c["bit0"], c["window"])
        assert oracle.compress(got) == bytes.fromhex(c["compressed"]), c


def test_tile_fail_closed(gpu, oracle, synth):
    n = 20
    pts = oracle.gen_points(120, n)
    sc = synth.scalars(121, n, 0)
    for nbits, bit0, window, scratch in ((255, 0, 0, True), (255, 0, 25, True), (255, 255, 4, True),
                                         (0, 0, 4, True), (257, 0, 4, True), (255, 0, 4, False)):
        got = gpu.p1s_tile_pippenger(pts, sc, n, nbits, bit0, window, scratch=scratch)
        assert oracle.compress(got) == INF, (nbits, bit0, window, scratch)
    assert oracle.compress(gpu.p1s_tile_pippenger(pts, sc, 0, 255, 0, 4)) == INF


@pytest.mark.parametrize("window", [5, 13, 17])
def test_tiles_fold_to_msm(gpu, oracle, synth, window):
    """sum_w 2^(w c) tile(w c, c) over the reference's window decomposition
    (multi_scalar.cpp:911-921: windows 0 .. nbits / c) equals the whole MSM.
    The tile API needs bit0 < nbits, so the scalars are taken as 256-bit
    (bit 255 is zero for Fr scalars): when c divides 255 the carry window at
    bit 255 is then a legal tile."""
    n = 3000
    pts = oracle.gen_points(130 + window, n)
    sc = synth.scalars(131 + window, n, 0)
    acc = None
    for bit0 in range(0, 256, window):
        t = gpu.p1s_tile_pippenger(pts, sc, n, 256, bit0, window)
        term = oracle.mult(t, (1 << bit0).to_bytes(32, "little"), 256)
        acc = term if acc is None else oracle.add(acc, term)
    assert oracle.compress(acc) == oracle.msm(pts, sc, n, 255)
