"""GPU parity for batched commitments over a resident basis: every MSM of a
batch equals the oracle's single MSM over the same leading basis points,
byte for byte (compressed), with and without CUDA-graph replay, across window
widths, and for the empty and full-basis edge cases."""
import random

import pytest

pytestmark = pytest.mark.gpu


def _batch(oracle, synth, n, nmsm, seed):
    rnd = random.Random(seed)
    counts = [int(2 ** rnd.uniform(8, 12)) for _ in range(nmsm)]
    counts[0] = 0
    counts[1] = n
    counts[2] = 1
    total = sum(counts)
    sc = synth.scalars(seed, total, 0)
    return counts, sc


def _check(oracle, basis_pts, counts, sc, out):
    off = 0
    for j, k in enumerate(counts):
        got = oracle.compress(out[144 * j:144 * j + 144])
        if k == 0:
            assert got == bytes([0xC0]) + bytes(47), j
        else:
            exp = oracle.msm(basis_pts[:96 * k], sc[32 * off:32 * (off + k)], k, 256)
            assert got == exp, (j, k)
        off += k


def test_batch_matches_oracle(gpu, oracle, synth):
    n = 4096
    pts = oracle.gen_points(600, n)
    b = gpu.Basis(pts, n)
    counts, sc = _batch(oracle, synth, n, 24, 601)
    out = b.msm_batch(counts, sc, use_graph=True)
    _check(oracle, pts, counts, sc, out)
    # replay the captured graph with a different batch of the same size
    counts2, sc2 = _batch(oracle, synth, n, 24, 602)
    out2 = b.msm_batch(counts2, sc2, use_graph=True)
    _check(oracle, pts, counts2, sc2, out2)
    # without the graph: the same points (Jacobian bytes may differ in Z: the
    # accumulation order inside a bucket is not fixed)
    out3 = b.msm_batch(counts2, sc2, use_graph=False)
    for j in range(len(counts2)):
        assert oracle.compress(out3[144 * j:144 * j + 144]) == oracle.compress(out2[144 * j:144 * j + 144])
    b.close()


@pytest.mark.parametrize("window", [2, 7, 9, 13, 16])
def test_batch_windows(gpu, oracle, synth, window):
    n = 700
    pts = oracle.gen_points(610 + window, n)
    b = gpu.Basis(pts, n, window)
    rnd = random.Random(window)
    counts = [rnd.randrange(0, n + 1) for _ in range(6)] + [n]
    sc = synth.scalars(620 + window, sum(counts), 0)
    out = b.msm_batch(counts, sc)
    _check(oracle, pts, counts, sc, out)
    b.close()


def test_batch_autotune_persists(gpu, oracle, synth, tmp_path, monkeypatch):
    monkeypatch.setenv("CATMSM_TUNE_CACHE", str(tmp_path / "tune.txt"))
    n = 1024
    pts = oracle.gen_points(630, n)
    b = gpu.Basis(pts, n)
    counts = [512] * 8
    sc = synth.scalars(631, sum(counts), 0)
    w, c = b.autotune(counts, sc)
    assert 9 <= w <= 13 and c in (8, 16, 32)
    text = (tmp_path / "tune.txt").read_text()
    assert "n=1024 nmsm=8" in text and ("|%d %d" % (w, c)) in text
    b.set_config(9, 8)
    assert b.autotune(counts, sc) == (w, c)          # served from the cache
    _check(oracle, pts, counts, sc, b.msm_batch(counts, sc))
    b.close()


def test_batch_commitments_match_reference_golden(gpu, oracle, synth, golden):
    """The batched-commitments workload itself: 1024 commitments over the
    4096-point basis (k_j = floor(2^U), U ~ U[8, 12]), every result against
    the reference's own blst_p1s_mult_pippenger output, with the library's
    default (window, chunk) and with the (11, 96) the autotuner picks for this
    batch on a GB300."""
    import numpy as np
    g = golden["batch_commitments"]
    nb, seed = g["n_basis"], g["seed"]
    counts = g["counts"]
    rng = np.random.default_rng(seed)
    assert [int(2 ** u) for u in rng.uniform(8, 12, len(counts))] == counts
    pts = gpu.points_from_scalars(synth.point_scalars(seed, nb), nb)
    sc = synth.scalars(seed + 3000, sum(counts), 0)
    b = gpu.Basis(pts, nb)
    for cfg in (None, (11, 96)):
        if cfg:
            b.set_config(*cfg)
        out = b.msm_batch(counts, sc)
        got = [oracle.compress(out[144 * j:144 * j + 144]).hex() for j in range(len(counts))]
        bad = [j for j in range(len(counts)) if got[j] != g["compressed"][j]]
        assert not bad, (cfg, bad[:8])
    b.close()
