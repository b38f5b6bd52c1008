"""GPU parity for the batch-affine bucket accumulation: the variable-time
field inversion against big-integer arithmetic, and whole MSMs with 1, 2, 3
and 5 affine rounds forced on (at every size, also where the size rule
would not choose them) against the reference's golden bytes and the
oracle, including the cases that take the special branches of an affine
addition: equal points (doubling), opposite points (infinity), infinity
operands and runs of infinities.  Integer arithmetic: byte equality."""
import random

import pytest

pytestmark = pytest.mark.gpu

P = 0x1a0111ea397fe69a4b1ba7b6434bacd764774b84f38512bf6730d2a0f6b0f6241eabfffeb153ffffb9feffffffffaaab
R = 0x73eda753299d7d483339d80809a1d80553bda402fffe5bfeffffffff00000001
RM = (1 << 384) % P
ROUNDS = (1, 2, 3, 5)


def test_fp_inv_matches_bigint(gpu):
    rnd = random.Random(11)
    vals = [0, 1, 2, P - 1, P - 2, P, P + 1, 2 * P - 1, RM, RM * RM % P, (P + 1) // 2, 1 << 380, (1 << 381) - 1,
            1 << 32, (1 << 32) - 1]
    vals += [rnd.randrange(2 * P) for _ in range(5000)]
    vals += [rnd.randrange(1 << rnd.randrange(1, 381)) for _ in range(1000)]   # short operands
    buf = b"".join(v.to_bytes(48, "little") for v in vals)
    out = gpu.fp_inv(buf, len(vals))
    for i, v in enumerate(vals):
        got = int.from_bytes(out[48 * i:48 * i + 48], "little")
        a = v * pow(RM, -1, P) % P                     # the field element v represents
        exp = 0 if a == 0 else pow(a, -1, P) * RM % P
        assert got == exp, (i, hex(v))


def _msm_inputs(oracle, gpu, synth, c):
    n, nbits = c["n"], c["nbits"]
    if n > 4096:
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


@pytest.fixture
def restore_rounds(gpu):
    prev = gpu.msm_affine_rounds(-2)
    yield
    gpu.msm_affine_rounds(prev)


def test_affine_rounds_match_reference_golden(gpu, oracle, synth, golden, restore_rounds):
    """Every golden MSM up to 2^20 points (uniform, 64-bit, zero scalars with
    duplicated points; nbits 1 .. 256) with each forced round count."""
    for c in golden["msm"]:
        if c["n"] > (1 << 20):
            continue
        pts, sc = _msm_inputs(oracle, gpu, synth, c)
        for r in ROUNDS:
            gpu.msm_affine_rounds(r)
            got = oracle.compress(gpu.p1s_mult_pippenger(pts, sc, c["n"], c["nbits"]))
            assert got.hex() == c["compressed"], (c["seed"], c["n"], r)


def _edge_cases(oracle, synth):
    n = 3000
    base = oracle.gen_points(811, n)
    one = base[:96]
    k = synth.scalars(812, 1, 0)
    kneg = (R - int.from_bytes(k, "little")).to_bytes(32, "little")
    cases = {
        # every window's buckets hold copies of one point: all pairs double
        "equal_points_equal_scalars": (one * n, k * n, n, 255),
        # P and -P (k and r - k) in the same buckets: pairs cancel to infinity
        "opposite_pairs": (one * n, (k + kneg) * (n // 2), n, 255),
        # infinity operands among ordinary points
        "infinity_points": (b"".join(bytes(96) if i % 7 == 3 else base[96 * i:96 * i + 96] for i in range(n)),
                            synth.scalars(813, n, 0), n, 255),
        # without the GLV split (64-bit scalars), equal points
        "equal_points_64bit": (one * n, synth.scalars(814, 1, 1)[:8] * n, n, 64),
        "pair_of_points": (base[:192], synth.scalars(815, 2, 0), 2, 255),
        "one_point": (base[:96], synth.scalars(816, 1, 0), 1, 255),
    }
    # all-infinity input and a mix of equal points and their negatives in runs
    cases["all_infinity"] = (bytes(96 * 64), synth.scalars(817, 64, 0), 64, 255)
    mixed = [k if (i // 5) % 2 == 0 else kneg for i in range(n)]
    cases["runs_of_opposites"] = (one * n, b"".join(mixed), n, 255)
    return cases


@pytest.mark.parametrize("name", ["equal_points_equal_scalars", "opposite_pairs", "infinity_points",
                                  "equal_points_64bit", "pair_of_points", "one_point", "all_infinity",
                                  "runs_of_opposites"])
def test_affine_rounds_special_cases(gpu, oracle, synth, restore_rounds, name):
    pts, sc, n, nbits = _edge_cases(oracle, synth)[name]
    exp = oracle.msm(pts, sc, n, nbits)
    for r in ROUNDS:
        gpu.msm_affine_rounds(r)
        assert oracle.compress(gpu.p1s_mult_pippenger(pts, sc, n, nbits)) == exp, (name, r)
