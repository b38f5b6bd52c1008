"""GPU parity for batched point decoding and validation against the
reference's blst_p1_uncompress / blst_p1_deserialize / blst_p1_affine_in_g1
on crafted encodings (tests/golden/decode.json, generated by the reference):
the same error code for every element, the same output bytes, and the
caller's bytes left untouched on failure."""
import json
import os

import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def dec():
    return json.load(open(os.path.join(HERE, "golden", "decode.json")))


@pytest.mark.parametrize("kind", ["uncompress", "deserialize"])
def test_decode_matches_reference(gpu, dec, kind):
    cases = dec[kind]
    n = len(cases)
    enc = b"".join(bytes.fromhex(c["in"]) for c in cases)
    init = bytes(range(96)) * n
    rc, errs, out = gpu.p1s_decode(enc, n, kind == "uncompress", init)
    assert rc == 0
    for i, c in enumerate(cases):
        assert errs[i] == c["err"], (i, c["in"][:8], errs[i], c["err"])
        assert out[96 * i:96 * i + 96].hex() == c["out"], i


def test_in_g1_matches_reference(gpu, dec):
    cases = dec["in_g1"]
    pts = b"".join(bytes.fromhex(c["point"]) for c in cases)
    rc, res = gpu.p1s_affine_in_g1(pts, len(cases))
    assert rc == 0
    assert res == [c["in_g1"] for c in cases]
    assert sum(1 for c in cases if not c["in_g1"]) >= 30


def test_decode_with_group_check(gpu, dec, oracle):
    cases = dec["deserialize"]
    enc = b"".join(bytes.fromhex(c["in"]) for c in cases)
    member = {c["point"]: c["in_g1"] for c in dec["in_g1"]}
    rc, errs, out = gpu.p1s_decode(enc, len(cases), False, bytes(96 * len(cases)), check_group=True)
    assert rc == 0
    for i, c in enumerate(cases):
        exp = c["err"]
        if exp == 0 and not member[c["out"]]:
            exp = 3
        assert errs[i] == exp, i


def test_decode_round_trip_at_scale(gpu, oracle, synth):
    n = 1 << 16
    pts = gpu.points_from_scalars(synth.point_scalars(88, n), n)
    comp = b"".join(oracle.compress(oracle.from_affine(pts[96 * i:96 * i + 96])) for i in range(0, n, 64))
    m = len(comp) // 48
    rc, errs, out = gpu.p1s_decode(comp, m, True, check_group=True)
    assert rc == 0 and errs == [0] * m
    assert out == b"".join(pts[96 * i:96 * i + 96] for i in range(0, n, 64))
    rc, res = gpu.p1s_affine_in_g1(pts, n)
    assert rc == 0 and all(res)
