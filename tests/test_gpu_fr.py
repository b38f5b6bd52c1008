"""GPU parity for the scalar-field entry points: blst_p1s_mult_pippenger_fr
(Montgomery Fr scalars) and blst_fr_fft / blst_fr_fft_with_domain, byte for
byte against the reference's golden vectors, plus the reference's argument
and failure rules."""
import hashlib

import pytest

pytestmark = pytest.mark.gpu


def _frs(oracle, seed, n):
    sc = oracle.gen_scalars(seed, n, 0)
    return b"".join(oracle.fr_to_mont(sc[32 * i:32 * i + 32]) for i in range(n))


def test_msm_fr_golden(gpu, oracle, golden):
    for c in golden["msm_fr"]:
        n = c["n"]
        pts = oracle.gen_points(c["seed"], n)
        ok, ret = gpu.p1s_mult_pippenger_fr(pts, _frs(oracle, c["seed"] + 1000, n), n)
        assert ok and oracle.compress(ret).hex() == c["compressed"], n


def test_msm_fr_argument_rules(gpu, oracle):
    n = 50
    pts = oracle.gen_points(61, n)
    frs = _frs(oracle, 62, n)
    sentinel = bytes(range(144))
    need = gpu.p1s_mult_pippenger_fr_scratch_sizeof(n)
    assert need == oracle.scratch_sizeof(n) + 32 * n
    assert gpu.p1s_mult_pippenger_fr_scratch_sizeof(0) == 0
    assert gpu.p1s_mult_pippenger_fr_scratch_sizeof(1) == 32
    ok, ret = gpu.p1s_mult_pippenger_fr(pts, frs, 0, ret_init=sentinel)    # empty: infinity, true
    assert ok and ret == bytes(144)
    ok, ret = gpu.p1s_mult_pippenger_fr(pts, frs, n, scratch_size=need - 1, ret_init=sentinel)
    assert not ok and ret == sentinel                                        # short scratch: unchanged
    ok, ret = gpu.p1s_mult_pippenger_fr(pts, frs, n, scratch_size=-1, ret_init=sentinel)
    assert not ok and ret == sentinel                                        # NULL scratch
    ok, ret = gpu.p1s_mult_pippenger_fr(None, frs, n, ret_init=sentinel)
    assert not ok and ret == sentinel
    ok, ret = gpu.p1s_mult_pippenger_fr(pts, frs, n)
    assert ok and oracle.compress(ret) == oracle.msm_fr(pts, frs, n)


def test_fr_fft_golden(gpu, oracle, golden):
    for c in golden["fr_fft"]:
        n = c["n"]
        vals = _frs(oracle, c["seed"], n)
        if c["mode"] in ("fwd", "inv"):
            ok, out = gpu.fr_fft(vals, n, c["mode"] == "inv")
        else:
            d = gpu.fr_fft_domain_init(n)[1]
            ok, out = gpu.fr_fft_with_domain(vals, n, d, n + 2, c["mode"] == "dinv")
        assert ok and hashlib.sha256(out).hexdigest() == c["sha256"], (n, c["mode"])


def test_fr_fft_large_round_trip_and_rejections(gpu, oracle):
    n = 1 << 20
    import numpy as np
    vals = np.random.default_rng(3).integers(0, 1 << 62, size=(n, 4), dtype=np.uint64).tobytes()  # < r
    ok, f = gpu.fr_fft(vals, n, False)
    ok2, b = gpu.fr_fft(f, n, True)
    assert ok and ok2 and b == vals
    d = gpu.fr_fft_domain_init(64)[1]
    v = _frs(oracle, 70, 64)
    bad = bytearray(d)
    bad[-1] ^= 1
    assert gpu.fr_fft_with_domain(v, 64, bytes(bad), 66, False) == (False, v)
    assert gpu.fr_fft_with_domain(v, 64, d, 65, False) == (False, v)
    assert gpu.fr_fft(v[:32 * 3], 3, False) == (False, v[:32 * 3])
    # arbitrary domain values follow the same schedule and root indexing
    dd = bytearray(d)
    for i in range(1, 64):
        dd[32 * i:32 * i + 32] = oracle.fr_to_mont((5 + 3 * i).to_bytes(32, "little"))
    for inv in (False, True):
        assert gpu.fr_fft_with_domain(v, 64, bytes(dd), 66, inv) == oracle.fr_fft_with_domain(v, 64, bytes(dd), 66, inv)
