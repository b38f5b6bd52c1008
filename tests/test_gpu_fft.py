"""GPU parity for the G1 FFT entry points through the C ABI: every element's
96-byte serialization against the reference's golden vectors, round trips,
FFT-in-the-exponent, domain bytes, and the reference's rejection cases
(values untouched)."""
import hashlib

import pytest

pytestmark = pytest.mark.gpu


def _run(gpu, oracle, c, jac, n):
    mode = c["mode"]
    dl = n + 2
    ok_d, d = gpu.fr_fft_domain_init(n)
    assert ok_d
    if mode == "fwd":
        return gpu.p1_fft(jac, n, False)
    if mode == "inv":
        return gpu.p1_fft(jac, n, True)
    if mode == "dfwd":
        return gpu.p1_fft_with_domain(jac, n, d, dl, False)
    if mode == "dinv":
        return gpu.p1_fft_with_domain(jac, n, d, dl, True)
    return gpu.p1_ifft_unscaled_with_domain(jac, n, d, dl)


def test_fft_golden(gpu, oracle, golden):
    for c in golden["fft"]:
        n = c["n"]
        aff = oracle.gen_points(c["seed"], n)
        jac = oracle.jacobian_randomize(c["seed"], n, aff)
        ok, out = _run(gpu, oracle, c, jac, n)
        assert ok, c
        ser = b"".join(oracle.serialize(out[144 * i:144 * i + 144]) for i in range(n))
        assert hashlib.sha256(ser).hexdigest() == c["sha256"], (n, c["mode"])


def test_domain_init_matches_golden(gpu, golden):
    for c in golden["domain"]:
        ok, d = gpu.fr_fft_domain_init(c["n"])
        assert ok
        assert hashlib.sha256(d).hexdigest() == c["sha256"], c["n"]


def test_fft_round_trip(gpu, oracle):
    n = 1 << 12
    aff = oracle.gen_points(71, n)
    jac = oracle.jacobian_randomize(71, n, aff)
    ok, d = gpu.fr_fft_domain_init(n)
    ok1, f = gpu.p1_fft_with_domain(jac, n, d, n + 2, False)
    ok2, b = gpu.p1_fft_with_domain(f, n, d, n + 2, True)
    assert ok and ok1 and ok2
    for i in range(n):
        assert oracle.compress(b[144 * i:144 * i + 144]) == oracle.compress(jac[144 * i:144 * i + 144])


def test_fft_in_the_exponent(gpu, oracle):
    n = 16
    G = oracle.generator()
    vals, frs = b"", b""
    for i in range(n):
        k = (7 * i + 1).to_bytes(32, "little")
        vals += oracle.mult(G, k, 256)
        frs += oracle.fr_to_mont(k)
    ok, fx = gpu.p1_fft(vals, n, False)
    ok2, ff = oracle.fr_fft(frs, n, False)
    assert ok and ok2
    for i in range(n):
        k = oracle.fr_from_mont(ff[32 * i:32 * i + 32])
        assert oracle.compress(fx[144 * i:144 * i + 144]) == oracle.compress(oracle.mult(G, k, 256))


def test_fft_rejections_leave_values(gpu, oracle):
    n = 4
    jac = oracle.jacobian_randomize(5, n, oracle.gen_points(5, n))
    ok, d = gpu.fr_fft_domain_init(n)
    assert ok
    ok, out = gpu.p1_fft(jac[:3 * 144], 3, False)
    assert not ok and out == jac[:3 * 144]
    bad = bytearray(d)
    bad[-1] ^= 1
    ok, out = gpu.p1_fft_with_domain(jac, n, bytes(bad), n + 2, False)
    assert not ok and out == jac
    ok, out = gpu.p1_fft_with_domain(jac, n, d, n + 1, True)
    assert not ok and out == jac
    ok, out = gpu.p1_ifft_unscaled_with_domain(jac, n, d, n + 3)
    assert not ok and out == jac
    ok, out = gpu.p1_fft_with_domain(jac, n, None, n + 2, False)
    assert not ok and out == jac
    ok, _ = gpu.fr_fft_domain_init(3)
    assert not ok
    ok, _ = gpu.fr_fft_domain_init(4, 5)
    assert not ok


def test_fft_matches_oracle_arbitrary_domain_values(gpu, oracle):
    """A domain whose roots are not powers of one root (only the tag is
    checked): the butterfly schedule and root indexing must still match."""
    n = 8
    jac = oracle.jacobian_randomize(6, n, oracle.gen_points(6, n))
    d = bytearray(oracle.domain(n))
    for i in range(1, n):
        d[32 * i:32 * i + 32] = oracle.fr_to_mont((1000 + 17 * i).to_bytes(32, "little"))
    d = bytes(d)
    for inv in (False, True):
        ok, g = gpu.p1_fft_with_domain(jac, n, d, n + 2, inv)
        ok2, o = oracle.p1_fft_with_domain(jac, n, d, n + 2, inv)
        assert ok and ok2
        for i in range(n):
            assert oracle.serialize(g[144 * i:144 * i + 144]) == oracle.serialize(o[144 * i:144 * i + 144])


def test_fft_batch_matches_golden(gpu, oracle, golden):
    """Every golden FFT case (sizes 1..4096, all five modes) in ONE batch."""
    vals, ns, doms, modes, cases = [], [], [], [], []
    mode_of = {"dfwd": 0, "dinv": 1, "dunscaled": 2}
    for c in golden["fft"]:
        if c["mode"] not in mode_of:
            continue
        n = c["n"]
        aff = oracle.gen_points(c["seed"], n)
        vals.append(oracle.jacobian_randomize(c["seed"], n, aff))
        ns.append(n)
        doms.append(gpu.fr_fft_domain_init(n)[1])
        modes.append(mode_of[c["mode"]])
        cases.append(c)
    rc, outs = gpu.p1_fft_batch(vals, ns, doms, modes)
    assert rc == 0
    for c, out in zip(cases, outs):
        n = c["n"]
        ser = b"".join(oracle.serialize(out[144 * i:144 * i + 144]) for i in range(n))
        assert hashlib.sha256(ser).hexdigest() == c["sha256"], (n, c["mode"])


def test_fft_batch_large_lane_per_butterfly(gpu, oracle, golden):
    """The golden 4096-point cases, six copies each, in one batch: every stage
    launch holds more butterflies than one wave fits at four lanes each, so
    the stages and the inverse scale run one lane per butterfly (smaller
    launches, as in the tests above, use quad point operations)."""
    mode_of = {"dfwd": 0, "dinv": 1, "dunscaled": 2}
    big = [c for c in golden["fft"] if c["mode"] in mode_of and c["n"] == 4096]
    assert big
    vals, ns, doms, modes, cases = [], [], [], [], []
    d = gpu.fr_fft_domain_init(4096)[1]
    for c in big:
        v = oracle.jacobian_randomize(c["seed"], 4096, oracle.gen_points(c["seed"], 4096))
        for _ in range(6):
            vals.append(v)
            ns.append(4096)
            doms.append(d)
            modes.append(mode_of[c["mode"]])
            cases.append(c)
    assert len(cases) * 2048 > 9728          # butterflies per stage launch; quads fit at most 9728 on a GB300
    rc, outs = gpu.p1_fft_batch(vals, ns, doms, modes)
    assert rc == 0
    for c, out in zip(cases, outs):
        ser = b"".join(oracle.serialize(out[144 * i:144 * i + 144]) for i in range(4096))
        assert hashlib.sha256(ser).hexdigest() == c["sha256"], c["mode"]


def test_fft_round_trip_2_16(gpu, oracle, synth):
    """2^16 points (32768 butterflies per stage, one lane each): the inverse
    of the forward transform is the identity."""
    n = 1 << 16
    aff = gpu.points_from_scalars(synth.point_scalars(72, n), n)
    jac = oracle.jacobian_randomize(72, n, aff)
    ok, d = gpu.fr_fft_domain_init(n)
    ok1, f = gpu.p1_fft_with_domain(jac, n, d, n + 2, False)
    ok2, b = gpu.p1_fft_with_domain(f, n, d, n + 2, True)
    assert ok and ok1 and ok2
    assert f != jac
    for i in range(0, n, 7):
        assert oracle.compress(b[144 * i:144 * i + 144]) == oracle.compress(jac[144 * i:144 * i + 144]), i


def _padded(oracle, seed, n, xn):
    jac = bytearray(oracle.jacobian_randomize(seed, n, oracle.gen_points(seed, n)))
    jac[144 * xn:] = bytes(144 * (n - xn))
    return bytes(jac)


def test_fft_truncated_prefix_matches_golden(gpu, oracle, golden):
    """catmsm_p1_fft_truncated_prefix against the reference template's own
    outputs (golden fft_truncated: n = 32, 1024, 4096, xn from 1 to n, and
    n = 2^16 with xn = 8192, where a level of half-active groups runs on one
    root per warp)."""
    cases = golden["fft_truncated"]
    assert len(cases) >= 20
    base = {}
    for c in cases:
        n, xn = c["n"], c["xn"]
        if (c["seed"], n) not in base:
            base[(c["seed"], n)] = oracle.jacobian_randomize(c["seed"], n, oracle.gen_points(c["seed"], n))
        jac = base[(c["seed"], n)][:144 * xn] + bytes(144 * (n - xn))
        ok, tr = gpu.p1_fft_truncated_prefix(jac, n, xn, gpu.fr_fft_domain_init(n)[1], n + 2)
        assert ok
        ser = b"".join(oracle.serialize(tr[144 * i:144 * i + 144]) for i in range(n))
        assert hashlib.sha256(ser).hexdigest() == c["sha256"], (n, xn)


def test_fft_truncated_prefix_matches_oracle(gpu, oracle):
    """catmsm_p1_fft_truncated_prefix against the oracle's restatement of the
    reference's truncated-prefix plan (and so against the full transform),
    bit for bit, over the reference test's xn and around powers of two."""
    for n, xns in ((32, (1, 5, 13, 24, 32)), (1024, (1, 2, 3, 100, 511, 512, 513, 1000, 1024))):
        d = oracle.domain(n)
        for xn in xns:
            jac = _padded(oracle, 300 + xn, n, xn)
            ok, got = gpu.p1_fft_truncated_prefix(jac, n, xn, d, n + 2)
            ok2, exp = oracle.p1_fft_truncated_prefix(jac, n, xn, d, n + 2)
            assert ok and ok2
            for i in range(n):
                assert oracle.serialize(got[144 * i:144 * i + 144]) == oracle.serialize(exp[144 * i:144 * i + 144]), (n, xn, i)


@pytest.mark.parametrize("xn", [5000, 8192])
def test_fft_truncated_prefix_large_equals_full(gpu, oracle, synth, xn):
    """n = 2^16: the early stages run only the active groups (quads while they
    fit one wave, one lane per butterfly after); the outputs equal the full
    forward transform of the same input.  xn = 8192: at the second level 8192
    of 16384 groups are active (a multiple of 32, too many butterflies for
    quads), so the lanes of a warp share one root over bit-reversed groups,
    where the full transform maps its groups in order."""
    n = 1 << 16
    aff = gpu.points_from_scalars(synth.point_scalars(73, xn), xn)
    jac = oracle.jacobian_randomize(73, xn, aff) + bytes(144 * (n - xn))
    d = gpu.fr_fft_domain_init(n)[1]
    ok, tr = gpu.p1_fft_truncated_prefix(jac, n, xn, d, n + 2)
    ok2, full = gpu.p1_fft_with_domain(jac, n, d, n + 2, False)
    assert ok and ok2
    assert tr == full


def test_fft_truncated_prefix_rejects_before_writing(gpu, oracle):
    n = 16
    d = oracle.domain(n)
    jac = _padded(oracle, 333, n, 6)
    for xn, dl in ((0, n + 2), (n + 1, n + 2), (6, n + 1)):
        ok, out = gpu.p1_fft_truncated_prefix(jac, n, xn, d, dl)
        assert not ok and out == jac
    # a non-identity element past xn
    ok, out = gpu.p1_fft_truncated_prefix(jac, n, 5, d, n + 2)
    assert not ok and out == jac
    ok, out = gpu.p1_fft_truncated_prefix(jac, 12, 6, d, n + 2)    # not a power of two
    assert not ok and out == jac
    assert gpu.p1_fft_truncated_prefix(jac, n, 6, d, n + 2)[0]


def test_fft_batch_rejects_before_writing(gpu, oracle):
    n = 8
    jac = oracle.jacobian_randomize(9, n, oracle.gen_points(9, n))
    d = gpu.fr_fft_domain_init(n)[1]
    bad = bytearray(d)
    bad[-1] ^= 1
    rc, outs = gpu.p1_fft_batch([jac, jac], [n, n], [d, bytes(bad)], [0, 0])
    assert rc != 0 and outs == [jac, jac]
    rc, outs = gpu.p1_fft_batch([jac], [n], [d], [3])
    assert rc != 0 and outs == [jac]


def test_fft_batch_workload_golden(gpu, oracle, golden, synth):
    """The batched-FFT workload's inputs (the first n points of the seeded
    2^16-point set as Jacobian with z = 1, prepared domains) for n = 2^10 ..
    2^16, forward and inverse in ONE batch, against the reference's
    blst_p1_fft_with_domain output (sha256 of every element's serialization)."""
    g = golden["bench_fft"]
    big = 1 << 16
    aff = gpu.points_from_scalars(synth.point_scalars(g["seed"], big), big)
    P = 0x1a0111ea397fe69a4b1ba7b6434bacd764774b84f38512bf6730d2a0f6b0f6241eabfffeb153ffffb9feffffffffaaab
    one = ((1 << 384) % P).to_bytes(48, "little")
    cases = g["cases"]
    vals, ns, doms, modes = [], [], [], []
    for c in cases:
        n = c["n"]
        vals.append(b"".join(aff[96 * i:96 * i + 96] + one for i in range(n)))
        ns.append(n)
        ok, d = gpu.fr_fft_domain_init(n)
        assert ok
        doms.append(d)
        modes.append(1 if c["mode"] == "dinv" else 0)
    rc, outs = gpu.p1_fft_batch(vals, ns, doms, modes)
    assert rc == 0
    for c, n, out in zip(cases, ns, outs):
        ser = b"".join(oracle.serialize(out[144 * i:144 * i + 144]) for i in range(n))
        assert hashlib.sha256(ser).hexdigest() == c["sha256"], (n, c["mode"])
