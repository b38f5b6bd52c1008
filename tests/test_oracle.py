"""CPU checks: the oracle restatement against the reference's golden vectors,
the seeded generators against each other, and (where the reference tree was
present at build time) the oracle against the reference library itself."""
import ctypes as C
import hashlib
import os

import pytest

import oracle as om


def _msm_inputs(o, c):
    n, nbits = c["n"], c["nbits"]
    pts = o.gen_points(c["seed"], n)
    if c["dup"]:
        pts = o.duplicate_points(c["seed"], n, pts)
    sc = o.gen_scalars(c["seed"] + 1000, n, c["kind"])
    nb = (nbits + 7) // 8
    if nb != 32:
        sc = b"".join(sc[32 * i:32 * i + nb] for i in range(n))
    return pts, sc


def test_oracle_msm_matches_golden(golden, oracle):
    cases = [c for c in golden["msm"] if c["n"] <= (1 << 16)]
    assert len(cases) >= 18
    for c in cases:
        pts, sc = _msm_inputs(oracle, c)
        got = oracle.msm(pts, sc, c["n"], c["nbits"])
        assert got.hex() == c["compressed"], c


def test_oracle_fft_matches_golden(golden, oracle):
    for c in golden["fft"]:
        n = c["n"]
        if n > 256:
            continue
        aff = oracle.gen_points(c["seed"], n)
        jac = oracle.jacobian_randomize(c["seed"], n, aff)
        d = oracle.domain(n)
        mode = c["mode"]
        if mode == "fwd":
            ok, out = oracle.p1_fft(jac, n, False)
        elif mode == "inv":
            ok, out = oracle.p1_fft(jac, n, True)
        elif mode == "dfwd":
            ok, out = oracle.p1_fft_with_domain(jac, n, d, n + 2, False)
        elif mode == "dinv":
            ok, out = oracle.p1_fft_with_domain(jac, n, d, n + 2, True)
        else:
            ok, out = oracle.p1_ifft_unscaled_with_domain(jac, n, d, n + 2)
        assert ok
        ser = b"".join(oracle.serialize(out[144 * i:144 * i + 144]) for i in range(n))
        assert hashlib.sha256(ser).hexdigest() == c["sha256"], (n, mode)


def test_oracle_domains_match_golden(golden, oracle):
    for c in golden["domain"]:
        assert hashlib.sha256(oracle.domain(c["n"])).hexdigest() == c["sha256"], c["n"]


def test_oracle_naive_and_windows_agree(oracle):
    n = 40
    pts = oracle.gen_points(101, n)
    sc = oracle.gen_scalars(102, n, 0)
    ref = oracle.msm_naive(pts, sc, n, 255)
    assert oracle.msm(pts, sc, n, 255) == ref
    for w in (1, 2, 3, 5, 8, 13):
        assert oracle.msm_window(pts, sc, n, 255, w) == ref


def test_oracle_fft_round_trip_and_exponent(oracle):
    """FFT-in-the-exponent: fft(i*G) == fr_fft(i)*G (reference test
    BindingHeader_tests.cpp:480-569), and inverse(forward(x)) == x."""
    n = 8
    G = oracle.generator()
    vals = b""
    frs = b""
    for i in range(n):
        k = (i + 3).to_bytes(32, "little")
        vals += oracle.mult(G, k, 256)
        frs += oracle.fr_to_mont(k)
    ok, fx = oracle.p1_fft(vals, n, False)
    assert ok
    ok, ff = oracle.fr_fft(frs, n, False)
    assert ok
    for i in range(n):
        k = oracle.fr_from_mont(ff[32 * i:32 * i + 32])
        assert oracle.compress(fx[144 * i:144 * i + 144]) == oracle.compress(oracle.mult(G, k, 256))
    ok, back = oracle.p1_fft(fx, n, True)
    assert ok
    for i in range(n):
        assert oracle.compress(back[144 * i:144 * i + 144]) == oracle.compress(vals[144 * i:144 * i + 144])


def test_oracle_rejects_bad_fft_inputs(oracle):
    jac = oracle.jacobian_randomize(5, 4, oracle.gen_points(5, 4))
    d = oracle.domain(4)
    ok, out = oracle.p1_fft(jac[:3 * 144], 3, False)
    assert not ok
    bad = bytearray(d)
    bad[-1] ^= 1
    ok, out = oracle.p1_fft_with_domain(jac, 4, bytes(bad), 6, False)
    assert not ok and out == jac
    ok, out = oracle.p1_fft_with_domain(jac, 4, d, 5, False)
    assert not ok and out == jac


def test_synth_matches_oracle_generator(oracle, synth):
    for kind in (0, 1, 2):
        for seed in (1, 7, 123456789):
            assert synth.scalars(seed, 777, kind) == oracle.gen_scalars(seed, 777, kind), (seed, kind)
    n = 500
    pts = oracle.gen_points(9, n)
    assert synth.point_scalars(9, n) == oracle.gen_scalars(9 ^ 0xA5A5A5A5, n, 0)
    dup = oracle.duplicate_points(9, n, pts)
    assert bytes(synth.apply_duplicates(bytearray(pts), 9, n)) == dup


@pytest.mark.skipif(not om.reference_available(), reason="reference library not built here")
def test_oracle_matches_reference_descriptor_arrays(oracle):
    """Non-contiguous descriptor arrays and the fail-closed cases, oracle vs
    the reference's own C ABI (reference tests C_api_tests.cpp:1517-1611)."""
    ref = om.Reference()
    n = 9
    pts = bytearray(oracle.gen_points(55, n))
    sc = bytearray(oracle.gen_scalars(56, n, 0))
    pb = (C.c_char * len(pts)).from_buffer(pts)
    sb = (C.c_char * len(sc)).from_buffer(sc)
    base_p, base_s = C.addressof(pb), C.addressof(sb)
    order = [3, 0, 5, 1, 8, 2, 7, 4, 6]
    pa = (C.c_void_p * n)(*[base_p + 96 * i for i in order])
    sa = (C.c_void_p * n)(*[base_s + 32 * i for i in order])
    scratch = (C.c_uint64 * 4096)()
    r1, r2 = bytearray(144), bytearray(144)
    oracle.L.oracle_p1s_mult_pippenger((C.c_char * 144).from_buffer(r1), pa, n, sa, 255, scratch)
    ref.L.blst_p1s_mult_pippenger((C.c_char * 144).from_buffer(r2), pa, n, sa, 255, scratch)
    assert oracle.compress(bytes(r1)) == ref.compress(bytes(r2))
    # mixed: two explicit heads then NULL continuation
    pa2 = (C.c_void_p * 3)(base_p, base_p + 96, None)
    sa2 = (C.c_void_p * 3)(base_s, base_s + 32, None)
    oracle.L.oracle_p1s_mult_pippenger((C.c_char * 144).from_buffer(r1), pa2, n, sa2, 255, scratch)
    ref.L.blst_p1s_mult_pippenger((C.c_char * 144).from_buffer(r2), pa2, n, sa2, 255, scratch)
    assert oracle.compress(bytes(r1)) == ref.compress(bytes(r2))
    # null scratch with n > 1 -> infinity in both
    oracle.L.oracle_p1s_mult_pippenger((C.c_char * 144).from_buffer(r1), pa, n, sa, 255, None)
    ref.L.blst_p1s_mult_pippenger((C.c_char * 144).from_buffer(r2), pa, n, sa, 255, None)
    assert oracle.compress(bytes(r1)) == ref.compress(bytes(r2)) == bytes([0xC0]) + bytes(47)


def _frs(oracle, seed, n):
    sc = oracle.gen_scalars(seed, n, 0)
    return b"".join(oracle.fr_to_mont(sc[32 * i:32 * i + 32]) for i in range(n))


def test_oracle_msm_fr_matches_golden(golden, oracle):
    for c in golden["msm_fr"]:
        n = c["n"]
        pts = oracle.gen_points(c["seed"], n)
        frs = _frs(oracle, c["seed"] + 1000, n)
        assert oracle.msm_fr(pts, frs, n).hex() == c["compressed"], n


def test_oracle_fr_fft_matches_golden(golden, oracle):
    for c in golden["fr_fft"]:
        n = c["n"]
        vals = _frs(oracle, c["seed"], n)
        d = oracle.domain(n)
        if c["mode"] in ("fwd", "inv"):
            ok, out = oracle.fr_fft(vals, n, c["mode"] == "inv")
        else:
            ok, out = oracle.fr_fft_with_domain(vals, n, d, n + 2, c["mode"] == "dinv")
        assert ok and hashlib.sha256(out).hexdigest() == c["sha256"], (n, c["mode"])


def _wbits_inputs(oracle, c):
    """Inputs of a golden wbits case: seeded points (duplicates, one point at
    infinity at index seed % n, as flagged) and packed scalars."""
    pts, sc = _msm_inputs(oracle, c)
    if c["inf"]:
        k = c["seed"] % c["n"]
        pts = pts[:96 * k] + bytes(96) + pts[96 * (k + 1):]
    return pts, sc


def test_oracle_wbits_matches_golden(golden, oracle):
    cases = golden["wbits"]
    assert len(cases) >= 12
    for c in cases:
        if c["n"] << (c["wbits"] - 1) > 40000:
            continue
        pts, sc = _wbits_inputs(oracle, c)
        table = oracle.wbits_table(pts, c["n"], c["wbits"])
        assert hashlib.sha256(table).hexdigest() == c["table_sha256"], c
        assert oracle.wbits_msm(table, c["wbits"], c["n"], sc, c["nbits"]).hex() == c["compressed"], c


@pytest.mark.skipif(not om.reference_available(), reason="reference library not built here")
def test_oracle_wbits_matches_reference_edge_cases(oracle):
    """Packed points in the table's tail, explicit descriptor arrays and the
    fail-closed cases, oracle vs the reference's own C ABI."""
    ref = om.Reference()
    n, w = 7, 4
    m = 1 << (w - 1)
    pts = oracle.gen_points(77, n)
    sc = oracle.gen_scalars(78, n, 0)
    exp = ref.wbits_table(pts, n, w)
    assert oracle.wbits_table(pts, n, w) == exp
    for lib in (oracle, ref):
        pre = getattr(lib.L, "oracle_p1s_mult_wbits_precompute" if lib is oracle else "blst_p1s_mult_wbits_precompute")
        table = bytearray(96 * n * m)
        table[-96 * n:] = pts                       # packed input in the tail
        tb = (C.c_char * len(table)).from_buffer(table)
        parr = (C.c_void_p * 2)(C.addressof(tb) + len(table) - 96 * n, None)
        pre(tb, w, parr, n)
        assert bytes(table) == exp
        # invalid wbits / NULL head: the table is left untouched
        for bad_w, head in ((1, True), (15, True), (4, False)):
            junk = bytearray(b"\x5a" * len(table))
            jb = (C.c_char * len(junk)).from_buffer(junk)
            parr = (C.c_void_p * 2)(C.addressof(tb) if head else None, None)
            pre(jb, bad_w, parr, n)
            assert bytes(junk) == b"\x5a" * len(table)
    # explicit scalar descriptors in shuffled order
    order = [4, 0, 6, 2, 1, 5, 3]
    sb = (C.c_char * len(sc)).from_buffer(bytearray(sc))
    sarr = (C.c_void_p * n)(*[C.addressof(sb) + 32 * i for i in order])
    pshuf = b"".join(pts[96 * i:96 * i + 96] for i in order)
    tshuf = ref.wbits_table(pshuf, n, w)
    tb2 = (C.c_char * len(tshuf)).from_buffer(bytearray(tshuf))
    scratch = (C.c_uint64 * 2048)()
    r1, r2 = bytearray(144), bytearray(144)
    oracle.L.oracle_p1s_mult_wbits((C.c_char * 144).from_buffer(r1), tb2, w, n, sarr, 255, scratch)
    ref.L.blst_p1s_mult_wbits((C.c_char * 144).from_buffer(r2), tb2, w, n, sarr, 255, scratch)
    assert oracle.compress(bytes(r1)) == ref.compress(bytes(r2)) == ref.msm(pts, sc, n, 255)
    # fail-closed: NULL scratch, wbits 15, nbits 257 -> infinity
    inf = bytes([0xC0]) + bytes(47)
    for args in ((w, 255, None), (15, 255, scratch), (w, 257, scratch)):
        oracle.L.oracle_p1s_mult_wbits((C.c_char * 144).from_buffer(r1), tb2, args[0], n, sarr, args[1], args[2])
        ref.L.blst_p1s_mult_wbits((C.c_char * 144).from_buffer(r2), tb2, args[0], n, sarr, args[1], args[2])
        assert oracle.compress(bytes(r1)) == ref.compress(bytes(r2)) == inf


def test_oracle_matches_fr_msm_variant_goldens(golden, oracle):
    """blst_p1s_mult_fr / blst_p1s_mult_batch_affine_fr outputs of the
    reference equal the oracle's MSM of the same Montgomery scalars."""
    for c in golden["msm_fr_variants"]["cases"]:
        n = c["n"]
        if n > 5000:
            continue
        pts = oracle.gen_points(c["seed"], n)
        if c["inf"]:
            k = c["seed"] % n
            pts = pts[:96 * k] + bytes(96) + pts[96 * (k + 1):]
        frs = _frs(oracle, c["seed"] + 1000, n)
        assert oracle.msm_fr(pts, frs, n).hex() == c["compressed"], (c["api"], n)


def test_oracle_tile_matches_golden(golden, oracle):
    """The oracle's restatement of blst_p1s_tile_pippenger against the
    reference's outputs (edge windows: bit0 = 0, top windows, window 1)."""
    cases = golden["tile"]
    assert len(cases) >= 12
    for c in cases:
        pts, sc = _msm_inputs(oracle, c)
        assert oracle.tile(pts, sc, c["n"], c["nbits"], c["bit0"], c["window"]).hex() == c["compressed"], c


def test_oracle_fft_truncated_prefix_matches_full(oracle):
    """The reference's TruncatedForwardPrefixMatchesFullG1 (test/Fft_tests.cpp:
    974-1006) on the oracle: m = 32, xn in {1, 5, 13, 24, 32}, inputs [xn, m)
    the identity; the truncated transform equals the full forward one."""
    m = 32
    d = oracle.domain(m)
    for xn in (1, 5, 13, 24, 32):
        jac = bytearray(oracle.jacobian_randomize(200 + xn, m, oracle.gen_points(200 + xn, m)))
        jac[144 * xn:] = bytes(144 * (m - xn))
        jac = bytes(jac)
        ok1, full = oracle.p1_fft_with_domain(jac, m, d, m + 2, False)
        ok2, tr = oracle.p1_fft_truncated_prefix(jac, m, xn, d, m + 2)
        assert ok1 and ok2
        for i in range(m):
            assert oracle.serialize(full[144 * i:144 * i + 144]) == oracle.serialize(tr[144 * i:144 * i + 144]), xn
    zero = bytes(144 * m)
    assert not oracle.p1_fft_truncated_prefix(zero, m, 0, d, m + 2)[0]
    assert not oracle.p1_fft_truncated_prefix(zero, m, m + 1, d, m + 2)[0]
    assert not oracle.p1_fft_truncated_prefix(zero, m, 4, d, m + 1)[0]


def test_oracle_fft_truncated_prefix_matches_golden(golden, oracle):
    """The oracle's restatement of the truncated-prefix plan against the
    reference template's outputs (golden fft_truncated, n <= 1024 here; the
    GPU test covers every case)."""
    cases = [c for c in golden["fft_truncated"] if c["n"] <= 1024]
    assert len(cases) >= 14
    base = {}
    for c in cases:
        n, xn = c["n"], c["xn"]
        if (c["seed"], n) not in base:
            base[(c["seed"], n)] = oracle.jacobian_randomize(c["seed"], n, oracle.gen_points(c["seed"], n))
        jac = base[(c["seed"], n)][:144 * xn] + bytes(144 * (n - xn))
        ok, tr = oracle.p1_fft_truncated_prefix(jac, n, xn, oracle.domain(n), n + 2)
        assert ok
        ser = b"".join(oracle.serialize(tr[144 * i:144 * i + 144]) for i in range(n))
        assert hashlib.sha256(ser).hexdigest() == c["sha256"], (n, xn)

