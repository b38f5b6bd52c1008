"""GPU parity for the fixed-table (wbits) MSM drop-ins against the reference's
blst_p1s_mult_wbits_precompute / blst_p1s_mult_wbits (golden tables and
results generated by the reference, tests/golden/make_golden.py): the table
bytes identical, the MSM the same group element, the reference's descriptor,
in-place and fail-closed behaviour, and a 2^15-point table checked against
the oracle on sampled rows."""
import ctypes as C
import hashlib
import random

import pytest

pytestmark = pytest.mark.gpu

INF = bytes([0xC0]) + bytes(47)


def _inputs(oracle, c):
    pts = oracle.gen_points(c["seed"], c["n"])
    if c["dup"]:
        pts = oracle.duplicate_points(c["seed"], c["n"], pts)
    sc = oracle.gen_scalars(c["seed"] + 1000, c["n"], c["kind"])
    nb = (c["nbits"] + 7) // 8
    if nb != 32:
        sc = b"".join(sc[32 * i:32 * i + nb] for i in range(c["n"]))
    if c["inf"]:
        k = c["seed"] % c["n"]
        pts = pts[:96 * k] + bytes(96) + pts[96 * (k + 1):]
    return pts, sc


def test_wbits_table_and_msm_match_reference(gpu, golden, oracle):
    cases = golden["wbits"]
    assert len(cases) >= 12
    for c in cases:
        pts, sc = _inputs(oracle, c)
        n, w = c["n"], c["wbits"]
        table = gpu.p1s_mult_wbits_precompute(pts, n, w)
        assert len(table) == 96 * n << (w - 1)
        assert hashlib.sha256(table).hexdigest() == c["table_sha256"], (c["seed"], n, w)
        res = gpu.p1s_mult_wbits(table, w, n, sc, c["nbits"])
        assert oracle.compress(res) == bytes.fromhex(c["compressed"]), (c["seed"], n, w)


def test_wbits_precompute_in_place_and_descriptors(gpu, oracle):
    """Packed points in the final n entries of the table (the one overlap the
    reference allows), and an explicit shuffled descriptor array."""
    n, w = 37, 5
    m = 1 << (w - 1)
    pts = oracle.gen_points(501, n)
    exp = gpu.p1s_mult_wbits_precompute(pts, n, w)
    table = bytearray(96 * n * m)
    table[-96 * n:] = pts
    tb = (C.c_char * len(table)).from_buffer(table)
    tail = C.addressof(tb) + len(table) - 96 * n
    gpu.p1s_mult_wbits_precompute(None, n, w, table=table, point_ptrs=[tail, None])
    assert bytes(table) == exp
    order = list(range(n))
    random.Random(5).shuffle(order)
    pbuf = bytearray(pts)
    pb = (C.c_char * len(pbuf)).from_buffer(pbuf)
    ptrs = [C.addressof(pb) + 96 * i for i in order]
    got = gpu.p1s_mult_wbits_precompute(None, n, w, point_ptrs=ptrs)
    shuffled = b"".join(pts[96 * i:96 * i + 96] for i in order)
    assert got == gpu.p1s_mult_wbits_precompute(shuffled, n, w)
    # mixed descriptors: two heads, then NULL continuation from the second
    got = gpu.p1s_mult_wbits_precompute(None, n, w, point_ptrs=[C.addressof(pb), C.addressof(pb) + 96, None])
    assert got == exp


def test_wbits_msm_scalar_descriptors(gpu, oracle):
    n, w = 29, 6
    pts = oracle.gen_points(502, n)
    sc = bytearray(oracle.gen_scalars(503, n, 0))
    table = gpu.p1s_mult_wbits_precompute(pts, n, w)
    sb = (C.c_char * len(sc)).from_buffer(sc)
    order = list(range(n))
    random.Random(6).shuffle(order)
    ptrs = [C.addressof(sb) + 32 * i for i in order]
    tshuf = gpu.p1s_mult_wbits_precompute(b"".join(pts[96 * i:96 * i + 96] for i in order), n, w)
    got = gpu.p1s_mult_wbits(tshuf, w, n, None, 255, scalar_ptrs=ptrs)
    assert oracle.compress(got) == oracle.msm(pts, bytes(sc), n, 255)
    assert oracle.compress(gpu.p1s_mult_wbits(table, w, n, bytes(sc), 255)) == oracle.msm(pts, bytes(sc), n, 255)


def test_wbits_fail_closed(gpu, oracle):
    n, w = 8, 3
    pts = oracle.gen_points(504, n)
    sc = oracle.gen_scalars(505, n, 0)
    table = gpu.p1s_mult_wbits_precompute(pts, n, w)
    # invalid wbits or a NULL head: the caller's table is untouched
    for bad_w, ptrs in ((1, None), (15, None), (w, [None, None])):
        junk = bytearray(b"\x5a" * len(table))
        gpu.p1s_mult_wbits_precompute(pts, n, bad_w, table=junk, point_ptrs=ptrs)
        assert bytes(junk) == b"\x5a" * len(table)
    # empty input, zero bits, and every invalid argument -> infinity
    assert oracle.compress(gpu.p1s_mult_wbits(table, w, 0, sc, 255)) == INF
    assert oracle.compress(gpu.p1s_mult_wbits(table, w, n, sc, 0)) == INF
    assert oracle.compress(gpu.p1s_mult_wbits(table, w, n, sc, 257)) == INF
    assert oracle.compress(gpu.p1s_mult_wbits(table, 15, n, sc, 255)) == INF
    assert oracle.compress(gpu.p1s_mult_wbits(table, 1, n, sc, 255)) == INF
    assert oracle.compress(gpu.p1s_mult_wbits(table, w, n, sc, 255, scratch=False)) == INF
    assert oracle.compress(gpu.p1s_mult_wbits(None, w, n, sc, 255)) == INF
    assert oracle.compress(gpu.p1s_mult_wbits(table, w, n, None, 255, scalar_ptrs=[None, None])) == INF
    # and the call after a rejected one is unaffected
    assert oracle.compress(gpu.p1s_mult_wbits(table, w, n, sc, 255)) == oracle.msm(pts, sc, n, 255)


def test_wbits_large_table_sampled_rows(gpu, oracle, synth):
    """2^15 points, wbits 6: sampled rows equal the oracle's rows bit for bit,
    every row's first entry is its point, and the table MSM equals the GPU
    Pippenger MSM over the same points and scalars."""
    n, w = 1 << 15, 6
    m = 1 << (w - 1)
    pts = gpu.points_from_scalars(synth.point_scalars(91, n), n)
    table = gpu.p1s_mult_wbits_precompute(pts, n, w)
    for i in random.Random(7).sample(range(n), 24):
        row = table[96 * m * i:96 * m * (i + 1)]
        assert row == oracle.wbits_table(pts[96 * i:96 * i + 96], 1, w), i
    heads = b"".join(table[96 * m * i:96 * m * i + 96] for i in range(n))
    assert heads == pts
    sc = synth.scalars(92, n, 0)
    a = gpu.p1s_mult_wbits(table, w, n, sc, 255)
    b = gpu.p1s_mult_pippenger(pts, sc, n, 255)
    assert oracle.compress(a) == oracle.compress(b)
