"""The MSM entry point that allocates nothing (catmsm_p1s_mult_pippenger_noalloc).

It exists for callers that must not allocate device memory at call time, for
instance because another framework already holds the GPU's memory in its own
pool, or because cudaMalloc/cudaFree would stall a latency-critical path.  It
works inside one fixed scratch array owned by the library, so these tests
check that its results equal the regular blst_p1s_mult_pippenger entry point
byte for byte on two calls in a row (the array keeps the previous call's
contents, which must not leak into the next result), that they equal the
reference's own output where a golden vector exists, that device memory use
does not change across the calls, and that oversized calls are refused.

This file is collected last so that, if it fails, a run stopping at the
first failure has already run every other test.
"""
import ctypes as C

import pytest

pytestmark = pytest.mark.gpu

MAX_POINTS = 4096
TOO_LARGE = -2
MIB = 1 << 20


def _bind(gpu):
    L = gpu.load()
    L.catmsm_p1s_mult_pippenger_noalloc.restype = C.c_int
    L.catmsm_p1s_mult_pippenger_noalloc.argtypes = [C.c_void_p, C.c_char_p, C.c_size_t, C.c_char_p, C.c_size_t]
    return L


def _noalloc(L, pts, sc, n, nbits):
    ret = (C.c_char * 144)()
    rc = L.catmsm_p1s_mult_pippenger_noalloc(ret, pts, n, sc, nbits)
    return rc, bytes(ret)


def _inputs(oracle, synth, n, nbits, kind, seed):
    pts = oracle.gen_points(seed, n)
    sc = synth.scalars(seed + 1, n, kind)
    nb = (nbits + 7) // 8
    if nb != 32:
        sc = b"".join(sc[32 * i:32 * i + nb] for i in range(n))
    return pts, sc, n, nbits


def test_noalloc_matches_regular_entry_point(gpu, oracle, synth):
    import torch
    L = _bind(gpu)
    inputs = [_inputs(oracle, synth, MAX_POINTS, 255, 0, 501), _inputs(oracle, synth, 777, 64, 1, 502)]
    # The first call on a device does the one-time set-up, and the CUDA runtime
    # loads the library's module (which carries the fixed scratch array) on
    # first use.  Device memory must then stay constant across further calls.
    rc, _ = _noalloc(L, *inputs[1])
    assert rc == 0
    torch.cuda.synchronize()
    free_before = torch.cuda.mem_get_info()[0]
    got = [_noalloc(L, *x) for x in inputs]          # two calls in a row
    torch.cuda.synchronize()
    free_after = torch.cuda.mem_get_info()[0]
    # mem_get_info is the free memory of the whole device, which another
    # context could change; any cudaMalloc of this process would take at least
    # one 2 MiB allocation granule, so a change below 1 MiB is not one of ours
    assert abs(free_after - free_before) < MIB
    for (rc, out), (pts, sc, n, nbits) in zip(got, inputs):
        assert rc == 0
        assert out == gpu.p1s_mult_pippenger(pts, sc, n, nbits)
    # the same inputs again after the other call: identical bytes
    rc, again = _noalloc(L, *inputs[0])
    assert rc == 0 and again == got[0][1]


def test_noalloc_reference_golden_and_limits(gpu, oracle, synth, golden):
    """The plain n = 4096 workload (seed 1) against the reference's own bytes,
    then the largest window count (nbits = 256: 33 windows), a single point,
    and 4096 equal scalars (every entry of a window in one bucket, whose
    chunk carries take the block join), each checked against the regular
    entry point and the oracle, back to back."""
    L = _bind(gpu)
    c = next(c for c in golden["msm"] if c["seed"] == 1 and c["n"] == MAX_POINTS)
    pts = oracle.gen_points(1, MAX_POINTS)
    sc = synth.scalars(1001, MAX_POINTS, 0)
    rc, out = _noalloc(L, pts, sc, MAX_POINTS, 255)
    assert rc == 0 and oracle.compress(out).hex() == c["compressed"]
    same = synth.scalars(511, 1, 0) * MAX_POINTS
    cases = [_inputs(oracle, synth, MAX_POINTS, 256, 0, 503), _inputs(oracle, synth, 1, 255, 0, 505),
             (oracle.gen_points(507, MAX_POINTS), same, MAX_POINTS, 255)]
    for pts, sc, n, nbits in cases:
        rc, out = _noalloc(L, pts, sc, n, nbits)
        assert rc == 0, (n, nbits)
        assert out == gpu.p1s_mult_pippenger(pts, sc, n, nbits), (n, nbits)
        assert oracle.compress(out) == oracle.msm(pts, sc, n, nbits), (n, nbits)


def test_noalloc_rejects_oversized_calls(gpu, oracle, synth):
    L = _bind(gpu)
    n = MAX_POINTS + 1
    pts = bytes(96 * n)
    sc = bytes(32 * n)
    rc, out = _noalloc(L, pts, sc, n, 255)
    assert rc == TOO_LARGE and out == bytes(144)
    rc, out = _noalloc(L, pts[:96], sc[:33], 1, 257)
    assert rc == TOO_LARGE and out == bytes(144)
