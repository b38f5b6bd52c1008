"""The reference has no global mutable state, so concurrent calls with
disjoint buffers are safe (bindings/blst_fft.h:34-36, README).  Here every
calling thread gets its own stream and workspaces: MSMs, FFTs and Fr MSMs
issued from several host threads at once each equal the oracle's result for
the same inputs (ctypes releases the GIL for the duration of each call).
A thread's workspaces are released when the thread exits, so MSMs run from
short-lived threads, and the worker threads of a server that is destroyed,
leave no device memory behind (with a leak, each 2^18-point MSM thread kept
~0.6 GB and a 2^20-point one ~4.5 GB)."""
import threading

import pytest

pytestmark = pytest.mark.gpu


def test_concurrent_calls_from_threads(gpu, oracle, synth):
    jobs = []
    for t in range(6):
        n = 3000 + 517 * t
        pts = oracle.gen_points(700 + t, n)
        sc = synth.scalars(800 + t, n, 0)
        jobs.append(("msm", n, pts, sc, oracle.msm(pts, sc, n, 255)))
    for t in range(2):
        n = 64
        aff = oracle.gen_points(900 + t, n)
        jac = oracle.jacobian_randomize(900 + t, n, aff)
        ok, exp = oracle.p1_fft(jac, n, False)
        assert ok
        jobs.append(("fft", n, jac, None, exp))
    frs_n = 2000
    pts = oracle.gen_points(950, frs_n)
    frs = b"".join(oracle.fr_to_mont(oracle.gen_scalars(951, frs_n, 0)[32 * i:32 * i + 32]) for i in range(frs_n))
    jobs.append(("fr", frs_n, pts, frs, oracle.msm_fr(pts, frs, frs_n)))

    results = [None] * len(jobs)
    errors = []

    def work(i):
        try:
            kind, n, a, b, _ = jobs[i]
            for _ in range(3):                     # repeated calls on the thread's own context
                if kind == "msm":
                    results[i] = oracle.compress(gpu.p1s_mult_pippenger(a, b, n, 255))
                elif kind == "fr":
                    ok, ret = gpu.p1s_mult_pippenger_fr(a, b, n)
                    assert ok
                    results[i] = oracle.compress(ret)
                else:
                    ok, out = gpu.p1_fft(a, n, False)
                    assert ok
                    results[i] = out
        except Exception as e:  # surfaced below
            errors.append((i, repr(e)))

    threads = [threading.Thread(target=work, args=(i,)) for i in range(len(jobs))]
    for th in threads:
        th.start()
    for th in threads:
        th.join()
    assert not errors, errors
    for i, (kind, n, a, b, exp) in enumerate(jobs):
        if kind == "fft":
            for j in range(n):
                assert oracle.compress(results[i][144 * j:144 * j + 144]) == oracle.compress(exp[144 * j:144 * j + 144])
        else:
            assert results[i] == exp, (kind, n)


SLACK = 96 << 20   # device-wide free memory may move by a few MB (other allocations, the CUDA runtime)


def _free():
    import torch
    torch.cuda.synchronize()
    return torch.cuda.mem_get_info()[0]


def _released(free0, limit_s=5.0):
    """Whether free device memory comes back to within SLACK of free0.  A
    Python thread's join returns when its Python code is done; the OS thread
    runs its C++ thread-exit destructors (the library's release) after that,
    so the check polls for a few seconds."""
    import time
    t_end = time.time() + limit_s
    while True:
        if _free() >= free0 - SLACK:
            return True
        if time.time() > t_end:
            return False
        time.sleep(0.05)


def test_thread_contexts_released(gpu, synth):
    n = 1 << 18
    pts = gpu.points_from_scalars(synth.point_scalars(61, n), n)
    sc = synth.scalars(62, n, 0)
    exp = gpu.p1s_mult_pippenger(pts, sc, n, 255)        # this thread's context (kept)
    free0 = _free()
    for _ in range(3):
        out = []
        t = threading.Thread(target=lambda: out.append(gpu.p1s_mult_pippenger(pts, sc, n, 255)))
        t.start()
        t.join()
        assert out == [exp]
        assert _released(free0)


def test_server_workers_release_memory(gpu, oracle, synth):
    n = 1 << 20
    pts = gpu.points_from_scalars(synth.point_scalars(63, n), n)
    basis = gpu.Basis(pts, n, 10)
    sc = synth.scalars(64, n, 0)
    exp = gpu.p1s_mult_pippenger(pts, sc, n, 255)
    try:
        free0 = _free()
        for _ in range(2):
            server = gpu.Server(basis, workers=2, hbm_budget=16 << 30)
            try:
                rc, out = server.wait(server.submit_msm(sc, n))[:2]
                assert rc == 0 and oracle.compress(out) == oracle.compress(exp)
            finally:
                server.close()
            assert _released(free0)
    finally:
        basis.close()
