"""The reference has no global mutable state, so concurrent calls with
disjoint buffers are safe (bindings/blst_fft.h:34-36, README).  Here every
calling thread gets its own stream and workspaces: MSMs, FFTs and Fr MSMs
issued from several host threads at once each equal the oracle's result for
the same inputs (ctypes releases the GIL for the duration of each call)."""
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
