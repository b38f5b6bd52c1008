"""Serving engine: a mix of MSM and FFT requests submitted concurrently from
several host threads is continuously batched over a resident basis; every
result must equal the same request run alone (compressed / serialized bytes:
exact integer results, so the tolerance is zero)."""
import random
import threading

import pytest

pytestmark = pytest.mark.gpu


def test_serving_mix_equals_alone(gpu, oracle, synth):
    n = 4096
    pts = oracle.gen_points(700, n)
    basis = gpu.Basis(pts, n, 10)
    server = gpu.Server(basis, workers=3, hbm_budget=1 << 30)
    rnd = random.Random(701)
    reqs = []
    for r in range(48):
        if rnd.random() < 0.7:
            k = int(2 ** rnd.uniform(4, 12))
            reqs.append(("msm", k, synth.scalars(800 + r, k, 0)))
        else:
            m = 1 << rnd.choice([4, 6, 8])
            jac = oracle.jacobian_randomize(900 + r, m, oracle.gen_points(900 + r, m))
            reqs.append(("fft", m, jac, gpu.fr_fft_domain_init(m)[1], rnd.choice([0, 1, 2])))
    results = [None] * len(reqs)

    def client(idx):
        tickets = []
        for i in idx:
            q = reqs[i]
            t = server.submit_msm(q[2], q[1]) if q[0] == "msm" else server.submit_fft(q[2], q[1], q[3], q[4])
            tickets.append((i, t))
        for i, t in tickets:
            results[i] = server.wait(t)

    ths = [threading.Thread(target=client, args=(list(range(c, len(reqs), 4)),)) for c in range(4)]
    for t in ths:
        t.start()
    for t in ths:
        t.join()
    st = server.stats()
    assert st["requests"] == len(reqs)
    # alone: each request by itself through the non-serving entry points
    for q, res in zip(reqs, results):
        rc, out, qms, lat = res
        assert rc == 0 and lat >= qms >= 0
        if q[0] == "msm":
            alone = basis.msm_batch([q[1]], q[2])
            assert oracle.compress(out) == oracle.compress(alone)
            assert oracle.compress(out) == oracle.msm(pts[:96 * q[1]], q[2], q[1], 256)
        else:
            m, jac, dom, mode = q[1], q[2], q[3], q[4]
            if mode == 2:
                ok, alone = gpu.p1_ifft_unscaled_with_domain(jac, m, dom, m + 2)
            else:
                ok, alone = gpu.p1_fft_with_domain(jac, m, dom, m + 2, mode == 1)
            assert ok
            for i in range(m):
                assert oracle.serialize(out[144 * i:144 * i + 144]) == oracle.serialize(alone[144 * i:144 * i + 144])
    server.close()
    basis.close()


def test_serving_batches_and_overlaps(gpu, oracle, synth):
    """Continuous batching is real, not a serial queue: three FFTs of
    different sizes (three size classes) occupy three workers at once, and
    a burst of same-class MSMs submitted meanwhile is taken as batches of
    more than one request; a large MSM (the plain-pipeline route) and the
    burst results equal the oracle."""
    n = 1 << 18
    pts = gpu.points_from_scalars(synth.point_scalars(710, n), n)
    basis = gpu.Basis(pts, n, 10)
    server = gpu.Server(basis, workers=3, hbm_budget=4 << 30)
    ffts = []
    for e in (12, 13, 14):
        m = 1 << e
        jac = oracle.jacobian_randomize(711 + e, m, oracle.gen_points(711 + e, m))
        dom = gpu.fr_fft_domain_init(m)[1]
        ffts.append((m, jac, dom, server.submit_fft(jac, m, dom, 0)))
    burst = []
    for r in range(64):
        k = 300 + r
        sc = synth.scalars(720 + r, k, 0)
        burst.append((k, sc, server.submit_msm(sc, k)))
    big_sc = synth.scalars(799, n, 0)
    big = server.submit_msm(big_sc, n)
    for m, jac, dom, t in ffts:
        rc, out, qms, lat = server.wait(t)
        assert rc == 0
        ok, alone = gpu.p1_fft_with_domain(jac, m, dom, m + 2, False)
        assert ok and all(oracle.serialize(out[144 * i:144 * i + 144]) == oracle.serialize(alone[144 * i:144 * i + 144])
                          for i in range(0, m, 97))
    for k, sc, t in burst:
        rc, out, _, _ = server.wait(t)
        assert rc == 0 and oracle.compress(out) == oracle.msm(pts[:96 * k], sc, k, 256)
    rc, out, _, _ = server.wait(big)
    assert rc == 0 and oracle.compress(out) == oracle.compress(gpu.p1s_mult_pippenger(pts, big_sc, n, 256))
    st = server.stats()
    assert st["requests"] == 3 + 64 + 1
    assert st["max_batch"] > 1, st          # requests that queued meanwhile were batched
    assert st["max_concurrent"] > 1, st     # batches of different workers overlapped
    server.close()
    basis.close()
