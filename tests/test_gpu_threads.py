"""Per-thread contexts: a thread's device workspaces are released when the
thread exits, so MSMs run from short-lived threads, and the worker threads of
a server that is destroyed, leave no device memory behind (with a leak, each
2^18-point MSM thread kept ~0.6 GB and a 2^20-point one ~4.5 GB)."""
import threading

import pytest

pytestmark = pytest.mark.gpu

SLACK = 96 << 20   # device-wide free memory may move by a few MB (other allocations, the driver)


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
