"""CPU check of bench.py's multi-rank logic with world_size 2 over gloo:
every rank runs its own MSM replica, the reported time is the MAX over ranks,
and the whole-job throughput counts the points of all replicas."""
import importlib.util
import os
import socket

import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _bench():
    spec = importlib.util.spec_from_file_location("bench_mod", os.path.join(ROOT, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank(rank, ws, port, q):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(ws),
                      LOCAL_RANK=str(rank))
    b = _bench()
    wsz, r, local = b.dist_setup()
    dist.init_process_group("gloo", rank=r, world_size=wsz)
    times = b.max_over_ranks([10.0 + rank, 100.0 - rank], dist, "cpu")
    q.put((rank, times, b.aggregate_mpoints(wsz, 1 << 20, times[0])))
    dist.destroy_process_group()


def test_max_over_ranks_gloo_world2():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    out = sorted(q.get(timeout=120) for _ in ps)
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, times, mpts in out:
        assert times == [11.0, 100.0]
        assert abs(mpts - 2 * (1 << 20) / 11e-3 / 1e6) < 1e-9


def test_reference_arm_other_ranks_exit_clean():
    b = _bench()

    class A:
        n = 1 << 10
        steps = 1
        warmup = 0
    assert b.run_reference(A(), 2, 1) == 0


def test_bench_affine_encodings_match_oracle():
    """bench.py checks GPU outputs against the reference's golden bytes with
    its own Python normalisation and encodings (one batched inversion);
    they must equal the oracle's blst_p1_compress / blst_p1_serialize,
    including infinity and non-unit z."""
    import oracle as om
    b = _bench()
    o = om.Oracle()
    n = 40
    jac = o.jacobian_randomize(9, n, o.gen_points(9, n))
    blobs = [jac[144 * i:144 * i + 144] for i in range(n)]
    blobs[3] = bytes(144)                                  # infinity (z = 0)
    xys = b._affine_many(blobs)
    assert xys[3] is None
    for blob, xy in zip(blobs, xys):
        assert b._compress_xy(xy) == o.compress(blob)
        assert b._serialize_xy(xy) == o.serialize(blob)
