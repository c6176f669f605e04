"""Multi-GPU is replicas only (each rank runs its own workload; no data-path
collective).  The harness's N>1 logic — process group, barrier, max of the
ranks' times, whole-job throughput — runs here as two gloo ranks on CPU."""
import os
import socket
import sys

import pytest

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), os.pardir))


def free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank(rank, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE="2", RANK=str(rank),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import bench
    d = bench.Dist(backend="gloo")
    d.barrier()
    ms_local = 100.0 if rank == 0 else 250.0  # the slower rank bounds the job
    ms_max, value = bench.aggregate(d, ms_local, units_per_rank=1000)
    q.put((rank, d.ws, ms_max, value))
    d.close()


def test_two_gloo_ranks_aggregate():
    mp = pytest.importorskip("torch.multiprocessing")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = free_port()
    ps = [ctx.Process(target=_rank, args=(r, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    out = sorted(q.get(timeout=120) for _ in ps)
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, ws, ms_max, value in out:
        assert ws == 2 and ms_max == 250.0
        assert value == pytest.approx(2 * 1000 / 0.25)


def test_single_rank_needs_no_process_group():
    sys.path.insert(0, ROOT)
    import bench
    for k in ("WORLD_SIZE", "RANK", "LOCAL_RANK"):
        os.environ.pop(k, None)
    d = bench.Dist()
    assert d.ws == 1 and d.pg is None
    assert bench.aggregate(d, 500.0, 10) == (500.0, 20.0)
