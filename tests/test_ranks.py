"""The multi-rank bookkeeping of bench.py (one process per GPU under torchrun) on the host: two
gloo ranks agree on the slowest rank's time and on the whole-job throughput, and a single process
needs no process group."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def rank_main(rank, world, port, out):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import bench
    r = bench.Ranks("gloo", "cpu")
    r.barrier()
    ms = 10.0 + 5.0 * rank          # rank 1 is the slow one
    slowest = r.max(ms)
    value = r.throughput(1000, ms)  # 1000 units per rank
    r.barrier()
    out.put((rank, slowest, value))
    r.dist.destroy_process_group()


def test_two_gloo_ranks_agree_on_the_slowest_time_and_the_job_throughput():
    mp = pytest.importorskip("torch.multiprocessing")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = free_port()
    procs = [ctx.Process(target=rank_main, args=(k, 2, port, q)) for k in range(2)]
    for p in procs:
        p.start()
    results = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, slowest, value in results:
        assert slowest == 15.0
        assert value == pytest.approx(2 * 1000 / 15e-3)


def test_single_process_needs_no_process_group(monkeypatch):
    for k in ("RANK", "WORLD_SIZE", "LOCAL_RANK"):
        monkeypatch.delenv(k, raising=False)
    sys.path.insert(0, ROOT)
    import bench
    r = bench.Ranks("gloo", "cpu")
    assert r.dist is None and r.world == 1
    r.barrier()
    assert r.max(7.5) == 7.5 and r.throughput(300, 10.0) == pytest.approx(300 / 10e-3)
