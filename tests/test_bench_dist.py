"""The multi-process plumbing of bench.py (replicas: one full workload per rank, a barrier
around the timed region and the maximum time over ranks), run as two gloo ranks on CPU."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket(socket.AF_INET, socket.SOCK_STREAM) as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, q):
    sys.path.insert(0, ROOT)
    os.environ.update({"RANK": str(rank), "WORLD_SIZE": str(world), "MASTER_ADDR": "127.0.0.1",
                       "MASTER_PORT": str(port)})
    import bench
    r, w = bench.dist_init()
    bench.barrier(w)
    t = bench.allreduce_max(10.0 * (rank + 1), w)
    bench.barrier(w)
    import torch.distributed as dist
    dist.destroy_process_group()
    q.put((r, w, t))


def test_two_rank_barrier_and_max_time():
    mp = pytest.importorskip("torch.multiprocessing")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r for r, _, _ in res] == [0, 1]
    assert all(w == 2 for _, w, _ in res)
    assert all(t == 20.0 for _, _, t in res)     # the maximum over ranks, seen by every rank


def test_single_process_defaults(monkeypatch):
    monkeypatch.delenv("WORLD_SIZE", raising=False)
    monkeypatch.delenv("RANK", raising=False)
    sys.path.insert(0, ROOT)
    import bench
    assert bench.dist_init() == (0, 1)
    assert bench.allreduce_max(3.5, 1) == 3.5
