"""bench.py at N > 1 runs N independent replicas of the scene, one per rank (no data-path collective; the
path has no exchange step on one GPU per scene). Its host side is checked here with two gloo ranks on the
CPU: the rendezvous, the barrier and the whole-job value (the units of all ranks over the slowest rank's
time)."""
import os
import socket
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, ws, port, out):
    os.environ.update({"RANK": str(rank), "WORLD_SIZE": str(ws), "LOCAL_RANK": str(rank),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port), "GPE_BENCH_BACKEND": "gloo"})
    sys.path.insert(0, str(ROOT))
    import torch.distributed as dist

    import bench

    r, w = bench.dist_init()
    assert (r, w) == (rank, ws)
    bench.barrier(w)
    # rank k took 1 + k seconds for its 100 units: the job did 200 units in 2 s
    v = bench.replica_value(100.0, 1.0 + rank, w)
    bench.barrier(w)
    dist.destroy_process_group()
    out.put((rank, v))


def test_two_gloo_replicas_aggregate_over_the_slowest_rank():
    torch = pytest.importorskip("torch")
    mp = torch.multiprocessing.get_context("spawn")
    q = mp.Queue()
    port = _free_port()
    procs = [mp.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
    assert all(p.exitcode == 0 for p in procs)
    got = dict(q.get(timeout=5) for _ in range(2))
    assert got == {0: 100.0, 1: 100.0}
