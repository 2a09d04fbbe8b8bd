"""CPU: the N>1 path of bench.py (replicas only: one independent world per GPU, no data-path collective)
on two gloo ranks — the rendezvous, the barrier around the timed region and the max over ranks of the
per-rank step time, which is what makes `value` the whole-job figure."""
import os
import socket
import sys
from pathlib import Path

import pytest

torch = pytest.importorskip("torch")
import torch.multiprocessing as mp

ROOT = Path(__file__).resolve().parents[1]


def _free_port() -> int:
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank_main(rank: int, world: int, port: int, q):
    os.environ.update({"MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port), "WORLD_SIZE": str(world),
                       "RANK": str(rank), "LOCAL_RANK": str(rank)})
    sys.path.insert(0, str(ROOT))
    import bench
    dist, r, ws = bench.dist_setup()
    bench.barrier(dist)
    m = bench.max_over_ranks(dist, 1.5 + r)   # rank r's "step time"
    bench.barrier(dist)
    q.put((r, ws, m))
    dist.destroy_process_group()


def test_two_gloo_ranks_take_the_max_step_time():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert out == [(0, 2, 2.5), (1, 2, 2.5)]
