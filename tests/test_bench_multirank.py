"""Host logic of bench.py under torchrun, on CPU with two gloo ranks: the
rendezvous, the barrier and the max-over-ranks timing that turn per-rank
times into the whole-job value (weak scaling, no collective on the data
path).  The GPU work itself is one independent replica per rank."""
import os
import socket
import sys

import pytest
import torch.multiprocessing as tmp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    os.environ.update(RANK=str(rank), LOCAL_RANK=str(rank), WORLD_SIZE=str(world),
                      MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import bench
    r, ws, dist = bench.dist_setup()
    assert (r, ws) == (rank, world)
    assert dist.get_backend() == "gloo"
    bench.barrier(dist)
    local_ms = 100.0 + 50.0 * rank
    out[rank] = bench.reduce_max(dist, local_ms)
    dist.destroy_process_group()


def test_two_rank_max_timing():
    port = _free_port()
    mgr = tmp.Manager()
    out = mgr.dict()
    tmp.spawn(_worker, args=(2, port, out), nprocs=2, join=True)
    assert out[0] == out[1] == 150.0


def test_single_rank_needs_no_process_group(monkeypatch):
    monkeypatch.delenv("WORLD_SIZE", raising=False)
    sys.path.insert(0, ROOT)
    import bench
    assert bench.dist_setup() == (0, 1, None)
    assert bench.reduce_max(None, 3.0) == 3.0
