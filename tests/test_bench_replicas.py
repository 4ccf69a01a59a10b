"""bench.py's multi-GPU form runs independent replicas and reduces only the
timings: the max over ranks of the elapsed time (CPU, gloo, world size 2)."""
import os
import socket
import sys

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist          # noqa: E402
import torch.multiprocessing as mp        # noqa: E402

from conftest import ROOT                 # noqa: E402


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import bench
    ws, r, local = bench.dist_setup()
    assert (ws, r, local) == (world, rank, rank)
    bench.barrier(ws)
    t = bench.max_over_ranks(ws, 10.0 * (rank + 1))
    out[rank] = t
    dist.destroy_process_group()


def test_replica_timing_reduction_gloo():
    world = 2
    port = _free_port()
    out = mp.Manager().dict()
    mp.start_processes(_rank, args=(world, port, out), nprocs=world, join=True,
                       start_method="spawn")
    assert dict(out) == {0: 20.0, 1: 20.0}
