"""bench.py under torchrun runs one independent replica (gauge configuration)
per GPU; the ranks only agree on the slowest time.  Checked here with two gloo
ranks on the CPU."""
import os
import socket
import sys
from pathlib import Path

import pytest

torch = pytest.importorskip("torch")
import torch.multiprocessing as mp  # noqa: E402

REPO = Path(__file__).resolve().parents[1]


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    sys.path.insert(0, str(REPO))
    import bench
    r, w, local, dist = bench.dist_setup(world, backend="gloo")
    assert (r, w, local) == (rank, world, rank)
    bench.barrier(dist)
    out[rank] = bench.max_over_ranks(dist, 1.5 + rank)
    dist.destroy_process_group()


def test_two_replicas_agree_on_the_slowest_time():
    world, port = 2, _free_port()
    out = mp.Manager().dict()
    mp.spawn(_rank, args=(world, port, out), nprocs=world, join=True)
    assert dict(out) == {0: 2.5, 1: 2.5}


def test_single_process_has_no_group():
    sys.path.insert(0, str(REPO))
    import bench
    for k in ("WORLD_SIZE", "RANK", "LOCAL_RANK"):
        os.environ.pop(k, None)
    assert bench.dist_setup(1)[3] is None
    assert bench.max_over_ranks(None, 3.25) == 3.25
