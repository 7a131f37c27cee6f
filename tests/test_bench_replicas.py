"""bench.py's multi-GPU path is replicas only: one scene per rank, no
collective on the data path; the timing takes the max over ranks and the
value sums the ranks' particle-steps.  Checked here on CPU with two gloo
ranks (host logic only, no GPU)."""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import sys
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    w, r, loc = bench.dist_env()
    t = bench.max_over_ranks(1.0 + rank)  # rank 1 is the slow replica
    out[rank] = (w, r, loc, t, bench.replica_throughput(1000, 10, t, w))
    dist.destroy_process_group()


def test_two_replicas_on_gloo():
    world = 2
    mgr = mp.Manager()
    out = mgr.dict()
    mp.spawn(_rank, args=(world, _free_port(), out), nprocs=world, join=True)
    for rank in range(world):
        w, r, loc, t, v = out[rank]
        assert (w, r, loc) == (world, rank, rank)
        assert t == 2.0                       # max over ranks
        assert v == pytest.approx(2 * 1000 * 10 / 2.0)  # whole-job value


def test_single_process_has_no_collective():
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import bench
    assert bench.max_over_ranks(3.5) == 3.5
