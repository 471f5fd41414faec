"""Several GPUs run independent replicas (the path shards by launch ray /
transmitter with no exchange): the whole-job totals sum the segments over
ranks and take the slowest rank's time.  Checked with world_size 2 on the
gloo backend, on CPU."""
import os
import socket
import sys

import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    seg, sec = (100.0, 2.0) if rank == 0 else (300.0, 3.0)
    res = bench.replica_totals(dist, world, seg, sec, seg / 2, sec * 2)
    out.put((rank, res))
    dist.barrier()
    dist.destroy_process_group()


def test_replica_totals_world2():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    got = dict(q.get(timeout=120) for _ in ps)
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    for r in (0, 1):
        assert got[r] == (400.0, 3.0, 200.0, 6.0)


def test_replica_totals_single():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.replica_totals(None, 1, 5.0, 1.0, 4.0, 2.0) == (5.0, 1.0, 4.0, 2.0)
