"""Multi-GPU runs are replicas (every rank solves its own scene, no data-path
collective): the whole-job time is the slowest rank's and the cell count the
sum of all ranks'.  Checked with two gloo ranks on CPU."""
import os
import socket
import sys

import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    ms, cells = bench.replica_totals(10.0 + rank, 1000 * (rank + 1), dist, device="cpu")
    out[rank] = (ms, cells)
    dist.destroy_process_group()


def test_replica_totals_gloo():
    world = 2
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_rank, args=(world, _free_port(), out), nprocs=world, join=True)
        res = dict(out)
    assert res == {0: (11.0, 3000.0), 1: (11.0, 3000.0)}


def test_replica_totals_single():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.replica_totals(5.0, 42, None) == (5.0, 42.0)
