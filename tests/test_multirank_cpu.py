"""The replica path of bench.py under torch.distributed, on CPU with gloo
(world size 2): the job time is the slowest rank's, the value counts every
rank's cells, and each rank runs its own seeded workload."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, out):
    import torch.distributed as dist
    import bench
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        mine = [1.5, 4.0][rank]  # seconds this rank took
        slowest = bench.max_over_ranks(mine, dist, "cpu")
        value = bench.replica_value(100.0, 10, world, slowest)
        g = bench.workload(bench.SEED + rank)
        out[rank] = (slowest, value, hash(g["kind"].tobytes()))
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_replicas_take_the_slowest_rank_and_count_all_cells():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    manager = ctx.Manager()
    out = manager.dict()
    port = _free_port()
    procs = [ctx.Process(target=_worker_entry, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    assert out[0][0] == out[1][0] == 4.0
    assert out[0][1] == out[1][1] == pytest.approx(100.0 * 10 * 2 / 4.0)
    # each rank builds its own seeded obstacle layout
    assert out[0][2] != out[1][2]


def _worker_entry(rank, world, port, out):
    import sys
    from pathlib import Path
    root = Path(__file__).resolve().parents[1]
    if str(root) not in sys.path:
        sys.path.insert(0, str(root))
    import bench
    bench.IMAX, bench.JMAX, bench.NRECTS = 256, 64, 4  # a small workload keeps the test quick
    _worker(rank, world, port, out)
