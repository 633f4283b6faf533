"""The N > 1 path of bench.py: independent replicas (one process per GPU), no data exchange,
the slowest replica's time sets the job time.  Run here as two gloo processes on the CPU."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist          # noqa: E402
import torch.multiprocessing as mp        # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    import bench
    d, r, w = bench.dist_setup("gloo")
    assert (r, w) == (rank, world)
    local = [1.5 + rank, 10.0 - rank]                 # per-rank step and e2e seconds
    mx = bench.max_over_ranks(local, d, device="cpu")
    out[rank] = (bench.replica_seed(7, r), mx, bench.aggregate_value(100.0, w, mx[0]))
    d.barrier()
    d.destroy_process_group()


def test_two_replicas_gloo():
    world = 2
    port = _free_port()
    with mp.get_context("spawn").Manager() as m:
        out = m.dict()
        mp.spawn(_worker, args=(world, port, out), nprocs=world, join=True)
        res = dict(out)
    seeds = {res[r][0] for r in range(world)}
    assert seeds == {7, 8}                                   # every replica draws its own chunk
    for r in range(world):
        assert res[r][1] == [2.5, 10.0]                      # max over ranks, element-wise
        assert res[r][2] == pytest.approx(2 * 100.0 / 2.5)   # all units over the slowest time
