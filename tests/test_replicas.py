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


def test_bench_spawns_replicas_without_a_launcher():
    """`python bench.py --gpus 2` with no WORLD_SIZE in the environment starts two replica
    processes itself (here the gloo self-test leg, no GPU) and prints one line for the job."""
    import json
    import subprocess
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    env = {k: v for k, v in os.environ.items() if k not in ("WORLD_SIZE", "RANK", "LOCAL_RANK")}
    r = subprocess.run([sys.executable, os.path.join(root, "bench.py"), "--gpus", "2", "--selftest-replicas"],
                       capture_output=True, text=True, env=env, timeout=300)
    assert r.returncode == 0, r.stderr
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["n_gpus"] == 2 and d["parallelism"] == "replicas"
    assert d["seeds"] == [1, 2] and d["max_s"] == 0.75
    assert d["value"] == pytest.approx(2 * 100.0 / 0.75)
