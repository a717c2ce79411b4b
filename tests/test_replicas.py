"""Multi-GPU form of the benchmark: replicas only.  Every (geometry, gap,
frequency) solve is independent (the reference's MPI task farm,
src/transfer-mpi.cpp:91-190, hands them out with no data exchange), so ranks
split the step list and the only cross-rank operations are the barrier and
the maximum of the timings.  Covered here with world_size 2 on the gloo
backend (CPU), and the reference arm under torchrun."""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


@pytest.mark.parametrize("world", [1, 2, 3, 8])
def test_shards_partition_the_grid(world):
    grid = bench.step_grid(bench.WORKLOADS["ico3"])
    shards = [bench.shard_steps(grid, r, world) for r in range(world)]
    assert sum(len(s) for s in shards) == len(grid)
    assert sorted(x for s in shards for x in s) == sorted(grid)
    assert max(len(s) for s in shards) - min(len(s) for s in shards) <= 1


def _rank_main(rank, world, port, out):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    grid = bench.step_grid(bench.WORKLOADS["mix"])
    mine = bench.shard_steps(grid, rank, world)
    everyone = [None] * world
    dist.all_gather_object(everyone, mine)
    dist.barrier()
    ms = bench.max_over_ranks(10.0 + rank, world)
    with open(os.path.join(out, f"r{rank}.json"), "w") as f:
        json.dump({"ms": ms, "n": len(mine), "union": sorted(map(tuple, (x for s in everyone for x in s))) ==
                   sorted(map(tuple, grid))}, f)
    dist.destroy_process_group()


def test_two_gloo_ranks_split_and_take_the_slowest(tmp_path):
    import torch.multiprocessing as mp
    world = 2
    mp.spawn(_rank_main, args=(world, _free_port(), str(tmp_path)), nprocs=world, join=True)
    res = [json.load(open(tmp_path / f"r{r}.json")) for r in range(world)]
    assert all(r["ms"] == 11.0 for r in res)
    assert all(r["union"] for r in res)
    assert sum(r["n"] for r in res) == len(bench.step_grid(bench.WORKLOADS["mix"]))


def test_reference_arm_under_torchrun_prints_once():
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(_free_port()),
           os.path.join(ROOT, "bench.py"), "--impl", "reference", "--workload", "cube4", "--gpus", "2",
           "--steps", "1", "--warmup", "3"]
    out = subprocess.run(cmd, capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [ln for ln in out.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
