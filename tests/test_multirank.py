"""Multi-rank host logic on CPU (gloo, world size 2).

Cells shard across ranks with no data-path collective; what runs across
ranks is the barrier and the reductions of the timing and of the processed
units (mkpp_gb300/shard.py), and `bench.py --impl reference` under torchrun,
where rank 0 alone times the CPU reference and prints the line.
"""

import json
import os
import socket
import subprocess
import sys
from pathlib import Path

import numpy as np
import pytest

from mkpp_gb300 import shard, workloads

ROOT = Path(__file__).resolve().parent.parent


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port):
    import torch.distributed as dist

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE=str(world), RANK=str(rank),
                      LOCAL_RANK=str(rank))
    env = shard.rank_env()
    assert (env.world, env.rank) == (world, rank)
    shard.init(env, "gloo")
    try:
        assert shard.max_over_ranks(10.0 + rank) == 10.0 + world - 1
        assert shard.sum_over_ranks(rank + 1) == world * (world + 1) / 2
        # Rank r processed 100 (r + 1) units in 2 (r + 1) seconds: the job did
        # 300 units in 4 s (the slowest rank's time).
        units, seconds, rate = shard.job_throughput(100.0 * (rank + 1), 2.0 * (rank + 1))
        assert (units, seconds, rate) == (300.0, 4.0, 75.0)
        shard.barrier()
    finally:
        dist.destroy_process_group()


def test_reductions_and_throughput_on_two_gloo_ranks():
    import torch.multiprocessing as mp

    mp.start_processes(_rank_main, args=(2, _free_port()), nprocs=2, start_method="spawn")


def test_single_rank_needs_no_process_group():
    assert shard.max_over_ranks(3.5) == 3.5
    assert shard.sum_over_ranks(7) == 7.0
    shard.barrier()


@pytest.mark.parametrize("total,world", [(262144, 2), (262144, 8), (1000003, 8), (5, 8)])
def test_cell_blocks_partition_the_cells(total, world):
    blocks = [shard.cell_block(total, world, r) for r in range(world)]
    assert blocks[0][0] == 0 and blocks[-1][1] == total
    for (b0, e0), (b1, e1) in zip(blocks, blocks[1:]):
        assert e0 == b1
    sizes = [e - b for b, e in blocks]
    assert max(sizes) - min(sizes) <= 1


def test_ranks_draw_different_cells():
    a = workloads.make("chapman", 64, seed=shard.shard_seed(workloads.SEED, 0))
    b = workloads.make("chapman", 64, seed=shard.shard_seed(workloads.SEED, 1))
    a2 = workloads.make("chapman", 64, seed=shard.shard_seed(workloads.SEED, 0))
    assert not np.array_equal(a.conc, b.conc)
    assert np.array_equal(a.conc, a2.conc)


def test_reference_arm_under_torchrun_two_ranks():
    """torchrun with 2 ranks: exit 0, exactly one JSON line, from rank 0."""
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(_free_port()), str(ROOT / "bench.py"),
           "--impl", "reference", "--gpus", "2", "--workload", "chapman", "--cpu-cells", "16",
           "--steps", "1", "--warmup", "0"]
    env = dict(os.environ, OMP_NUM_THREADS="1")
    proc = subprocess.run(cmd, capture_output=True, text=True, timeout=600, cwd=ROOT, env=env)
    assert proc.returncode == 0, proc.stderr[-2000:]
    lines = [ln for ln in proc.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, proc.stdout
    line = json.loads(lines[0])
    assert line["impl"] == "reference" and line["n_gpus"] == 2
    assert line["value"] > 0 and line["e2e"]["h2d_bytes_per_step"] == 0
