"""CPU tests of the multi-rank (replicas) path of bench.py with the gloo backend, world size 2:
the max-over-ranks timing, the whole-job value, and the reference arm running on rank 0 only."""
import json
import os
import socket
import subprocess
import sys

import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, values, out):
    sys.path.insert(0, ROOT)
    import bench
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    try:
        got = bench.max_over_ranks(values[rank], world, "cpu")
        dist.barrier()
    finally:
        dist.destroy_process_group()
    with open(os.path.join(out, f"rank{rank}.txt"), "w") as f:
        f.write(repr(got))


def test_max_over_ranks_gloo(tmp_path):
    values = [12.5, 31.25]
    mp.start_processes(_rank, args=(2, _free_port(), values, str(tmp_path)), nprocs=2, start_method="spawn")
    for r in range(2):
        assert float((tmp_path / f"rank{r}.txt").read_text()) == 31.25


def test_replica_value_counts_all_ranks():
    import bench
    # 2 replicas of 1,000 particles, 10 steps, slowest rank 20 ms: 2 * 1000 * 10 / 0.02 s
    assert bench.replica_value(1000, 10, 20.0, 2) == pytest.approx(1e6)
    assert bench.replica_value(1000, 10, 20.0, 1) == pytest.approx(5e5)


@pytest.mark.parametrize("rank", [0, 1])
def test_reference_arm_runs_on_rank_zero_only(rank):
    env = dict(os.environ, RANK=str(rank), WORLD_SIZE="2", LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--n", "4096",
                        "--steps", "1", "--warmup", "1"], env=env, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    if rank == 0:
        assert len(lines) == 1
        line = json.loads(lines[0])
        assert line["impl"] == "reference" and line["value"] > 0 and line["cpu_baseline"]["cores"] >= 1
    else:
        assert lines == []
