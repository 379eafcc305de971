"""Multi-rank bookkeeping of bench.py on the CPU: two gloo ranks stand in for
two GPUs running independent replicas.  Checks the slowest-rank timing, the
whole-job throughput, per-rank seeds, and that only rank 0 prints the
reference arm's line."""
from __future__ import annotations

import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank: int, world: int, port: int, out_dir: str):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    ms_local = [10.0, 30.0, 20.0, 5.0][rank]
    ms = bench.max_over_ranks(ms_local, "cpu")
    dist.barrier()
    value = bench.replica_throughput(1_000_000, ms, world)
    with open(os.path.join(out_dir, f"rank{rank}.json"), "w") as fh:
        json.dump({"ms": ms, "value": value, "seed": bench.replica_seed(1, rank)}, fh)
    dist.destroy_process_group()


@pytest.mark.parametrize("world", [2, 4])
def test_replica_aggregation_gloo(tmp_path, world):
    import torch.multiprocessing as mp
    port = _free_port()
    mp.start_processes(_rank_main, args=(world, port, str(tmp_path)), nprocs=world, join=True,
                       start_method="spawn")
    res = [json.load(open(tmp_path / f"rank{r}.json")) for r in range(world)]
    slowest = max([10.0, 30.0, 20.0, 5.0][:world])
    for r in res:
        assert r["ms"] == slowest
        assert r["value"] == pytest.approx(world * 1_000_000 / (slowest / 1000.0))
    assert len({r["seed"] for r in res}) == world


def test_single_rank_identity():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(12.5) == 12.5
    assert bench.replica_throughput(1000, 500.0, 1) == pytest.approx(2000.0)


def test_reference_arm_other_ranks_silent():
    """Under torchrun only rank 0 runs the CPU reference arm; other ranks
    print nothing and exit 0."""
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "3"], env=env, capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    assert r.stdout.strip() == ""


def test_reference_arm_line():
    """Rank 0 of the reference arm prints one JSON line of the bench contract."""
    env = dict(os.environ, RANK="0", WORLD_SIZE="1", LOCAL_RANK="0")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "2",
                        "--warmup", "3", "--workload", "plain_small", "--reference-budget-s", "1"],
                       env=env, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    lines = [ln for ln in r.stdout.splitlines() if ln.strip()]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["metric"] == "histories/s" and d["value"] > 0
    assert d["cpu_baseline"]["kind"] == "port" and d["cpu_baseline"]["cores"] >= 1
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["e2e"]["value"] == d["value"]
