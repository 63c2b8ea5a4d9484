"""CPU checks of bench.py's multi-rank harness (replicas: one independent state per rank, no data-path
collective). Two gloo ranks on 127.0.0.1 stand in for two GPUs: the timing reduction gives every rank
the slowest rank's times, and the whole-job value counts every replica's bytes over that time."""
from __future__ import annotations

import json
import os
import socket
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def _free_port() -> int:
    with socket.socket(socket.AF_INET, socket.SOCK_STREAM) as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank: int, world: int, port: int, out_dir: str) -> None:
    import torch.distributed as dist

    sys.path.insert(0, str(ROOT))
    import bench

    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    try:
        # rank r: device time 1 + r s, end-to-end time 5 - r s
        dev_s, e2e_s = bench.slowest_rank_seconds(dist, [1.0 + rank, 5.0 - rank], "cpu")
        value = bench.job_gbs(3.0e9, world, dev_s)
        dist.barrier()
    finally:
        dist.destroy_process_group()
    Path(out_dir, f"rank{rank}.json").write_text(json.dumps({"dev_s": dev_s, "e2e_s": e2e_s, "value": value}))


def test_slowest_rank_times_and_job_value_with_two_gloo_ranks(tmp_path):
    mp = pytest.importorskip("torch.multiprocessing")
    world = 2
    mp.start_processes(_rank_main, args=(world, _free_port(), str(tmp_path)), nprocs=world, join=True,
                       start_method="spawn")
    for rank in range(world):
        r = json.loads((tmp_path / f"rank{rank}.json").read_text())
        assert r["dev_s"] == 2.0 and r["e2e_s"] == 5.0
        # both replicas' bytes (3 GB each) over the slowest rank's 2 s
        assert r["value"] == pytest.approx(3.0)


def test_single_process_keeps_its_own_times():
    sys.path.insert(0, str(ROOT))
    import bench

    assert bench.slowest_rank_seconds(None, [0.25, 0.5], "cpu") == [0.25, 0.5]
    assert bench.job_gbs(34.36e9, 1, 0.5) == pytest.approx(68.72)


def test_reference_arm_runs_on_rank_zero_only():
    """Under torchrun the reference arm's rank 0 alone times the host sample; the other ranks exit 0
    without work or output."""
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    res = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--steps", "2",
                          "--warmup", "3", "--cpu-qubits", "12", "--gpus", "2"], capture_output=True, text=True,
                         timeout=300, cwd=ROOT, env=env)
    assert res.returncode == 0, res.stderr
    assert not [line for line in res.stdout.splitlines() if line.startswith("{")]
