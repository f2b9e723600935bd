"""Host-side logic of bench.py's multi-GPU mode (replicas only), on CPU: the
barrier, the max-over-ranks timing and the whole-job value with two gloo ranks,
and the reference arm's rank handling (rank 0 alone runs and prints)."""
import json
import os
import socket
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out_dir):
    import torch.distributed as dist

    sys.path.insert(0, str(ROOT))
    import bench

    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank,
                            world_size=world)
    bench.barrier(world)
    ms = bench.max_over_ranks(100.0 + 10.0 * rank, world)  # rank 1 is the slow one
    value = bench.job_value(ms, 20, world)
    bench.barrier(world)
    dist.destroy_process_group()
    Path(out_dir, f"rank{rank}.json").write_text(json.dumps({"ms": ms, "value": value}))


def test_replicas_max_over_ranks_gloo(tmp_path):
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp

    port = _free_port()
    mp.start_processes(_rank_main, args=(2, port, str(tmp_path)), nprocs=2, start_method="spawn",
                       join=True)
    for r in range(2):
        d = json.loads((tmp_path / f"rank{r}.json").read_text())
        assert d["ms"] == 110.0  # both ranks see the slowest replica
        assert abs(d["value"] - 2 * 20 / 0.110) < 1e-9


def test_reference_arm_runs_on_rank0_only():
    base = [sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--gpus", "2",
            "--m", "40", "--nsim", "200", "--cpu-sample", "50", "--steps", "2", "--warmup", "3",
            "--burn-in", "3", "--cpu-burn-in-draws", "50"]
    env = dict(os.environ, WORLD_SIZE="2", MASTER_ADDR="127.0.0.1")
    r1 = subprocess.run(base, env=dict(env, RANK="1"), capture_output=True, text=True, timeout=300)
    assert r1.returncode == 0 and r1.stdout.strip() == ""
    r0 = subprocess.run(base, env=dict(env, RANK="0"), capture_output=True, text=True, timeout=300)
    assert r0.returncode == 0, r0.stderr
    line = json.loads(r0.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["n_gpus"] == 2
    assert line["cpu_baseline"]["kind"] == "port" and line["value"] > 0
    assert line["e2e"]["h2d_bytes_per_step"] == 0
    # whole steps at the declared draw count; the line reports what ran
    assert line["steps"] == 2 and line["warmup"] == 1
    assert line["config"]["precision"] == "fp64" and line["config"]["nsim"] == 200
    assert abs(line["ms_per_step"] * line["steps"] / 1000.0 * line["value"] - line["steps"]) < 1e-9
