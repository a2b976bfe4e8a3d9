"""bench.py's host-side contract, on the CPU.

- The multi-rank timing: every rank's timed region reduced to the slowest
  one over a world-size-2 gloo group, and the whole-job throughput (each rank
  sorts its own replica of the workload, so the keys of all ranks count).
- The reference arm (the oracle's per-segment std::stable_sort, the
  reference's mseq algorithm, src/mseq.cu:44-49) alone and under
  torchrun: rank 0 prints the one JSON line, the other ranks exit 0 without
  work.
"""
from __future__ import annotations

import json
import os
import socket
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT))
import bench  # noqa: E402


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _max_rank(rank: int, world: int, port: int, values: list, out_dir: str) -> None:
    import torch.distributed as dist
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank,
                            world_size=world)
    try:
        got = bench.max_over_ranks(values[rank], world)
        Path(out_dir, f"{rank}.json").write_text(json.dumps(got))
    finally:
        dist.destroy_process_group()


def test_max_over_ranks_gloo(tmp_path):
    import torch.multiprocessing as mp
    values = [3.25, 7.5]
    mp.spawn(_max_rank, args=(2, _free_port(), values, str(tmp_path)), nprocs=2, join=True)
    got = [json.loads(Path(tmp_path, f"{r}.json").read_text()) for r in range(2)]
    assert got == [7.5, 7.5]


def test_max_over_ranks_one_rank():
    assert bench.max_over_ranks(4.0, 1) == 4.0


def test_whole_job_gkeys():
    # 20 instances of 2^24 keys a step, 3 steps, 2 ranks, 100 ms for the slowest.
    assert bench.whole_job_gkeys(20 << 24, 3, 2, 100.0) == pytest.approx(20.13265920, rel=1e-9)
    assert bench.whole_job_gkeys(20 << 24, 3, 1, 100.0) == pytest.approx(10.06632960, rel=1e-9)


BENCH_ARGS = ["--impl", "reference", "--steps", "1", "--warmup", "1", "--log-n", "14",
              "--lengths", "1,6,12"]


def _json_lines(text: str) -> list[dict]:
    return [json.loads(l) for l in text.splitlines() if l.startswith("{")]


def _check_reference_line(d: dict, gpus: int) -> None:
    assert d["impl"] == "reference"
    assert d["metric"] == bench.METRIC and d["unit"] == "Gkeys/s" and d["higher_is_better"]
    assert d["n_gpus"] == gpus and d["steps"] == 1 and d["warmup"] == 1
    assert d["value"] > 0 and d["cpu_baseline"]["value"] == d["value"]
    assert d["cpu_baseline"]["kind"] == "port" and d["cpu_baseline"]["cores"] >= 1
    assert d["e2e"] == {"value": d["value"], "unit": "Gkeys/s", "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}


def test_reference_arm_one_process():
    r = subprocess.run([sys.executable, "bench.py", *BENCH_ARGS], cwd=ROOT, capture_output=True,
                       text=True, timeout=900)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = _json_lines(r.stdout)
    assert len(lines) == 1
    _check_reference_line(lines[0], 1)


def test_reference_arm_under_torchrun():
    env = dict(os.environ, MASTER_ADDR="127.0.0.1")
    r = subprocess.run([sys.executable, "-m", "torch.distributed.run", "--nnodes=1",
                        "--nproc-per-node", "2", "--master-addr", "127.0.0.1", "--master-port",
                        str(_free_port()), "bench.py", "--gpus", "2", *BENCH_ARGS],
                       cwd=ROOT, capture_output=True, text=True, timeout=900, env=env)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = _json_lines(r.stdout)
    assert len(lines) == 1  # rank 0 alone prints
    _check_reference_line(lines[0], 2)


def test_config_names_the_workload():
    """The default run is the sweep of 2^24-pair instances over lengths 2^1..2^20,
    above L2; other runs say what they are, and whether they fit in L2."""
    d = bench.bench_config(1 << 24, list(range(1, 21)), 1)
    assert d["workload"] == bench.WORKLOAD and d["l2"].startswith("inputs larger than L2: 128 MiB")
    small = bench.bench_config(1 << 20, [1, 10, 18], 2)
    assert "2^20 uint32" in small["workload"] and "2^1, 2^10, 2^18" in small["workload"]
    assert small["l2"].startswith("inputs smaller than L2") and small["parallelism"] == "replicas2"
