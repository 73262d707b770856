"""bench.py's multi-rank logic on CPU: world_size-2 gloo ranks.

Replicas run independent reconstructions; the job's time is the slowest
rank's, and its rate counts every rank's units.  The reference arm runs on
rank 0 only and the other ranks exit 0 without work.
"""
import importlib.util
import json
import os
import socket
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def _bench():
    spec = importlib.util.spec_from_file_location("bench_mod", ROOT / "bench.py")
    m = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(m)
    return m


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank: int, world: int, port: int, q) -> None:
    import torch.distributed as dist

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    b = _bench()
    local_ms = [120.0, 185.5][rank]  # rank 1 is the slow replica
    ms = b.max_over_ranks(local_ms, dist)
    rate = b.whole_job_rate(world, 32 * 5, ms / 1000.0)
    q.put((rank, ms, rate))
    dist.destroy_process_group()


def test_max_over_ranks_and_whole_job_rate_gloo():
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, ms, rate in out:
        assert ms == 185.5  # every rank reports the slowest
        assert rate == pytest.approx(2 * 160 / 0.1855)


def test_single_rank_needs_no_process_group():
    b = _bench()
    assert b.max_over_ranks(7.25, None) == 7.25
    assert b.whole_job_rate(1, 64, 0.5) == 128


def test_reference_arm_other_ranks_exit_without_work():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    r = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--gpus", "2",
                        "--steps", "1", "--warmup", "0"], env=env, capture_output=True, text=True, timeout=120)
    assert r.returncode == 0
    assert r.stdout.strip() == ""


def test_gpu_arm_refuses_without_device():
    """Without a CUDA device the product path raises; it never falls back to the CPU."""
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    r = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--steps", "1", "--warmup", "0"],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode != 0
    assert not any(line.startswith("{") for line in r.stdout.splitlines()), r.stdout


def test_reference_line_shape(monkeypatch, capsys):
    """The reference arm's JSON line: metric, config and the cpu_baseline / e2e objects,
    with the oracle timing stubbed out (no CPU work here)."""
    b = _bench()
    monkeypatch.setattr(b, "cpu_subiterations",
                        lambda n, w, *a, **k: {"value": 0.5, "unit": b.UNIT, "cores": 4, "kind": "port",
                                               "seconds": 2.0 * n, "sample": "stub"})
    monkeypatch.setenv("RANK", "0")

    class A:
        gpus, steps, warmup = 1, 2, 0

    assert b.run_reference(A()) == 0
    line = json.loads(capsys.readouterr().out)
    assert line["impl"] == "reference" and line["metric"] == b.METRIC and line["unit"] == b.UNIT
    assert line["e2e"] == {"value": 0.5, "unit": b.UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    assert line["cpu_baseline"]["kind"] == "port" and line["cpu_baseline"]["cores"] == 4
    assert line["config"]["workload"] == b.WORKLOAD
