"""The multi-GPU path of bench.py runs independent replicas (the sweep has
no cross-rank exchange): each rank times its own work and the job's time is
the slowest rank's. These tests run that aggregation as two gloo ranks on the
CPU, and check that the reference arm does no work on a rank other than 0."""
import argparse
import io
import os
import sys
from contextlib import redirect_stdout

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, REPO)
import bench  # noqa: E402


def _rank_main(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        elapsed = [120.0, 150.0][rank]  # ms: rank 1 is the slow replica
        slowest = bench.across_ranks_max(elapsed, world, "cpu")
        out[rank] = (slowest, bench.job_throughput(200, world, slowest / 1000.0))
    finally:
        dist.destroy_process_group()


def _free_port():
    import socket

    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_two_gloo_ranks_report_the_slowest_replica():
    world = 2
    with mp.Manager() as manager:
        out = manager.dict()
        mp.spawn(_rank_main, args=(world, _free_port(), out), nprocs=world, join=True)
        results = dict(out)
    assert results[0] == results[1]
    slowest, value = results[0]
    assert slowest == 150.0
    assert value == pytest.approx(2 * 200 / 0.150)


def test_single_rank_needs_no_process_group():
    assert bench.across_ranks_max(3.5, 1, "cpu") == 3.5
    assert bench.job_throughput(10, 1, 2.0) == 5.0


def test_reference_arm_runs_on_rank_zero_only(monkeypatch):
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("WORLD_SIZE", "2")
    monkeypatch.setenv("LOCAL_RANK", "1")
    args = argparse.Namespace(n=64, steps=1, warmup=0, cpu_seconds=0.01, gpus=2, impl="reference")
    buf = io.StringIO()
    with redirect_stdout(buf):
        bench.run_reference(args)
    assert buf.getvalue() == ""


def test_reference_arm_line_reports_what_it_timed(monkeypatch):
    """Rank 0 of the reference arm: one whole CPU evaluation per step, so
    steps x ms_per_step fits inside the call's own wall time; the line carries
    the host, the one-core and FP32 paths and the SIMD note."""
    import json
    import time

    for k in ("RANK", "WORLD_SIZE", "LOCAL_RANK"):
        monkeypatch.delenv(k, raising=False)
    args = argparse.Namespace(n=96, steps=3, warmup=1, cpu_seconds=0.02, gpus=1, impl="reference")
    buf = io.StringIO()
    t = time.perf_counter()
    with redirect_stdout(buf):
        bench.run_reference(args)
    wall_ms = 1000.0 * (time.perf_counter() - t)
    line = json.loads(buf.getvalue())
    assert line["impl"] == "reference" and line["config"]["evals_per_step"] == 1
    assert line["steps"] * line["ms_per_step"] <= wall_ms
    assert line["value"] == pytest.approx(1000.0 / line["ms_per_step"])
    paths = line["cpu_baseline"]["paths"]
    assert paths["serial_f64"]["cores"] == 1 and paths["threaded_f32"]["value"] > 0
    assert paths["host"]["uname_m"] and "avx" in paths
    assert line["e2e"]["h2d_bytes_per_step"] == 0
