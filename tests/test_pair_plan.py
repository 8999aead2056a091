"""CPU test of the unordered-pair plan (massivemds_gb300/csrc/pair_plan.h): builds
tests/pair_plan_check.cu (host code only) with nvcc and runs it. The driver walks
every CTA's unit range the way the pair kernels do and checks coverage of every
pair, the producer/consumer unit order and the slot tables; it replays the finish
kernel's index arithmetic for every finish shape and checks its reads stay inside
the partial buffers, read each partial once and write each gradient entry once."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)


def _nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    return None


def test_pair_plan_walk(tmp_path):
    nvcc = _nvcc()
    if nvcc is None:
        pytest.skip("nvcc not found")
    exe = str(tmp_path / "pair_plan_check")
    build = subprocess.run([nvcc, "-std=c++17", "-O2", "-I", os.path.join(REPO, "massivemds_gb300", "csrc"),
                            "-I", os.path.join(REPO, "include"), os.path.join(HERE, "pair_plan_check.cu"), "-o", exe],
                           capture_output=True, text=True)
    assert build.returncode == 0, build.stderr
    run = subprocess.run([exe], capture_output=True, text=True, timeout=600)
    assert run.returncode == 0 and run.stdout.strip().endswith("ok"), run.stdout + run.stderr
