"""The C++ drop-in (mds::CudaMultiDimensionalScaling over libmdsx.so) as a
compiled program: tests/dropin_driver.cpp builds the engine through a
factory-shaped function and replays the reference benchmark's call sequence
(src/benchmark.cpp:167-309) on the golden sequence data, which the reference
engine itself produced (tests/golden/make_golden.py). The CPU test compiles and
links the driver; the GPU test runs it in FP64 and in double-float (both at 1e-10
sum, 1e-9 gradient) and FP32 (1e-5) and also has it check the interface's
protected flags and its exception on a wrong length."""
import os
import shutil
import subprocess

import numpy as np
import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
DRIVER = os.path.join(REPO, "tests", "dropin_driver.cpp")
FLAG_FLOAT, FLAG_OPENCL, FLAG_TRUNC, FLAG_DOUBLE_FLOAT = 1 << 2, 1 << 4, 1 << 5, 1 << 12


def _build(mdsx_lib, out_dir):
    gxx = shutil.which("g++")
    if not gxx:
        pytest.skip("g++ not available")
    from massivemds_gb300.build import LIB_PATH

    exe = os.path.join(out_dir, "dropin_driver")
    lib_dir = os.path.dirname(LIB_PATH)
    res = subprocess.run([gxx, "-std=c++17", "-O2", "-I", os.path.join(REPO, "include"), DRIVER, "-o", exe,
                          "-L", lib_dir, "-lmdsx", f"-Wl,-rpath,{lib_dir}"], capture_output=True, text=True)
    assert res.returncode == 0, res.stderr
    return exe


def test_dropin_driver_builds_and_links(mdsx_lib, tmp_path):
    assert os.path.exists(_build(mdsx_lib, str(tmp_path)))


@pytest.mark.gpu
@pytest.mark.parametrize("flags,tol_s,tol_g", [(FLAG_OPENCL | FLAG_TRUNC, 1e-10, 1e-9),
                                               (FLAG_OPENCL | FLAG_TRUNC | FLAG_DOUBLE_FLOAT, 1e-10, 1e-9),
                                               (FLAG_OPENCL | FLAG_TRUNC | FLAG_FLOAT, 1e-5, 1e-5)])
def test_dropin_replays_the_reference_benchmark_sequence(mdsx_lib, golden, tmp_path, flags, tol_s, tol_g):
    data, _ = golden
    delta, x0, xs = data["seq.delta"], data["seq.x0"], data["seq.xs"]
    restores, tau = data["seq.restores"], float(data["seq.tau"])
    n, p = x0.shape
    iters = xs.shape[0]
    exe = _build(mdsx_lib, str(tmp_path))
    inp, out = tmp_path / "in.bin", tmp_path / "out.bin"
    with open(inp, "wb") as f:
        np.array([n, p, iters], dtype=np.int32).tofile(f)
        np.array([flags], dtype=np.int64).tofile(f)
        np.array([tau], dtype=np.float64).tofile(f)
        for a in (delta, x0, xs):
            np.ascontiguousarray(a, dtype=np.float64).tofile(f)
        np.asarray(restores, dtype=np.uint8).tofile(f)
    res = subprocess.run([exe, str(inp), str(out)], capture_output=True, text=True, timeout=120)
    assert res.returncode == 0, res.stderr
    raw = np.fromfile(out, dtype=np.float64)
    sums, grads = raw[:iters + 1], raw[iters + 1:].reshape(iters + 1, n, p)
    ref_s, ref_g = data["seq.sums"], data["seq.grads"]
    for k in range(iters + 1):
        assert abs(sums[k] - ref_s[k]) / abs(ref_s[k]) < tol_s, k
        g_ref = ref_g[k].reshape(n, p)
        assert np.abs(grads[k] - g_ref).max() / np.abs(g_ref).max() < tol_g, k
