"""Host checks of the double-float arithmetic and the double-float normal tail
table (massivemds_gb300/csrc/dd.h, normal_dd.h), compiled with the host C++
compiler: each operation against long double, and log Phi(z), phi(z) / Phi(z)
on [0, 9] against the C library's erfc, exp and log1p in long double, from the
double-float table and from the FP64 sweeps' double table (tests/dd_check.cpp
prints the measured errors and their bounds). No GPU."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "massivemds_gb300", "csrc")


def test_double_float_ops_and_normal_table(tmp_path):
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no host C++ compiler")
    exe = str(tmp_path / "dd_check")
    subprocess.run([cxx, "-O2", "-std=c++17", "-I", CSRC, os.path.join(HERE, "dd_check.cpp"), "-o", exe],
                   check=True)
    r = subprocess.run([exe], capture_output=True, text=True)
    lines = dict((ln.split()[0], (float(ln.split()[1]), float(ln.split()[2]))) for ln in r.stdout.splitlines())
    for name in ("add", "mul", "sqr", "fma", "rsqrt", "rcp", "div", "acc_fma_20000", "acc_sqr_20000",
                 "normal_logcdf_abs", "normal_ratio_abs", "normal_f64_logcdf_abs", "normal_f64_ratio_abs"):
        assert name in lines, r.stdout
    assert r.returncode == 0, r.stdout
    assert lines["normal_logcdf_abs"][0] < 5e-14 and lines["normal_ratio_abs"][0] < 5e-14
    # the FP64 sweeps' table (normal_f64): FP64-grade
    assert lines["normal_f64_logcdf_abs"][0] < 5e-16 and lines["normal_f64_ratio_abs"][0] < 5e-16


def test_double_float_flag_excludes_float(mdsx_lib):
    """MDSX_FLAG_DOUBLE_FLOAT with MDSX_FLAG_FLOAT is rejected before any device call."""
    import ctypes

    from massivemds_gb300 import flags as F

    h = ctypes.c_void_p()
    rc = mdsx_lib.mdsx_create(2, 16, F.DOUBLE_FLOAT | F.FLOAT, -1, ctypes.byref(h))
    assert rc == 1
    assert b"exclude" in mdsx_lib.mdsx_last_error(None)
