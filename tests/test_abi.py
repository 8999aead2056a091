"""CPU tests of the boundary: the C-ABI library builds, loads and exports every
symbol include/mdsx.h declares; host-side argument checks run without a GPU;
the C++ drop-in header compiles against the restated interface and, where the
reference tree exists, against the reference's own header."""
import ctypes
import os
import re
import shutil
import subprocess

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(REPO, "include", "mdsx.h")
from oracle import reference_root

_REF_ROOT = reference_root()
REF_SRC = os.path.join(_REF_ROOT, "src") if _REF_ROOT else None


def declared_symbols():
    text = open(HEADER).read()
    return sorted(set(re.findall(r"\b(mdsx_[a-z0-9_]+)\s*\(", text)))


def test_header_declares_the_reference_interface():
    names = declared_symbols()
    for method in ("create", "destroy", "update_locations", "get_sum_of_increments",
                   "get_log_likelihood_gradient", "store_state", "restore_state", "accept_state",
                   "set_pairwise_data", "set_parameters", "make_dirty", "get_internal_dimension"):
        assert f"mdsx_{method}" in names


def test_library_exports_every_declared_symbol(mdsx_lib):
    from massivemds_gb300 import _lib

    for name in declared_symbols():
        assert hasattr(mdsx_lib, name), name
        assert name in _lib.SIGNATURES, name


def test_version(mdsx_lib):
    assert mdsx_lib.mdsx_version().startswith(b"mdsx")


def test_argument_checks_before_any_device_work(mdsx_lib):
    from massivemds_gb300 import _lib

    h = ctypes.c_void_p()
    assert mdsx_lib.mdsx_create(0, 10, 0, -1, ctypes.byref(h)) == 1      # P < 1
    assert b"embeddingDimension" in mdsx_lib.mdsx_last_error(None)
    assert mdsx_lib.mdsx_create(11, 10, 0, -1, ctypes.byref(h)) == 6     # P > MDSX_MAX_DIMENSION
    assert mdsx_lib.mdsx_create(2, 0, 0, -1, ctypes.byref(h)) == 1       # N < 1
    assert mdsx_lib.mdsx_create(2, 10, 0, -1, None) == 1                 # out NULL
    for fn in ("mdsx_store_state", "mdsx_restore_state", "mdsx_accept_state", "mdsx_make_dirty",
               "mdsx_destroy"):
        assert getattr(mdsx_lib, fn)(None) == 1
    assert _lib.STATUS_NAMES[1] == "MDSX_EINVAL"


def test_create_without_gpu_fails_loudly(mdsx_lib):
    """No silent CPU fallback: on a machine without a GPU, creation reports ECUDA."""
    h = ctypes.c_void_p()
    rc = mdsx_lib.mdsx_create(2, 16, 0, -1, ctypes.byref(h))
    if rc == 0:  # a GPU is present
        mdsx_lib.mdsx_destroy(h)
        pytest.skip("a GPU is present")
    assert rc == 3
    assert mdsx_lib.mdsx_last_error(None)


def test_python_engine_raises_without_gpu(mdsx_lib):
    import massivemds_gb300 as m

    try:
        e = m.Engine(2, 16, m.flags.LEFT_TRUNCATION)
    except m.MdsxError as err:
        assert err.status == 3
    else:
        e.close()
        pytest.skip("a GPU is present")


def test_r_api_validation_messages():
    import massivemds_gb300 as m

    eng = m.MdsEngine(engine=None, embeddingDimension=2, locationCount=3, dataInitialized=False,
                      locationsInitialized=False, precision=None)
    with pytest.raises(RuntimeError, match="data are not set"):
        m.getLogLikelihood(eng)
    with pytest.raises(ValueError, match="Invalid data size"):
        m.setPairwiseData(eng, [1.0, 2.0])
    with pytest.raises(ValueError):
        m.factory(2, 3, m.flags.TBB)


def _compile_dropin(extra):
    gxx = shutil.which("g++")
    if not gxx:
        pytest.skip("g++ not available")
    src = ("#include \"mdsx/CudaMultiDimensionalScaling.hpp\"\n"
           "int main() { mds::SharedPtr p; (void)p; "
           "auto f = &mds::constructCudaMultiDimensionalScaling; (void)f; return 0; }\n")
    res = subprocess.run([gxx, "-std=c++17", "-fsyntax-only", "-x", "c++", "-", "-I", os.path.join(REPO, "include"),
                          *extra], input=src, capture_output=True, text=True)
    assert res.returncode == 0, res.stderr


def test_dropin_header_compiles_against_restated_interface():
    _compile_dropin([])


@pytest.mark.skipif(not REF_SRC, reason="reference sources not present")
def test_dropin_header_compiles_against_reference_header():
    shim = os.path.join(REPO, "oracle", "shim")
    _compile_dropin(["-DMDSX_USE_REFERENCE_HEADER", "-I", REF_SRC, "-I", shim])
