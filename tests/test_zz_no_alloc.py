"""GPU test of the allocation-free sweep entry point, mdsx_sweep_f32_noalloc.

That entry point exists for callers that cannot allocate device memory (hosts
whose GPU memory belongs to another allocator, loops that must not call
cudaMalloc/cudaFree): it keeps every intermediate in a static device array and
uses only the caller's buffers for delta, locations and results. Here it is
called through the C ABI, twice in a row on the same buffers, and each result
is compared with the engine's own FP32 sweep (mdsx_evaluate_device) within the
FP32 tolerance the other parity tests use. The second call checks that the
shared scratch, which keeps the previous call's contents, is re-initialised.

This file is collected last so a failure here leaves every other test run.
"""
import ctypes

import numpy as np
import pytest

from massivemds_gb300 import Engine, flags as F
from massivemds_gb300._lib import load

pytestmark = pytest.mark.gpu

TOL_F32 = 1e-5  # the FP32 tolerance of tests/test_engine_gpu.py


def rel(a, b):
    return abs(a - b) / max(abs(b), 1e-300)


def grad_rel(g, ref):
    return np.abs(g - ref).max() / max(np.abs(ref).max(), 1e-300)


def _inputs(n, p, seed):
    rng = np.random.default_rng(seed)
    y = rng.standard_normal((n, 10))
    delta = np.sqrt(((y[:, None] - y[None]) ** 2).sum(-1)).astype(np.float32)
    delta[3, 11] = np.nan  # a missing pair
    return delta, rng.standard_normal((n, p))


@pytest.mark.parametrize("truncation", [True, False])
def test_noalloc_matches_engine_twice(truncation):
    torch = pytest.importorskip("torch")
    lib = load()
    n, p, tau = 3001, 2, 2.0
    delta, x = _inputs(n, p, seed=31)

    # the existing entry point: the engine's device-resident sweep
    flags = F.FLOAT | (F.LEFT_TRUNCATION if truncation else 0)
    eng = Engine(p, n, flags)
    eng.setPairwiseData(delta)
    eng.setParameters([tau])
    dx = torch.tensor(x, dtype=torch.float64, device="cuda")
    ref_sum = torch.zeros(1, dtype=torch.float64, device="cuda")
    ref_grad = torch.zeros(n * p, dtype=torch.float64, device="cuda")
    eng.update_locations_device(dx.data_ptr())
    eng.evaluate_device(ref_sum.data_ptr(), ref_grad.data_ptr())
    torch.cuda.synchronize()
    s_ref, g_ref = float(ref_sum.item()), ref_grad.cpu().numpy()
    eng.close()

    # caller-owned buffers for the allocation-free call: delta with a padded row stride
    ld = (n + 3) // 4 * 4
    ddelta = torch.full((n, ld), float("nan"), dtype=torch.float32, device="cuda")
    ddelta[:, :n] = torch.from_numpy(delta).cuda()
    out_sum = torch.zeros(1, dtype=torch.float64, device="cuda")
    out_grad = torch.zeros(n * p, dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    for call in range(2):
        out_sum.fill_(0.0)
        out_grad.fill_(0.0)
        torch.cuda.synchronize()
        rc = lib.mdsx_sweep_f32_noalloc(ddelta.data_ptr(), ld, dx.data_ptr(), n, p, tau, int(truncation),
                                        out_sum.data_ptr(), out_grad.data_ptr(), stream)
        assert rc == 0, lib.mdsx_last_error(None)
        torch.cuda.synchronize()
        assert rel(float(out_sum.item()), s_ref) < TOL_F32, call
        assert grad_rel(out_grad.cpu().numpy(), g_ref) < TOL_F32, call


def test_noalloc_rejects_sizes_beyond_its_scratch():
    torch = pytest.importorskip("torch")
    lib = load()
    dummy = torch.zeros(16, dtype=torch.float64, device="cuda")
    n = 32769  # one above MDSX_NOALLOC_MAX_LOCATIONS
    rc = lib.mdsx_sweep_f32_noalloc(dummy.data_ptr(), n + 3, dummy.data_ptr(), n, 2, 1.0, 1, dummy.data_ptr(),
                                    dummy.data_ptr(), None)
    assert rc == 1
    assert b"MDSX_NOALLOC_MAX_LOCATIONS" in lib.mdsx_last_error(None)
