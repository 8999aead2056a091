"""GPU tests of the allocation-free sweep entry point, mdsx_sweep_f32_noalloc.

That entry point exists for callers that cannot allocate device memory (hosts
whose GPU memory belongs to another allocator, loops that must not call
cudaMalloc/cudaFree): it keeps every intermediate in a static device array and
uses only the caller's buffers for delta, locations and results. Every call
here goes through the C ABI.

* Two calls in a row on the same buffers, each compared with the engine's own
  FP32 sweep (mdsx_evaluate_device) within the FP32 tolerance the other parity
  tests use; the second call checks that the shared scratch, which keeps the
  previous call's contents, is re-initialised.
* Small and ragged sizes, P = 1, 3, 6, 10, missing pairs in one direction and
  whole missing rows, truncation on and off, against the FP64 oracle on the
  same FP32 delta (1e-5). Delta with NaN takes the call's second pass (scan
  for NaN rows, sweep again); delta without NaN is read once.
* The stated limit: N = MDSX_NOALLOC_MAX_LOCATIONS fits the static array for
  every P = 1..10 (gradient rows checked against the oracle), and N one above
  it is rejected with MDSX_EINVAL.

This file is collected last so a failure here leaves every other test run.
"""
import numpy as np
import pytest

import oracle
from massivemds_gb300 import Engine, flags as F
from massivemds_gb300._lib import load

pytestmark = pytest.mark.gpu

TOL_F32 = 1e-5  # the FP32 tolerance of tests/test_engine_gpu.py
MAX_LOCATIONS = 32768  # MDSX_NOALLOC_MAX_LOCATIONS


def rel(a, b):
    return abs(a - b) / max(abs(b), 1e-300)


def grad_rel(g, ref):
    return np.abs(g - ref).max() / max(np.abs(ref).max(), 1e-300)


def _inputs(n, p, seed, nan_pairs=0, nan_rows=0):
    rng = np.random.default_rng(seed)
    y = rng.standard_normal((n, 10))
    delta = np.sqrt(((y[:, None] - y[None]) ** 2).sum(-1)).astype(np.float32)
    for _ in range(nan_pairs if n > 1 else 0):
        i, j = rng.choice(n, 2, replace=False)
        delta[i, j] = np.nan  # one direction only
    for _ in range(nan_rows if n > 2 else 0):
        i = int(rng.integers(n))
        delta[i, :] = np.nan
        delta[:, i] = np.nan
    return delta, rng.standard_normal((n, p))


def _device_delta(torch, delta):
    """delta in a caller-owned device buffer with a padded row stride."""
    n = delta.shape[0]
    ld = (n + 3) // 4 * 4
    d = torch.full((n, ld), float("nan"), dtype=torch.float32, device="cuda")
    d[:, :n] = torch.from_numpy(delta).cuda()
    return d, ld


def _call(torch, lib, ddelta, ld, dx, n, p, tau, truncation):
    out_sum = torch.full((1,), float("nan"), dtype=torch.float64, device="cuda")
    out_grad = torch.full((n * p,), float("nan"), dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    rc = lib.mdsx_sweep_f32_noalloc(ddelta.data_ptr(), ld, dx.data_ptr(), n, p, tau, int(truncation),
                                    out_sum.data_ptr(), out_grad.data_ptr(), torch.cuda.current_stream().cuda_stream)
    assert rc == 0, lib.mdsx_last_error(None)
    torch.cuda.synchronize()
    return float(out_sum.item()), out_grad.cpu().numpy().reshape(n, p)


@pytest.mark.parametrize("p", [1, 2, 3, 6])
@pytest.mark.parametrize("truncation", [True, False])
def test_noalloc_matches_engine_twice(truncation, p):
    torch = pytest.importorskip("torch")
    lib = load()
    n, tau = 3001, 2.0
    delta, x = _inputs(n, p, seed=31 + p, nan_pairs=1)

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
    s_ref, g_ref = float(ref_sum.item()), ref_grad.cpu().numpy().reshape(n, p)
    eng.close()

    ddelta, ld = _device_delta(torch, delta)
    for call in range(2):
        s, g = _call(torch, lib, ddelta, ld, dx, n, p, tau, truncation)
        assert rel(s, s_ref) < TOL_F32, call
        assert grad_rel(g, g_ref) < TOL_F32, call


@pytest.mark.parametrize("n", [1, 2, 3, 33, 129, 257, 1000])
@pytest.mark.parametrize("p", [1, 3, 6, 10])
@pytest.mark.parametrize("missing", ["none", "pairs", "rows"])
@pytest.mark.parametrize("truncation", [True, False])
def test_noalloc_matches_oracle(n, p, missing, truncation):
    torch = pytest.importorskip("torch")
    lib = load()
    tau = 1.7
    delta, x = _inputs(n, p, seed=1000 * n + p, nan_pairs=3 if missing == "pairs" else 0,
                       nan_rows=1 if missing == "rows" else 0)
    s_ref = oracle.sum_of_increments(delta, x, tau, truncation)
    g_ref = oracle.gradient(delta, x, tau, truncation)
    ddelta, ld = _device_delta(torch, delta)
    dx = torch.tensor(x, dtype=torch.float64, device="cuda")
    s, g = _call(torch, lib, ddelta, ld, dx, n, p, tau, truncation)
    if n == 1:
        assert s == 0.0 and not np.any(g)
        return
    assert rel(s, s_ref) < TOL_F32
    assert grad_rel(g, g_ref) < TOL_F32


def test_noalloc_fits_its_stated_limit_for_every_dimension():
    """N = MDSX_NOALLOC_MAX_LOCATIONS: the plan fits the static array for P = 1..10."""
    torch = pytest.importorskip("torch")
    lib = load()
    n, tau, rows = MAX_LOCATIONS, 2.0, 64
    gen = torch.Generator(device="cuda").manual_seed(7)
    ddelta = torch.rand((n, n), generator=gen, dtype=torch.float32, device="cuda").mul_(4.0)
    top = ddelta[:rows].cpu().numpy()  # rows [0, 64) for the oracle
    rng = np.random.default_rng(8)
    for p in range(1, 11):
        x = rng.standard_normal((n, p))
        dx = torch.tensor(x, dtype=torch.float64, device="cuda")
        s, g = _call(torch, lib, ddelta, n, dx, n, p, tau, True)
        assert np.isfinite(s), p
        _, g_ref = oracle.sweep_rows(top, x, tau, True, 0, rows)
        assert grad_rel(g[:rows], g_ref) < TOL_F32, p
    del ddelta
    torch.cuda.empty_cache()


def test_noalloc_rejects_sizes_beyond_its_scratch():
    torch = pytest.importorskip("torch")
    lib = load()
    dummy = torch.zeros(16, dtype=torch.float64, device="cuda")
    n = MAX_LOCATIONS + 1
    rc = lib.mdsx_sweep_f32_noalloc(dummy.data_ptr(), n + 3, dummy.data_ptr(), n, 2, 1.0, 1, dummy.data_ptr(),
                                    dummy.data_ptr(), None)
    assert rc == 1
    assert b"MDSX_NOALLOC_MAX_LOCATIONS" in lib.mdsx_last_error(None)
