"""GPU parity tests of the double-float pair math (MDSX_FLAG_DOUBLE_FLOAT): the
FP64 modes' accuracy from FP32 arithmetic (csrc/dd.h, csrc/normal_dd.h), held to
the FP64 bars against the reference engine's golden vectors and the FP64 oracle:
sum of increments within 1e-10 relative, gradient within 1e-9 norm-relative
(max |dg| / max |g|).

Modes: "dd" = double-float pairs over FP64-stored delta (kept as (hi, lo) float
pairs), "dd32" = over FP32-stored delta (DELTA_F32; the oracle then runs on the
FP32-rounded delta). Both run on the unordered-pair schedule, P <= 6.
"""
import numpy as np
import pytest

import oracle
from massivemds_gb300 import Engine, MdsxError, flags as F

pytestmark = pytest.mark.gpu

TOL_SUM, TOL_GRAD = 1e-10, 1e-9
MODES = {"dd": F.DOUBLE_FLOAT, "dd32": F.DOUBLE_FLOAT | F.DELTA_F32}


def rel(a, b):
    return abs(a - b) / max(abs(b), 1e-300)


def grad_rel(g, ref):
    g = np.asarray(g).reshape(ref.shape)
    return np.abs(g - ref).max() / max(np.abs(ref).max(), 1e-300)


def inputs(n, p, seed, nans=0, asym=False):
    rng = np.random.default_rng(seed)
    y = rng.standard_normal((n, 6))
    delta = np.sqrt(((y[:, None] - y[None]) ** 2).sum(-1))
    if asym:
        delta = delta * (1.0 + 0.1 * rng.random((n, n)))
        np.fill_diagonal(delta, 0.0)
    for _ in range(nans):
        i, j = rng.choice(n, 2, replace=False)
        delta[i, j] = np.nan
    return delta, rng.standard_normal((n, p))


def make(mode, n, p, trunc, delta, x, tau):
    e = Engine(p, n, MODES[mode] | (F.LEFT_TRUNCATION if trunc else 0))
    e.setPairwiseData(delta)
    e.updateLocations(-1, x)
    e.setParameters([tau])
    return e


def odelta(delta, mode):
    return delta.astype(np.float32).astype(np.float64) if mode == "dd32" else delta


def check(mode, n, p, trunc, delta, x, tau):
    e = make(mode, n, p, trunc, delta, x, tau)
    try:
        s, g = e.getSumOfIncrements(), e.getLogLikelihoodGradient()
        assert e.sweep_schedule() == F.SWEEP_PAIRS
    finally:
        e.close()
    d = odelta(delta, mode)
    return s, g, oracle.sum_of_increments(d, x, tau, trunc), oracle.gradient(d, x, tau, trunc)


@pytest.fixture(scope="module")
def golden():
    import os
    z = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "golden.npz"))
    return {k: z[k] for k in z.files}


def test_matches_reference_golden(golden):
    """The reference's double engine on its golden cases (those with P <= 6)."""
    names = sorted({k.rsplit(".", 1)[0] for k in golden if k.endswith(".meta")})
    checked = 0
    for name in names:
        n, p, trunc, tau, use_float = golden[f"{name}.meta"]
        n, p, trunc = int(n), int(p), bool(trunc)
        if use_float or p > 6:
            continue
        delta, x = golden[f"{name}.delta"], golden[f"{name}.x"]
        e = make("dd", n, p, trunc, delta, x, float(tau))
        s, g = e.getSumOfIncrements(), e.getLogLikelihoodGradient()
        e.close()
        assert rel(s, float(golden[f"{name}.sum"])) < TOL_SUM, name
        assert grad_rel(g, golden[f"{name}.grad"].reshape(n, p)) < TOL_GRAD, name
        checked += 1
    assert checked >= 3


def test_reference_call_sequence_golden(golden):
    """store / update / sum / restore-or-accept / gradient (src/benchmark.cpp:250-309)."""
    delta, x0, tau = golden["seq.delta"], golden["seq.x0"], float(golden["seq.tau"])
    n, p = x0.shape
    e = make("dd", n, p, True, delta, x0, tau)
    assert rel(e.getSumOfIncrements(), golden["seq.sums"][0]) < TOL_SUM
    for k, (xn, restore) in enumerate(zip(golden["seq.xs"], golden["seq.restores"])):
        e.storeState()
        e.updateLocations(-1, xn)
        assert rel(e.getSumOfIncrements(), golden["seq.sums"][k + 1]) < TOL_SUM, k
        if restore:
            e.restoreState()
        else:
            e.acceptState()
        assert grad_rel(e.getLogLikelihoodGradient(), golden["seq.grads"][k + 1]) < TOL_GRAD, k
    e.close()


@pytest.mark.parametrize("mode", list(MODES))
@pytest.mark.parametrize("n", [2, 3, 5, 31, 32, 33, 127, 128, 129, 161, 257, 1000])
def test_sizes_and_edges(mode, n):
    p, tau = 2, 1.7
    delta, x = inputs(n, p, seed=n, nans=min(3, n // 10))
    for trunc in (True, False):
        s, g, s_ref, g_ref = check(mode, n, p, trunc, delta, x, tau)
        assert rel(s, s_ref) < TOL_SUM, (trunc, s, s_ref)
        assert grad_rel(g, g_ref) < TOL_GRAD, trunc


def test_single_location_and_fp32_input():
    """N = 1 (no pair: zero sum and gradient), and FP32 input data widened into
    the FP64-stored double-float layout."""
    e = make("dd", 1, 2, True, np.zeros((1, 1)), np.ones((1, 2)), 1.0)
    assert e.getSumOfIncrements() == 0.0 and np.all(e.getLogLikelihoodGradient() == 0.0)
    e.close()
    n, p, tau = 300, 2, 1.1
    delta, x = inputs(n, p, seed=63, nans=3)
    d32 = delta.astype(np.float32)
    s, g, s_ref, g_ref = check("dd", n, p, True, d32, x, tau)
    s_ref = oracle.sum_of_increments(d32.astype(np.float64), x, tau)
    g_ref = oracle.gradient(d32.astype(np.float64), x, tau)
    assert rel(s, s_ref) < TOL_SUM
    assert grad_rel(g, g_ref) < TOL_GRAD


@pytest.mark.parametrize("mode", list(MODES))
@pytest.mark.parametrize("p", [1, 3, 4, 5, 6])
def test_dimensions(mode, p):
    n, tau = 300, 0.8
    delta, x = inputs(n, p, seed=100 + p, nans=2, asym=True)
    for trunc in (True, False):
        s, g, s_ref, g_ref = check(mode, n, p, trunc, delta, x, tau)
        assert rel(s, s_ref) < TOL_SUM
        assert grad_rel(g, g_ref) < TOL_GRAD


def test_nan_rows_and_asymmetric_delta():
    n, p, tau = 400, 2, 2.0
    delta, x = inputs(n, p, seed=7, asym=True)
    delta[5, :] = np.nan
    delta[:, 9] = np.nan
    delta[100, 101] = np.nan
    for mode in MODES:
        s, g, s_ref, g_ref = check(mode, n, p, True, delta, x, tau)
        assert rel(s, s_ref) < TOL_SUM
        assert grad_rel(g, g_ref) < TOL_GRAD
        assert np.all(np.asarray(g).reshape(n, p)[5] == 0.0)


@pytest.mark.parametrize("tau", [1e-4, 1e-3, 0.05, 40.0, 400.0, 900.0])
def test_precision_extremes_and_tails(tau):
    """z = d sqrt(tau) near 0 (Phi ~ 1/2 for every pair) and far beyond the
    table's range (Q and phi below 1e-16), with missing pairs and asymmetry."""
    n, p = 300, 2
    delta, x = inputs(n, p, seed=80, nans=6, asym=True)
    for mode in MODES:
        s, g, s_ref, g_ref = check(mode, n, p, True, delta, x, tau)
        assert rel(s, s_ref) < TOL_SUM, (mode, tau)
        assert grad_rel(g, g_ref) < TOL_GRAD, (mode, tau)


def test_scaled_locations():
    """Locations far from unit scale (1e-3 and 1e3) and offset by 1e4: the
    double-float differences keep the FP64 bars."""
    n, p = 400, 2
    delta, x = inputs(n, p, seed=81)
    for scale, shift, tau in ((1e-3, 0.0, 1e6), (1e3, 0.0, 1e-6), (1.0, 1e4, 1.0)):
        xs = x * scale + shift
        ds = delta * scale
        for mode in MODES:
            s, g, s_ref, g_ref = check(mode, n, p, True, ds, xs, tau)
            assert rel(s, s_ref) < TOL_SUM, (mode, scale, shift)
            assert grad_rel(g, g_ref) < TOL_GRAD, (mode, scale, shift)


def test_coincident_points():
    """d = 0 for a non-missing pair: finite likelihood term, NaN gradient rows,
    as the reference and the FP64 modes give; every other row matches."""
    n, p, tau = 200, 2, 1.3
    delta, x = inputs(n, p, seed=60)
    x[7] = x[3]
    s_ref = oracle.sum_of_increments(delta, x, tau)
    with np.errstate(invalid="ignore", divide="ignore"):
        g_ref = oracle.gradient(delta, x, tau)
    e = make("dd", n, p, True, delta, x, tau)
    s, g = e.getSumOfIncrements(), np.asarray(e.getLogLikelihoodGradient()).reshape(n, p)
    e.close()
    assert np.isfinite(s) and rel(s, s_ref) < TOL_SUM
    rest = np.setdiff1d(np.arange(n), [3, 7])
    assert grad_rel(g[rest], g_ref[rest]) < TOL_GRAD
    assert np.isnan(g[[3, 7]]).all()


def test_single_location_updates_restore_and_determinism():
    n, p, tau = 500, 3, 2.0
    delta, x = inputs(n, p, seed=61)
    e = make("dd", n, p, True, delta, x, tau)
    s0, g0 = e.getSumOfIncrements(), e.getLogLikelihoodGradient().copy()
    e.makeDirty()
    assert e.getSumOfIncrements() == s0 and np.array_equal(e.getLogLikelihoodGradient(), g0)
    e.storeState()
    x2 = x.copy()
    x2[17] += 0.3
    x2[400] -= 0.2
    e.updateLocations(17, x2[17])
    e.updateLocations(400, x2[400])
    assert rel(e.getSumOfIncrements(), oracle.sum_of_increments(delta, x2, tau)) < TOL_SUM
    assert grad_rel(e.getLogLikelihoodGradient(), oracle.gradient(delta, x2, tau)) < TOL_GRAD
    e.restoreState()
    assert e.getSumOfIncrements() == s0
    assert np.array_equal(e.getLogLikelihoodGradient(), g0)
    e.close()


def test_device_api_matches_host_api():
    torch = pytest.importorskip("torch")
    n, p, tau = 700, 2, 2.0
    delta, x = inputs(n, p, seed=16)
    for mode in MODES:
        e = make(mode, n, p, True, delta, x, tau)
        s_host, g_host = e.getSumOfIncrements(), e.getLogLikelihoodGradient().copy()
        dx = torch.tensor(x, dtype=torch.float64, device="cuda")
        dsum = torch.zeros(1, dtype=torch.float64, device="cuda")
        dgrad = torch.zeros(n * p, dtype=torch.float64, device="cuda")
        stream = torch.cuda.Stream()
        e.set_stream(stream.cuda_stream)
        e.update_locations_device(dx.data_ptr())
        e.evaluate_device(dsum.data_ptr(), dgrad.data_ptr())
        stream.synchronize()
        assert e.last_launch_count() == 2
        assert float(dsum.item()) == s_host
        assert np.array_equal(dgrad.cpu().numpy(), g_host)
        e.set_stream(None)
        e.close()


def test_unsupported_combinations():
    n = 64
    delta, x = inputs(n, 2, seed=62)
    with pytest.raises(MdsxError) as err:
        Engine(7, n, F.DOUBLE_FLOAT)
    assert err.value.status == 6  # EUNSUPPORTED: P > 6 has no unordered-pair schedule
    with pytest.raises(MdsxError) as err:
        Engine(2, n, F.DOUBLE_FLOAT, rows=(0, 32))
    assert err.value.status == 6
    e = make("dd", n, 2, True, delta, x, 1.0)
    with pytest.raises(MdsxError) as err:
        e.set_sweep_schedule(F.SWEEP_ROWS)
    assert err.value.status == 6
    from massivemds_gb300.hmc import hmc
    with pytest.raises(MdsxError) as err:
        hmc(e, x, iterations=2)
    assert err.value.status == 6
    e.close()
