"""GPU parity tests: the CUDA engine, called through the C ABI, against the
reference engine's golden vectors and the FP64 oracle.

Tolerances (from the engine's stated targets):
  FP64 mode (and FP64 over FP32-stored delta): sum of increments within 1e-10
    relative, gradient within 1e-9 norm-relative (max |dg| / max |g|).
  FP32 mode (FP32 pairs, compensated FP32 partials, FP64 reductions): within
    1e-5 relative of the FP64 oracle on the same (FP32-rounded) delta, with
    either sweep schedule: "f32" is the engine's default (unordered pairs for
    P <= 6 with truncation, else row blocks), "f32rows" and "f32pairs" force one;
    the same for FP64 over FP32-stored delta ("f64s32", "f64s32rows", "f64s32pairs")
    and over FP64-stored delta ("f64", "f64rows", "f64pairs").
"""
import numpy as np
import pytest

import oracle
from massivemds_gb300 import Engine, MdsxError, flags as F
from massivemds_gb300 import data as gen

pytestmark = pytest.mark.gpu

TOL_F64_SUM, TOL_F64_GRAD = 1e-10, 1e-9
TOL_F32 = 1e-5


def rel(a, b):
    return abs(a - b) / max(abs(b), 1e-300)


def grad_rel(g, ref):
    g = np.asarray(g).reshape(ref.shape)
    return np.abs(g - ref).max() / max(np.abs(ref).max(), 1e-300)


def make_engine(n, p, trunc, mode, delta, x, tau):
    fl = F.LEFT_TRUNCATION if trunc else 0
    fl |= {"f64": 0, "f64rows": 0, "f64pairs": 0, "f32": F.FLOAT, "f32rows": F.FLOAT, "f32pairs": F.FLOAT,
           "f64s32": F.DELTA_F32, "f64s32rows": F.DELTA_F32, "f64s32pairs": F.DELTA_F32}[mode]
    e = Engine(p, n, fl)
    if mode.endswith("rows"):
        e.set_sweep_schedule(F.SWEEP_ROWS)
    if mode.endswith("pairs"):
        e.set_sweep_schedule(F.SWEEP_PAIRS)
    e.setPairwiseData(delta)
    e.updateLocations(-1, x)
    e.setParameters([tau])
    e.makeDirty()
    return e


def oracle_delta(delta, mode):
    return delta if mode.startswith("f64") and not mode.startswith("f64s32") else delta.astype(np.float32)


def tolerances(mode):
    return (TOL_F32, TOL_F32) if mode in ("f32", "f32rows", "f32pairs") else (TOL_F64_SUM, TOL_F64_GRAD)


# ------------------------------------------------------------- golden vectors

@pytest.mark.parametrize("mode", ["f64rows", "f64pairs"])
def test_fp64_matches_reference_golden(golden, mode):
    data, cases = golden
    for name in cases:
        n, p, trunc, tau, use_float = data[f"{name}.meta"]
        if use_float:
            continue
        n, p = int(n), int(p)
        if mode == "f64pairs" and p > 6:
            continue
        e = make_engine(n, p, bool(trunc), mode, data[f"{name}.delta"], data[f"{name}.x"], tau)
        s = e.getSumOfIncrements()
        g = e.getLogLikelihoodGradient()
        e.close()
        ref_g = data[f"{name}.grad"].reshape(n, p)
        assert rel(s, float(data[f"{name}.sum"])) < TOL_F64_SUM, name
        assert grad_rel(g, ref_g) < TOL_F64_GRAD, name


def test_fp32_matches_oracle_on_golden_inputs(golden):
    data, cases = golden
    for name in cases:
        n, p, trunc, tau, _ = data[f"{name}.meta"]
        n, p = int(n), int(p)
        delta, x = data[f"{name}.delta"], data[f"{name}.x"]
        e = make_engine(n, p, bool(trunc), "f32", delta, x, tau)
        s, g = e.getSumOfIncrements(), e.getLogLikelihoodGradient()
        e.close()
        d32 = delta.astype(np.float32)
        assert rel(s, oracle.sum_of_increments(d32, x, tau, bool(trunc))) < TOL_F32, name
        assert grad_rel(g, oracle.gradient(d32, x, tau, bool(trunc))) < TOL_F32, name


def test_reference_call_sequence_golden(golden):
    """The reference benchmark's store/update/sum/restore-or-accept/gradient loop
    (src/benchmark.cpp:250-309) gives the reference engine's sums and gradients."""
    data, _ = golden
    delta, x0, tau = data["seq.delta"], data["seq.x0"], float(data["seq.tau"])
    n, p = x0.shape
    for mode in ("f64rows", "f64pairs", "f32rows", "f32pairs"):
        tol_s, tol_g = tolerances(mode)
        e = make_engine(n, p, True, mode, delta, x0, tau)
        assert rel(e.getSumOfIncrements(), data["seq.sums"][0]) < tol_s
        for k, (xn, restore) in enumerate(zip(data["seq.xs"], data["seq.restores"])):
            e.storeState()
            e.updateLocations(-1, xn)
            assert rel(e.getSumOfIncrements(), data["seq.sums"][k + 1]) < tol_s, (mode, k)
            if restore:
                e.restoreState()
            else:
                e.acceptState()
            assert grad_rel(e.getLogLikelihoodGradient(), data["seq.grads"][k + 1]) < tol_g, (mode, k)
        e.close()


# ----------------------------------------------------------- random coverage

def _inputs(n, p, seed, nans=0, asym=False):
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


@pytest.mark.parametrize("mode", ["f64rows", "f64pairs", "f32rows", "f32pairs", "f64s32rows", "f64s32pairs"])
@pytest.mark.parametrize("n", [1, 2, 3, 5, 31, 32, 33, 127, 128, 129, 159, 160, 161, 257, 385, 1000])
def test_sizes_and_edges(mode, n):
    p, tau = 2, 1.7
    delta, x = _inputs(n, p, seed=n, nans=min(3, n // 10))
    tol_s, tol_g = tolerances(mode)
    for trunc in (True, False):
        e = make_engine(n, p, trunc, mode, delta, x, tau)
        s, g = e.getSumOfIncrements(), e.getLogLikelihoodGradient()
        e.close()
        od = oracle_delta(delta, mode)
        s_ref = oracle.sum_of_increments(od, x, tau, trunc)
        g_ref = oracle.gradient(od, x, tau, trunc)
        if n == 1:
            assert s == 0.0 and np.all(g == 0.0)
            continue
        assert rel(s, s_ref) < tol_s, (trunc, s, s_ref)
        assert grad_rel(g, g_ref) < tol_g, trunc


@pytest.mark.parametrize("mode", ["f64rows", "f64pairs", "f32rows", "f32pairs", "f64s32pairs"])
@pytest.mark.parametrize("p", [1, 3, 4, 5, 6, 7, 8, 9, 10])
def test_dimensions(mode, p):
    if mode.endswith("pairs") and p > 6:
        pytest.skip("the unordered-pair schedule is built for P <= 6")
    n, tau = 300, 0.8
    delta, x = _inputs(n, p, seed=100 + p, nans=2, asym=True)
    tol_s, tol_g = tolerances(mode)
    for trunc in (True, False):
        e = make_engine(n, p, trunc, mode, delta, x, tau)
        s, g = e.getSumOfIncrements(), e.getLogLikelihoodGradient()
        e.close()
        od = oracle_delta(delta, mode)
        assert rel(s, oracle.sum_of_increments(od, x, tau, trunc)) < tol_s
        assert grad_rel(g, oracle.gradient(od, x, tau, trunc)) < tol_g


def test_nan_rows_and_asymmetric_delta():
    n, p, tau = 400, 2, 2.0
    delta, x = _inputs(n, p, seed=7, nans=0, asym=True)
    delta[5, :] = np.nan       # a whole row missing
    delta[:, 9] = np.nan       # a whole column missing
    delta[100, 101] = np.nan
    for mode in ("f64rows", "f64pairs", "f32rows", "f32pairs", "f64s32pairs"):
        tol_s, tol_g = tolerances(mode)
        e = make_engine(n, p, True, mode, delta, x, tau)
        s, g = e.getSumOfIncrements(), e.getLogLikelihoodGradient()
        e.close()
        od = oracle_delta(delta, mode)
        assert rel(s, oracle.sum_of_increments(od, x, tau)) < tol_s
        gr = oracle.gradient(od, x, tau)
        assert grad_rel(g, gr) < tol_g
        assert np.all(np.asarray(g).reshape(n, p)[5] == 0.0)  # row 5 has no observed pair


def test_precision_extremes():
    n, p = 500, 2
    delta, x = _inputs(n, p, seed=9)
    for tau in (1e-3, 0.05, 40.0, 900.0):
        for mode in ("f64rows", "f64pairs", "f32rows", "f32pairs", "f64s32pairs"):
            tol_s, tol_g = tolerances(mode)
            e = make_engine(n, p, True, mode, delta, x, tau)
            s, g = e.getSumOfIncrements(), e.getLogLikelihoodGradient()
            e.close()
            od = oracle_delta(delta, mode)
            assert rel(s, oracle.sum_of_increments(od, x, tau)) < tol_s, (mode, tau)
            assert grad_rel(g, oracle.gradient(od, x, tau)) < tol_g, (mode, tau)


# ------------------------------------------------------------ state machine

def test_single_location_update_and_caching():
    n, p, tau = 200, 3, 1.2
    delta, x = _inputs(n, p, seed=11)
    e = make_engine(n, p, True, "f64", delta, x, tau)
    s0 = e.getSumOfIncrements()
    x2 = x.copy()
    x2[17] = [0.3, -0.2, 1.1]
    e.updateLocations(17, x2[17])
    s1 = e.getSumOfIncrements()
    assert rel(s1, oracle.sum_of_increments(delta, x2, tau)) < TOL_F64_SUM
    assert s1 != s0
    g = e.getLogLikelihoodGradient()
    assert grad_rel(g, oracle.gradient(delta, x2, tau)) < TOL_F64_GRAD
    # setParameters invalidates; untruncated sums rescale with the new precision
    e.setParameters([2.4])
    assert rel(e.getSumOfIncrements(), oracle.sum_of_increments(delta, x2, 2.4)) < TOL_F64_SUM
    e.close()
    e = make_engine(n, p, False, "f64", delta, x, tau)
    e.getSumOfIncrements()
    e.setParameters([3.3])
    assert rel(e.getSumOfIncrements(), oracle.sum_of_increments(delta, x, 3.3, False)) < TOL_F64_SUM
    assert grad_rel(e.getLogLikelihoodGradient(), oracle.gradient(delta, x, 3.3, False)) < TOL_F64_GRAD
    assert e.getInternalDimension() == p
    e.close()


def test_restore_returns_stored_sum_without_sweep():
    """restoreState brings back the stored sum as known (src/NewMultiDimensionalScaling.hpp:234-236)."""
    n, p, tau = 100, 2, 1.0
    delta, x = _inputs(n, p, seed=12)
    e = make_engine(n, p, True, "f64", delta, x, tau)
    s0 = e.getSumOfIncrements()
    g0 = e.getLogLikelihoodGradient().copy()
    e.storeState()
    e.updateLocations(-1, 1.5 * x)  # a rigid shift would leave every distance unchanged
    assert e.getSumOfIncrements() != s0
    e.restoreState()
    assert e.getSumOfIncrements() == s0
    assert np.array_equal(e.getLogLikelihoodGradient(), g0)
    e.close()


def test_deterministic_bitwise():
    n, p, tau = 3000, 2, 2.0
    delta, x = _inputs(n, p, seed=13)
    for mode in ("f32rows", "f32pairs", "f64rows", "f64pairs", "f64s32pairs"):
        e = make_engine(n, p, True, mode, delta, x, tau)
        s1, g1 = e.getSumOfIncrements(), e.getLogLikelihoodGradient().copy()
        e.makeDirty()
        s2, g2 = e.getSumOfIncrements(), e.getLogLikelihoodGradient().copy()
        e.close()
        assert s1 == s2 and np.array_equal(g1, g2), mode


def test_log_likelihood_assembly():
    n, p, tau = 150, 2, 1.4
    delta, x = _inputs(n, p, seed=14)
    e = make_engine(n, p, True, "f64", delta, x, tau)
    ll = e.getLogLikelihood()
    s = oracle.sum_of_increments(delta, x, tau)
    assert rel(ll, oracle.log_likelihood(s, n, tau)) < TOL_F64_SUM
    e.close()


# ------------------------------------------------------------------- errors

def test_error_statuses():
    n, p = 50, 2
    delta, x = _inputs(n, p, seed=15)
    e = Engine(p, n, F.LEFT_TRUNCATION)
    with pytest.raises(MdsxError) as err:
        e.getSumOfIncrements()
    assert err.value.status == 5  # ESTATE: no data yet
    with pytest.raises(MdsxError) as err:
        e.setPairwiseData(delta[:-1])
    assert err.value.status == 1
    e.setPairwiseData(delta)
    with pytest.raises(MdsxError) as err:
        e.updateLocations(-1, x[:-1])
    assert err.value.status == 1
    with pytest.raises(MdsxError):
        e.updateLocations(n, x[0])
    with pytest.raises(MdsxError):
        e.setParameters([-1.0])
    with pytest.raises(MdsxError):
        e.setParameters([1.0, 2.0])
    e.updateLocations(-1, x)
    with pytest.raises(MdsxError) as err:
        e.getSumOfIncrements()
    assert err.value.status == 5  # precision not set
    e.setParameters([1.0])
    assert np.isfinite(e.getSumOfIncrements())
    with pytest.raises(ValueError):
        e.getLogLikelihoodGradient(np.empty(3))
    e.close()


def test_sweep_schedules():
    """Truncated engines and FP64 engines default to the unordered-pair
    schedule (sweep + finish kernel) where it is built (P <= 6), untruncated
    FP32 ones to the row-block schedule; beyond that range the engine runs the
    row-block schedule and refuses the pair schedule; switching invalidates the
    cached results."""
    n, tau = 300, 1.3
    delta, x = _inputs(n, 2, seed=29)
    e = make_engine(n, 2, False, "f32", delta, x, tau)
    assert e.sweep_schedule() == F.SWEEP_ROWS
    e.set_sweep_schedule(F.SWEEP_PAIRS)
    assert rel(e.getSumOfIncrements(), oracle.sum_of_increments(delta.astype(np.float32), x, tau, False)) < TOL_F32
    e.close()
    for mode in ("f64", "f64s32"):
        e = make_engine(n, 2, False, mode, delta, x, tau)
        assert e.sweep_schedule() == F.SWEEP_PAIRS, mode
        assert rel(e.getSumOfIncrements(), oracle.sum_of_increments(oracle_delta(delta, mode), x, tau, False)) \
            < TOL_F64_SUM
        e.close()
    for p, mode, default in ((2, "f32", F.SWEEP_PAIRS), (4, "f32", F.SWEEP_PAIRS), (6, "f32", F.SWEEP_PAIRS),
                             (7, "f32", F.SWEEP_ROWS), (2, "f64", F.SWEEP_PAIRS), (6, "f64", F.SWEEP_PAIRS),
                             (7, "f64", F.SWEEP_ROWS), (2, "f64s32", F.SWEEP_PAIRS), (5, "f64s32", F.SWEEP_PAIRS),
                             (8, "f64s32", F.SWEEP_ROWS)):
        delta, x = _inputs(n, p, seed=30 + p)
        e = make_engine(n, p, True, mode, delta, x, tau)
        assert e.sweep_schedule() == default, (p, mode)
        if default == F.SWEEP_ROWS:
            with pytest.raises(MdsxError) as err:
                e.set_sweep_schedule(F.SWEEP_PAIRS)
            assert err.value.status == 6  # EUNSUPPORTED
            e.close()
            continue
        s_pairs = e.getSumOfIncrements()
        g_pairs = e.getLogLikelihoodGradient().copy()
        assert e.last_launch_count() == 2
        e.set_sweep_schedule(F.SWEEP_ROWS)
        s_rows = e.getSumOfIncrements()
        assert e.last_launch_count() == 1
        g_rows = e.getLogLikelihoodGradient()
        tol_s, tol_g = tolerances(mode)
        assert rel(s_pairs, s_rows) < tol_s and grad_rel(g_pairs, g_rows.reshape(n, p)) < tol_g
        with pytest.raises(MdsxError):
            e.set_sweep_schedule(7)
        e.close()


def test_pair_schedule_symmetric_pairs_and_missing_blocks():
    """Unordered-pair schedule edge cases: asymmetric delta with NaN in one
    direction only (each direction keeps its own mask), NaN rows inside the
    diagonal blocks, coincident block boundaries and a ragged last block."""
    for n in (128, 256, 300, 641):
        p, tau = 2, 0.9
        delta, x = _inputs(n, p, seed=40 + n, asym=True)
        rng = np.random.default_rng(n)
        for _ in range(8):
            i, j = rng.choice(n, 2, replace=False)
            delta[i, j] = np.nan  # (j, i) stays observed
        delta[n // 2, :] = np.nan
        for trunc in (True, False):
            for mode in ("f32pairs", "f64s32pairs", "f64pairs"):
                e = make_engine(n, p, trunc, mode, delta, x, tau)
                assert e.sweep_schedule() == F.SWEEP_PAIRS
                s, g = e.getSumOfIncrements(), e.getLogLikelihoodGradient()
                e.close()
                od = oracle_delta(delta, mode)
                tol_s, tol_g = tolerances(mode)
                assert rel(s, oracle.sum_of_increments(od, x, tau, trunc)) < tol_s, (n, trunc, mode)
                assert grad_rel(g, oracle.gradient(od, x, tau, trunc)) < tol_g, (n, trunc, mode)


# ------------------------------------------------------- device-resident API

def test_device_api_matches_host_api():
    torch = pytest.importorskip("torch")
    n, p, tau = 700, 2, 2.0
    delta, x = _inputs(n, p, seed=16)
    for mode in ("f32rows", "f32pairs", "f64rows", "f64pairs"):
        e = make_engine(n, p, True, mode, delta, x, tau)
        s_host, g_host = e.getSumOfIncrements(), e.getLogLikelihoodGradient().copy()
        dx = torch.tensor(x, dtype=torch.float64, device="cuda")
        dsum = torch.zeros(1, dtype=torch.float64, device="cuda")
        dgrad = torch.zeros(n * p, dtype=torch.float64, device="cuda")
        stream = torch.cuda.Stream()
        e.set_stream(stream.cuda_stream)
        e.update_locations_device(dx.data_ptr())
        e.evaluate_device(dsum.data_ptr(), dgrad.data_ptr())
        stream.synchronize()
        assert e.last_launch_count() >= 1
        assert float(dsum.item()) == s_host
        assert np.array_equal(dgrad.cpu().numpy(), g_host)
        e.set_stream(None)
        e.close()


# ------------------------------------------------------------ full size (N=20k)
# tests/test_c2_full_gpu.py: the reference engine's golden vectors and twenty
# oracle states at N = 20 000 in every precision mode.


# ------------------------------------------------- bounded waits (failure path)

def test_bounded_wait_gives_up_and_context_stays_usable():
    """A kernel waiting on a barrier that never completes gives up after its
    limit, records the timeout code and returns; the GPU context stays usable
    (an engine evaluates correctly afterwards). The wait ends by its time limit:
    no fault or trap is involved."""
    import ctypes
    from massivemds_gb300 import _lib
    lib = _lib.load()
    code = ctypes.c_int(-1)
    status = lib.mdsx_selftest_bounded_wait(ctypes.c_double(0.2), -1, ctypes.byref(code))
    assert status == 4 and code.value == 1  # MDSX_ETIMEOUT, device code: consumer wait timed out
    n, p, tau = 200, 2, 1.5
    delta, x = _inputs(n, p, seed=50)
    e = make_engine(n, p, True, "f32", delta, x, tau)
    assert rel(e.getSumOfIncrements(), oracle.sum_of_increments(delta.astype(np.float32), x, tau)) < TOL_F32
    e.close()


def test_fp64_math_helpers():
    """The FP64 sweeps' Newton-refined reciprocal and reciprocal square root
    within 2 ulp of the correctly rounded values over the normal range, and their
    normal CDF / density (Phi = 1 - phi R with R the Mills-ratio fit, whose error
    in Q is 9.4e-16 evaluated in double) within 2e-15 absolute / the
    exponential's argument rounding of the exact values; 0 gives NaN
    reciprocals (coincident points)."""
    import ctypes
    from scipy.special import ndtr
    from massivemds_gb300 import _lib
    lib = _lib.load()
    rng = np.random.default_rng(70)
    x = np.concatenate([10.0 ** rng.uniform(-307, 307, 200000), rng.uniform(0.0, 40.0, 100000),
                        np.linspace(0.0, 9.0, 9001), [0.0, 1.0, 2.0, 0.5, 4.0, np.nextafter(1.0, 2.0),
                                                      np.nextafter(1.0, 0.0), 2.2250738585072014e-308, 38.6, 50.0,
                                                      1e3]])
    out = np.empty((x.size, 4))
    dp = ctypes.POINTER(ctypes.c_double)
    assert lib.mdsx_selftest_math_f64(x.ctypes.data_as(dp), x.size, out.ctypes.data_as(dp), -1) == 0
    pos = x >= 2.2250738585072014e-308
    xl = x[pos].astype(np.longdouble)
    ulp = 2.0 ** -52
    rcp_err = np.abs((out[pos, 0] - 1 / xl) * xl)
    rsq_err = np.abs((out[pos, 1] - 1 / np.sqrt(xl)) * np.sqrt(xl))
    assert rcp_err.max() <= 2 * ulp and rsq_err.max() <= 2 * ulp, (rcp_err.max() / ulp, rsq_err.max() / ulp)
    assert np.isnan(out[x == 0.0, 0]).all() and np.isnan(out[x == 0.0, 1]).all()
    z = x[x <= 1e3]
    assert np.abs(out[x <= 1e3, 2] - ndtr(z)).max() <= 2e-15
    zl = z.astype(np.longdouble)
    pdf = np.exp(-0.5 * zl * zl) / np.sqrt(2 * np.pi, dtype=np.longdouble)
    pdf_err = np.abs(out[x <= 1e3, 3] - pdf)
    bound = (0.5 * z * z + 4.0) * ulp * pdf + 1e-300
    assert np.all(pdf_err <= bound), float(np.max(pdf_err / bound))


@pytest.mark.parametrize("mode", ["f64rows", "f64pairs", "f64s32pairs", "f32pairs"])
@pytest.mark.parametrize("tau", [1e-4, 400.0])
def test_truncation_tails(mode, tau):
    """z = d sqrt(tau) near 0 (Phi ~ 1/2 for every pair) and far in the tail
    (z up to ~100: phi underflows, Phi = 1, the truncation terms vanish), with
    missing pairs and an asymmetric delta, against the oracle at the mode's bar."""
    n, p = 150, 2
    delta, x = _inputs(n, p, seed=80, nans=6, asym=True)
    tol_s, tol_g = tolerances(mode)
    e = make_engine(n, p, True, mode, delta, x, tau)
    s, g = e.getSumOfIncrements(), e.getLogLikelihoodGradient()
    e.close()
    d = oracle_delta(delta, mode)
    assert rel(s, oracle.sum_of_increments(d, x, tau)) < tol_s
    assert grad_rel(g, oracle.gradient(d, x, tau)) < tol_g


def test_coincident_points():
    """Two distinct rows at the same location (d = 0 for a non-missing pair): the
    reference takes d = sqrt(0) = 0, so the likelihood term is finite, and
    divides by d in the gradient, so the two rows' gradients are NaN. FP64 modes
    reproduce both; FP32 modes reproduce the likelihood and keep the two rows'
    gradients finite (d^2 starts from 1e-30); every other row matches."""
    n, p, tau = 200, 2, 1.3
    delta, x = _inputs(n, p, seed=60)
    x[7] = x[3]
    for mode in ("f64rows", "f64pairs", "f64s32pairs", "f32rows", "f32pairs"):
        tol_s, tol_g = tolerances(mode)
        od = oracle_delta(delta, mode)
        s_ref = oracle.sum_of_increments(od, x, tau)
        with np.errstate(invalid="ignore", divide="ignore"):
            g_ref = oracle.gradient(od, x, tau)
        assert np.isfinite(s_ref) and np.isnan(g_ref[[3, 7]]).all()
        e = make_engine(n, p, True, mode, delta, x, tau)
        s, g = e.getSumOfIncrements(), np.asarray(e.getLogLikelihoodGradient()).reshape(n, p)
        e.close()
        assert np.isfinite(s) and rel(s, s_ref) < tol_s, mode
        rest = np.setdiff1d(np.arange(n), [3, 7])
        assert grad_rel(g[rest], g_ref[rest]) < tol_g, mode
        if mode.startswith("f64"):
            assert np.isnan(g[[3, 7]]).all(), mode
        else:
            assert np.isfinite(g[[3, 7]]).all(), mode
