"""The full-size sweep workload on the GPU, against the reference engine and the
oracle: N = 20 000, P = 2, tau = 2, truncation on, delta = distances of 20 000
points iid N(0, I_10) plus N(0, 0.05^2) noise drawn once per unordered pair,
mirrored and clipped at 0, stored FP32 (1.6 GB) -- the matrix bench.py times.

* Reference engine: tests/golden/golden_n20000.npz holds, for three location
  states, getSumOfIncrements() and getLogLikelihoodGradient() of the
  reference's own double engine and FLOAT engine on that delta
  (tests/golden/make_golden_n20000.py; the reference's
  src/NewMultiDimensionalScaling.hpp:193-334). Every precision mode and both
  sweep schedules are compared with the double engine: FP64 pair arithmetic
  over FP32-stored delta and over FP64-stored delta within 1e-10 (sum) and
  1e-9 (gradient, max |dg| / max |g|), and so are the double-float modes
  ("dd32" over FP32-stored delta, "dd" over FP64-stored delta); the FP32 mode
  within 1e-5; the FP32
  mode must also land closer to the double engine than the reference's own
  FLOAT engine does.
* Oracle: twenty more states at fresh locations, each evaluated by the FP64
  oracle (threaded, compensated) and by the FP32, FP64-over-FP32,
  FP64-stored and double-float-over-FP32 engines, with the same tolerances.

delta is regenerated from its seed and checked against the fingerprint stored
with the golden vectors before anything is compared.
"""
import os
import sys

import numpy as np
import pytest

import oracle
from massivemds_gb300 import Engine, flags as F

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
import make_golden_n20000 as c2gen  # noqa: E402

TOL_F64_SUM, TOL_F64_GRAD = 1e-10, 1e-9
TOL_F32 = 1e-5
FRESH_STATES = 20

MODES = {  # name: (flags, delta stored as FP64?, schedule or None for the default)
    "f32": (F.FLOAT, False, None),
    "f32rows": (F.FLOAT, False, F.SWEEP_ROWS),
    "f64s32": (F.DELTA_F32, False, None),
    "f64s32rows": (F.DELTA_F32, False, F.SWEEP_ROWS),
    "f64": (0, True, None),
    "f64rows": (0, True, F.SWEEP_ROWS),
    "dd32": (F.DOUBLE_FLOAT | F.DELTA_F32, False, None),
    "dd": (F.DOUBLE_FLOAT, True, None),
}


def rel(a, b):
    return abs(a - b) / max(abs(b), 1e-300)


def grad_rel(g, ref):
    g = np.asarray(g).reshape(ref.shape)
    return np.abs(g - ref).max() / max(np.abs(ref).max(), 1e-300)


def tolerances(mode):
    return (TOL_F32, TOL_F32) if mode.startswith("f32") else (TOL_F64_SUM, TOL_F64_GRAD)


@pytest.fixture(scope="module")
def c2():
    z = np.load(os.path.join(HERE, "golden", "golden_n20000.npz"))
    golden = {k: z[k] for k in z.files}
    delta = c2gen.workload_delta()
    fp = c2gen.fingerprint(delta)
    assert np.allclose(fp, golden["delta_fingerprint"], rtol=1e-12, atol=0), \
        "the regenerated delta differs from the one the golden vectors were made on"
    return delta, golden


def make_engine(mode, delta):
    flags, f64_delta, schedule = MODES[mode]
    e = Engine(c2gen.P, c2gen.N, flags | F.LEFT_TRUNCATION)
    if schedule is not None:
        e.set_sweep_schedule(schedule)
    e.setPairwiseData(delta.astype(np.float64) if f64_delta else delta)
    e.setParameters([c2gen.TAU])
    return e


@pytest.mark.parametrize("mode", list(MODES))
def test_full_size_against_reference_engine(c2, mode):
    delta, golden = c2
    tol_s, tol_g = tolerances(mode)
    e = make_engine(mode, delta)
    try:
        for k in range(golden["x"].shape[0]):
            e.updateLocations(-1, golden["x"][k].astype(np.float64))
            s, g = e.getSumOfIncrements(), e.getLogLikelihoodGradient()
            s_ref, g_ref = float(golden["sum_f64"][k]), golden["grad_f64"][k]
            es, eg = rel(s, s_ref), grad_rel(g, g_ref)
            assert es < tol_s, (k, es)
            assert eg < tol_g, (k, eg)
            if mode.startswith("f32"):
                # the reference's own FLOAT engine on the same delta and state
                fs = rel(float(golden["sum_float"][k]), s_ref)
                fg = grad_rel(golden["grad_float"][k].astype(np.float64), g_ref)
                assert es < fs and eg < fg, (k, es, fs, eg, fg)
    finally:
        e.close()


def test_full_size_fresh_states_against_oracle(c2):
    delta, _ = c2
    engines = {m: make_engine(m, delta) for m in ("f32", "f64s32", "f64", "dd32")}
    rng = np.random.default_rng(20001)
    try:
        for k in range(FRESH_STATES):
            x = rng.standard_normal((c2gen.N, c2gen.P))
            s_ref, g_ref = oracle.evaluate(delta, x, c2gen.TAU, True)
            for mode, e in engines.items():
                tol_s, tol_g = tolerances(mode)
                e.updateLocations(-1, x)
                s, g = e.getSumOfIncrements(), e.getLogLikelihoodGradient()
                assert rel(s, s_ref) < tol_s, (mode, k)
                assert grad_rel(g, g_ref) < tol_g, (mode, k)
    finally:
        for e in engines.values():
            e.close()
