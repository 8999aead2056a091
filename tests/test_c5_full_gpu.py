"""The N = 50 000, P = 3 workload of the large HMC run on the GPU against the
FP64 oracle at full size. delta is the matrix massivemds_gb300/hmc_large.py
samples on: distances of 50 000 points iid N(0, I_20) plus N(0, 0.05^2) noise
drawn once per unordered pair, mirrored and clipped at 0, stored FP32 (10 GB).
One location state (x ~ N(0, 3^2 I), distances of the same scale as delta) at
tau = 0.5, where d sqrt(tau) spans the normal-tail range, with truncation on:
every engine mode that serves P = 3 -- FP32 on both sweep schedules, FP64 pair
math and double-float pair math over the FP32-stored delta -- with the
tolerances of the N = 20 000 test (FP32 1e-5; FP64 1e-10 for the sum, 1e-9 for
the gradient, max |dg| / max |g|).

Beside it a size-independent property: the likelihood depends on the locations
only through their pairwise distances, so it is invariant under translation and
the gradient summed over all locations vanishes. Every pair term enters its two
rows with opposite signs (src/NewMultiDimensionalScaling.hpp:421-456 computes
row i's term from x_i - x_j), so the sum is zero up to the rounding of the row
sums, and each mode must keep it within its precision.
"""
import numpy as np
import pytest

import oracle
from massivemds_gb300 import Engine, flags as F

pytestmark = pytest.mark.gpu

N, P, TAU, SEED = 50_000, 3, 0.5, 5

# name: (flags, schedule or None for the default, sum tol, gradient tol, |sum_i g_i| / sum_i |g_i| tol)
MODES = {
    "f32": (F.FLOAT, None, 1e-5, 1e-5, 1e-6),
    "f32rows": (F.FLOAT, F.SWEEP_ROWS, 1e-5, 1e-5, 1e-6),
    "f64s32": (F.DELTA_F32, None, 1e-10, 1e-9, 1e-12),
    "dd32": (F.DOUBLE_FLOAT | F.DELTA_F32, None, 1e-10, 1e-9, 1e-12),
}


def net_gradient(g):
    """max over dimensions of |sum_i g_iq| / sum_i |g_iq|."""
    g = np.asarray(g, dtype=np.float64).reshape(N, P)
    return float((np.abs(g.sum(axis=0)) / np.abs(g).sum(axis=0)).max())


@pytest.fixture(scope="module")
def c5():
    torch = pytest.importorskip("torch")
    from massivemds_gb300.hmc_large import make_delta

    d = make_delta(N, 20, 0.05, SEED, torch.device("cuda", 0))
    delta = d.cpu().numpy()
    del d
    torch.cuda.empty_cache()
    x = 3.0 * np.random.default_rng(SEED).standard_normal((N, P))
    s_ref, g_ref = oracle.evaluate(delta, x, TAU, True)
    g_ref = np.asarray(g_ref).reshape(N, P)
    assert net_gradient(g_ref) < 1e-13
    return delta, x, s_ref, g_ref


@pytest.mark.parametrize("mode", list(MODES))
def test_c5_full_size_against_oracle(c5, mode):
    delta, x, s_ref, g_ref = c5
    flags, schedule, tol_s, tol_g, tol_net = MODES[mode]
    e = Engine(P, N, flags | F.LEFT_TRUNCATION)
    try:
        if schedule is not None:
            e.set_sweep_schedule(schedule)
        e.setPairwiseData(delta)
        e.setParameters([TAU])
        e.updateLocations(-1, x)
        s = e.getSumOfIncrements()
        g = np.asarray(e.getLogLikelihoodGradient(), dtype=np.float64).reshape(N, P)
    finally:
        e.close()
    es = abs(s - s_ref) / abs(s_ref)
    eg = float(np.abs(g - g_ref).max() / np.abs(g_ref).max())
    net = net_gradient(g)
    print(f"{mode}: sum {es:.3e}, gradient {eg:.3e}, net gradient {net:.3e}")
    assert es < tol_s and eg < tol_g and net < tol_net, (mode, es, eg, net)
