"""GPU tests of engines over a row range of delta (mdsx_create_rows), the
building block of splitting one problem across GPUs
(massivemds_gb300/partition.py).

The partitions of a problem run one after the other on this one GPU, each an
engine over its rows only; their sums of increments and log-likelihoods add up
to, and their gradient rows concatenate to, the whole-matrix engine's results
(within 1e-10 in FP64 modes: only the order of the final additions differs)
and the FP64 oracle's (the usual 1e-10 / 1e-9 FP64 and 1e-5 FP32 bars).
Ranges start and end off row-block boundaries, hold missing pairs and a missing
row, and the state machine (store / update / restore) runs per range.
"""
import numpy as np
import pytest

import oracle
from massivemds_gb300 import Engine, MdsxError, flags as F
from massivemds_gb300.partition import RowPartitionedEngine, row_ranges

pytestmark = pytest.mark.gpu

MODES = {"f64": 0, "f64s32": F.DELTA_F32, "f32": F.FLOAT}


def rel(a, b):
    return abs(a - b) / max(abs(b), 1e-300)


def grad_rel(g, ref):
    g = np.asarray(g).reshape(ref.shape)
    return np.abs(g - ref).max() / max(np.abs(ref).max(), 1e-300)


def _problem(n, p, seed):
    rng = np.random.default_rng(seed)
    y = rng.standard_normal((n, 10))
    delta = np.sqrt(((y[:, None] - y[None]) ** 2).sum(-1))
    for _ in range(7):
        i, j = rng.choice(n, 2, replace=False)
        delta[i, j] = np.nan  # one direction only
    delta[n // 2, :] = np.nan
    return delta, rng.standard_normal((n, p))


def _whole(mode, trunc, delta, x, tau):
    e = Engine(x.shape[1], x.shape[0], MODES[mode] | (F.LEFT_TRUNCATION if trunc else 0))
    e.set_sweep_schedule(F.SWEEP_ROWS)
    e.setPairwiseData(delta.astype(np.float32) if mode == "f32" else delta)
    e.updateLocations(-1, x)
    e.setParameters([tau])
    return e


def _parts(mode, trunc, delta, x, tau, world):
    n, p = x.shape
    parts = []
    for r0, r1 in row_ranges(n, world):
        e = Engine(p, n, MODES[mode] | (F.LEFT_TRUNCATION if trunc else 0), rows=(r0, r1))
        e.setPairwiseData(delta[r0:r1].astype(np.float32) if mode == "f32" else delta[r0:r1])
        e.updateLocations(-1, x)
        e.setParameters([tau])
        parts.append(e)
    return parts


def _combine(parts):
    s = sum(e.getSumOfIncrements() for e in parts)
    ll = sum(e.getLogLikelihood() for e in parts)
    g = np.concatenate([e.getLogLikelihoodGradient().reshape(-1, parts[0].embeddingDimension) for e in parts])
    return s, ll, g


@pytest.mark.parametrize("mode", list(MODES))
@pytest.mark.parametrize("world", [2, 3, 5])
@pytest.mark.parametrize("n,p,trunc", [(1000, 2, True), (777, 3, False), (4099, 6, True)])
def test_row_ranges_rebuild_the_whole_matrix(mode, world, n, p, trunc):
    tau = 1.3
    delta, x = _problem(n, p, 100 + n + world)
    whole = _whole(mode, trunc, delta, x, tau)
    s_w, ll_w, g_w = whole.getSumOfIncrements(), whole.getLogLikelihood(), whole.getLogLikelihoodGradient()
    whole.close()
    parts = _parts(mode, trunc, delta, x, tau, world)
    s, ll, g = _combine(parts)
    for e in parts:
        e.close()
    d_or = delta.astype(np.float32) if mode != "f64" else delta
    s_ref = oracle.sum_of_increments(d_or, x, tau, trunc)
    g_ref = oracle.gradient(d_or, x, tau, trunc)
    if mode == "f32":
        assert rel(s, s_ref) < 1e-5 and grad_rel(g, g_ref) < 1e-5
        assert rel(s, s_w) < 1e-6 and grad_rel(g, g_w.reshape(n, p)) < 1e-6
    else:
        assert rel(s, s_w) < 1e-10 and rel(ll, ll_w) < 1e-10
        assert grad_rel(g, g_w.reshape(n, p)) < 1e-12  # each gradient row is computed alike
        assert rel(s, s_ref) < 1e-10 and grad_rel(g, g_ref) < 1e-9


def test_row_range_state_machine_and_partitioned_engine_on_one_rank():
    n, p, tau = 600, 2, 0.8
    delta, x = _problem(n, p, 9)
    parts = _parts("f64", True, delta, x, tau, 2)
    s0, _, g0 = _combine(parts)
    for e in parts:
        e.storeState()
    x2 = x + 0.1
    for e in parts:
        e.updateLocations(-1, x2)
    s1, _, g1 = _combine(parts)
    assert rel(s1, oracle.sum_of_increments(delta, x2, tau)) < 1e-10
    for e in parts:
        e.restoreState()
    s2, _, g2 = _combine(parts)
    assert s2 == s0 and np.array_equal(g2, g0)
    for e in parts:
        e.close()
    # one rank, no process group: RowPartitionedEngine is the whole matrix
    with_all = RowPartitionedEngine(p, n, F.LEFT_TRUNCATION)
    with_all.setPairwiseData(delta)
    with_all.updateLocations(-1, x)
    with_all.setParameters([tau])
    assert rel(with_all.getSumOfIncrements(), s0) < 1e-10
    assert grad_rel(with_all.getLogLikelihoodGradient(), g0) < 1e-12
    with_all.close()


def test_row_range_errors():
    n, p = 300, 2
    with pytest.raises(MdsxError):
        Engine(p, n, 0, rows=(10, 10))
    with pytest.raises(MdsxError):
        Engine(p, n, 0, rows=(0, n + 1))
    e = Engine(p, n, F.LEFT_TRUNCATION, rows=(100, 200))
    with pytest.raises(MdsxError):
        e.setPairwiseData(np.zeros((n, n)))  # a row range takes its rows only
    with pytest.raises(MdsxError):
        e.set_sweep_schedule(F.SWEEP_PAIRS)  # needs the whole matrix
    e.setPairwiseData(np.ones((100, n)))
    e.updateLocations(-1, np.random.default_rng(0).standard_normal((n, p)))
    e.setParameters([1.0])
    assert e.getLogLikelihoodGradient().size == 100 * p
    with pytest.raises(ValueError):
        e.getLogLikelihoodGradient(np.empty(n * p))
    e.close()
