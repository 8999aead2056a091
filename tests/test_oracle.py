"""CPU tests: pin the oracle against the reference engine, its golden vectors and
the known-answer test from the reference's own fixtures."""
import numpy as np
import pytest

import oracle
from oracle.oracle import FLOAT, LEFT_TRUNCATION, ReferenceEngine

from . import kat


def _rel(a, b):
    return abs(a - b) / max(abs(b), 1e-300)


def _grad_rel(g, ref):
    return np.abs(g - ref).max() / max(np.abs(ref).max(), 1e-300)


def test_oracle_matches_golden_double(golden):
    data, cases = golden
    for name in cases:
        n, p, trunc, tau, use_float = data[f"{name}.meta"]
        if use_float:
            continue
        delta, x = data[f"{name}.delta"], data[f"{name}.x"]
        s = oracle.sum_of_increments(delta, x, tau, bool(trunc))
        g = oracle.gradient(delta, x, tau, bool(trunc))
        assert _rel(s, float(data[f"{name}.sum"])) < 1e-13, name
        assert _grad_rel(g, data[f"{name}.grad"].reshape(g.shape)) < 1e-13, name


def test_oracle_matches_golden_float_engine(golden):
    """The reference FLOAT engine stores delta and x as float and accumulates in
    float; the FP64 oracle on the same float-rounded inputs agrees to float
    accumulation error."""
    data, cases = golden
    for name in cases:
        n, p, trunc, tau, use_float = data[f"{name}.meta"]
        if not use_float:
            continue
        delta = data[f"{name}.delta"].astype(np.float32)
        x = data[f"{name}.x"].astype(np.float32).astype(np.float64)
        s = oracle.sum_of_increments(delta, x, tau, bool(trunc))
        g = oracle.gradient(delta, x, tau, bool(trunc))
        assert _rel(s, float(data[f"{name}.sum"])) < 1e-5, name
        assert _grad_rel(g, data[f"{name}.grad"].reshape(g.shape)) < 1e-4, name


def test_oracle_reproduces_reference_sequence(golden):
    """The benchmark-style store/update/restore sequence: the sum is taken at the
    proposed locations, the gradient after restore/accept."""
    data, _ = golden
    delta, tau = data["seq.delta"], float(data["seq.tau"])
    x = data["seq.x0"]
    assert _rel(oracle.sum_of_increments(delta, x, tau), data["seq.sums"][0]) < 1e-13
    for k, (xn, restore) in enumerate(zip(data["seq.xs"], data["seq.restores"])):
        assert _rel(oracle.sum_of_increments(delta, xn, tau), data["seq.sums"][k + 1]) < 1e-13
        if not restore:
            x = xn
        g = oracle.gradient(delta, x, tau)
        assert _grad_rel(g, data["seq.grads"][k + 1]) < 1e-13


needs_ref = pytest.mark.skipif(not oracle.reference_available(), reason="reference sources not present")


@needs_ref
@pytest.mark.parametrize("n,p,trunc,tau,nans", [
    (2, 1, True, 1.0, 0), (3, 2, True, 0.3, 0), (31, 4, False, 2.5, 1), (257, 2, True, 2.0, 4),
    (300, 5, True, 1.1, 0), (90, 7, False, 0.9, 2), (111, 8, True, 3.0, 0), (64, 9, True, 1.0, 1),
])
def test_oracle_vs_reference_engine(n, p, trunc, tau, nans):
    rng = np.random.default_rng(n * 100 + p)
    y = rng.standard_normal((n, 6))
    delta = np.sqrt(((y[:, None] - y[None]) ** 2).sum(-1))
    for _ in range(nans):
        i, j = rng.choice(n, 2, replace=False)
        delta[i, j] = np.nan  # asymmetric NaN on purpose: row i only
    x = rng.standard_normal((n, p))
    eng = ReferenceEngine(p, n, LEFT_TRUNCATION if trunc else 0)
    eng.setPairwiseData(delta)
    eng.updateLocations(-1, x)
    eng.setParameters(tau)
    eng.makeDirty()
    s_ref, g_ref = eng.getSumOfIncrements(), eng.getLogLikelihoodGradient()
    assert _rel(oracle.sum_of_increments(delta, x, tau, trunc), s_ref) < 1e-13
    assert _grad_rel(oracle.gradient(delta, x, tau, trunc), g_ref) < 1e-13


@needs_ref
def test_oracle_vs_reference_float_engine():
    n, p, tau = 500, 2, 2.0
    rng = np.random.default_rng(5)
    y = rng.standard_normal((n, 10))
    delta = np.sqrt(((y[:, None] - y[None]) ** 2).sum(-1))
    x = rng.standard_normal((n, p))
    eng = ReferenceEngine(p, n, LEFT_TRUNCATION | FLOAT)
    eng.setPairwiseData(delta)
    eng.updateLocations(-1, x)
    eng.setParameters(tau)
    eng.makeDirty()
    s_ref = eng.getSumOfIncrements()
    s = oracle.sum_of_increments(delta.astype(np.float32), x.astype(np.float32).astype(np.float64), tau)
    assert _rel(s, s_ref) < 1e-5


def test_oracle_thread_count_does_not_change_result():
    rng = np.random.default_rng(3)
    n = 301
    delta = np.abs(rng.standard_normal((n, n))) * 3
    x = rng.standard_normal((n, 3))
    a = oracle.sum_of_increments(delta, x, 1.3, True, threads=1)
    b = oracle.sum_of_increments(delta, x, 1.3, True, threads=7)
    assert a == b
    ga = oracle.gradient(delta, x, 1.3, True, threads=1)
    gb = oracle.gradient(delta, x, 1.3, True, threads=5)
    assert np.array_equal(ga, gb)


def test_port_matches_oracle_on_rows():
    """The timed CPU-baseline port computes the same sums as the oracle."""
    rng = np.random.default_rng(4)
    n = 200
    y = rng.standard_normal((n, 10))
    delta = np.sqrt(((y[:, None] - y[None]) ** 2).sum(-1))
    x = rng.standard_normal((n, 2))
    s_port, g_port = oracle.port_eval_rows(delta, x, 2.0, True, 10, 60, threads=3)
    rows, g = oracle.sweep_rows(delta, x, 2.0, True, 10, 60)
    assert _rel(s_port, rows.sum()) < 1e-12
    assert _grad_rel(g_port, g) < 1e-12


@pytest.mark.skipif(not kat.available(), reason="reference fixtures not present")
def test_kat_h3n2_untruncated_loglik_matches_beast():
    delta, x, tau, logged = kat.load_state()
    s = oracle.sum_of_increments(delta, x, tau, truncation=False)
    ll = oracle.log_likelihood(s, delta.shape[0], tau)
    assert _rel(ll, logged) < 1e-12


@pytest.mark.skipif(not (kat.available() and oracle.reference_available()), reason="reference not present")
def test_kat_h3n2_reference_engine_agrees():
    delta, x, tau, logged = kat.load_state()
    eng = ReferenceEngine(2, delta.shape[0], 0)
    eng.setPairwiseData(delta)
    eng.updateLocations(-1, x)
    eng.setParameters(tau)
    eng.makeDirty()
    ll = oracle.log_likelihood(eng.getSumOfIncrements(), delta.shape[0], tau)
    assert _rel(ll, logged) < 1e-12


def test_planted_error_is_detected():
    """A mistake planted in the oracle's inputs (one flipped residual sign in
    the gradient) must move the result far outside the parity tolerances."""
    rng = np.random.default_rng(8)
    n = 64
    y = rng.standard_normal((n, 10))
    delta = np.sqrt(((y[:, None] - y[None]) ** 2).sum(-1))
    x = rng.standard_normal((n, 2))
    g = oracle.gradient(delta, x, 1.0)
    wrong = delta.copy()
    wrong[3, 7] += 0.5  # a perturbed observation in row 3
    g2 = oracle.gradient(wrong, x, 1.0)
    assert _grad_rel(g2, g) > 1e-6


def _symmetric_delta(rng, n, nan_pairs=0):
    y = rng.standard_normal((n, 10))
    d = np.sqrt(((y[:, None] - y[None]) ** 2).sum(-1))
    e = np.triu(rng.standard_normal((n, n)) * 0.05, 1)
    d = np.clip(d + e + e.T, 0.0, None)
    for _ in range(nan_pairs):
        i, j = rng.choice(n, 2, replace=False)
        d[i, j] = d[j, i] = np.nan
    return d


@pytest.mark.parametrize("trunc", [True, False])
def test_oracle_distance_invariances(trunc):
    """The likelihood depends on the locations only through their pairwise
    distances: a translation or a rotation of every location leaves the sum and
    the gradient (rotated with them) unchanged, relabelling the locations
    permutes the gradient, and with a symmetric delta the gradient summed over
    all locations vanishes (each pair term enters its two rows with opposite
    signs, src/NewMultiDimensionalScaling.hpp:421-456)."""
    rng = np.random.default_rng(11)
    n, p, tau = 180, 3, 0.7
    delta = _symmetric_delta(rng, n, nan_pairs=5)
    x = 2.0 * rng.standard_normal((n, p))
    s, g = oracle.evaluate(delta, x, tau, trunc)
    g = np.asarray(g).reshape(n, p)

    net = np.abs(g.sum(axis=0)) / np.abs(g).sum(axis=0)
    assert net.max() < 1e-13, net

    s_t, g_t = oracle.evaluate(delta, x + np.array([0.75, -1.5, 2.25]), tau, trunc)
    assert _rel(s_t, s) < 1e-12
    assert _grad_rel(np.asarray(g_t).reshape(n, p), g) < 1e-10

    q, _ = np.linalg.qr(rng.standard_normal((p, p)))
    s_r, g_r = oracle.evaluate(delta, x @ q, tau, trunc)
    assert _rel(s_r, s) < 1e-12
    assert _grad_rel(np.asarray(g_r).reshape(n, p), g @ q) < 1e-10

    perm = rng.permutation(n)
    s_p, g_p = oracle.evaluate(delta[np.ix_(perm, perm)], x[perm], tau, trunc)
    assert _rel(s_p, s) < 1e-12
    assert _grad_rel(np.asarray(g_p).reshape(n, p), g[perm]) < 1e-12
