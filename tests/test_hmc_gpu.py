"""GPU tests of the on-device HMC driver (mdsx_hmc_run) against the numpy
restatement of one trajectory (oracle/hmc_oracle.py) and against the oracle's
log-likelihood. FP64 mode: Hamiltonian difference within 1e-7 absolute and
proposal within 1e-9 relative of the restatement."""
import numpy as np
import pytest

import oracle
from massivemds_gb300 import Engine, flags as F
from massivemds_gb300.hmc import hmc
from oracle import hmc_oracle

pytestmark = pytest.mark.gpu


def _problem(n, p, seed, clusters=0):
    rng = np.random.default_rng(seed)
    y = rng.standard_normal((n, 6)) + (3.0 * rng.standard_normal((clusters, 6))[np.arange(n) % clusters] if clusters else 0)
    delta = np.sqrt(((y[:, None] - y[None]) ** 2).sum(-1))
    x0 = 0.5 * rng.standard_normal((n, p))
    return delta, x0


def _engine(delta, p, tau, flags):
    e = Engine(p, delta.shape[0], flags | F.LEFT_TRUNCATION)
    e.setPairwiseData(delta)
    e.setParameters([tau])
    return e


@pytest.mark.parametrize("use_graph", [True, False])
def test_one_trajectory_matches_restatement(use_graph):
    n, p, tau, eps, steps, seed = 80, 2, 1.3, 0.004, 12, 21
    delta, x0 = _problem(n, p, 5)
    e = _engine(delta, p, tau, 0)
    res = hmc(e, x0, iterations=1, leapfrog_steps=steps, step_size=eps, seed=seed, use_graph=use_graph)
    e.close()
    x_ref, dh_ref = hmc_oracle.trajectory(delta, x0, tau, eps, steps, seed, iteration=0)
    assert abs(res.column("delta_h")[0] - dh_ref) < 1e-7
    expected = x_ref if res.column("accepted")[0] == 1.0 else x0
    assert np.abs(res.final_locations - expected).max() <= 1e-9 * max(1.0, np.abs(expected).max())
    s = oracle.sum_of_increments(delta, res.final_locations, tau)
    assert abs(res.column("log_likelihood")[0] - oracle.log_likelihood(s, n, tau)) < 1e-8 * abs(s)


@pytest.mark.parametrize("p", [1, 3, 4, 6])
def test_second_iteration_uses_its_own_momentum(p):
    # the truncated FP64 engine runs the unordered-pair sweep for P <= 6, whose
    # finish kernel applies the kick/drift: P = 6 is its widest instance
    n, tau, eps, steps, seed = 50, 0.9, 0.003, 8, 5
    delta, x0 = _problem(n, p, 6)
    e = _engine(delta, p, tau, 0)
    res = hmc(e, x0, iterations=2, leapfrog_steps=steps, step_size=eps, seed=seed)
    e.close()
    x1 = x0
    for it in range(2):
        prop, dh = hmc_oracle.trajectory(delta, x1, tau, eps, steps, seed, iteration=it)
        assert abs(res.column("delta_h")[it] - dh) < 1e-7
        if res.column("accepted")[it] == 1.0:
            x1 = prop
    assert np.abs(res.final_locations - x1).max() <= 1e-9 * max(1.0, np.abs(x1).max())


@pytest.mark.parametrize("p", [2, 6])
def test_fp32_chain_consistent_with_oracle(p):
    # P = 6: the column-pack pair math with the fused kick/drift
    n, tau = 400, 1.0
    delta, x0 = _problem(n, p, 7, clusters=5)
    e = _engine(delta.astype(np.float32), p, tau, F.FLOAT)
    res = hmc(e, x0, iterations=30, leapfrog_steps=10, step_size=0.002, seed=3)
    e.close()
    s = oracle.sum_of_increments(delta.astype(np.float32), res.final_locations, tau)
    ll = oracle.log_likelihood(s, n, tau)
    assert abs(res.column("log_likelihood")[-1] - ll) < 1e-5 * abs(ll)
    assert res.gradient_evaluations == 1 + 30 * 10


def test_same_seed_same_chain():
    n, p = 200, 2
    delta, x0 = _problem(n, p, 8)
    runs = []
    for _ in range(2):
        e = _engine(delta.astype(np.float32), p, 1.0, F.FLOAT)
        runs.append(hmc(e, x0, iterations=20, leapfrog_steps=5, step_size=0.003, seed=11,
                        traced_pairs=[[0, 1], [2, 3]], traced_locations=[4]))
        e.close()
    assert np.array_equal(runs[0].trace, runs[1].trace)
    assert np.array_equal(runs[0].final_locations, runs[1].final_locations)


def test_step_size_adaptation_reaches_target():
    n, p = 500, 2
    delta, x0 = _problem(n, p, 9, clusters=5)
    e = _engine(delta.astype(np.float32), p, 1.0, F.FLOAT)
    res = hmc(e, x0, iterations=400, burn_in=250, leapfrog_steps=20, step_size=0.01, adapt_step_size=True,
              target_accept=0.8, seed=1, traced_pairs=[[0, 1]], traced_locations=[0, 7])
    e.close()
    assert 0.55 < res.accept_rate <= 1.0
    assert np.all(res.column("step_size")[250:] == res.step_size)
    assert res.pair_distances.shape == (400, 1) and res.location_norms.shape == (400, 2)


def test_precision_and_trait_precision_moves():
    n, p = 300, 3
    delta, x0 = _problem(n, p, 10)
    e = _engine(delta.astype(np.float32), p, 1.0, F.FLOAT)
    res = hmc(e, x0, iterations=60, leapfrog_steps=10, step_size=0.002, learn_precision=True,
              precision_half_width=0.05, learn_trait_precision=True, seed=2)
    tau_final = res.precision
    assert np.all(res.column("precision") > 0)
    assert len(np.unique(res.column("precision"))) > 1
    assert res.column("precision")[-1] == tau_final
    # the engine is left at the chain's final state
    s = e.getSumOfIncrements()
    e.close()
    assert abs(s - oracle.sum_of_increments(delta.astype(np.float32), res.final_locations, tau_final)) < 1e-5 * abs(s)


@pytest.mark.parametrize("flags", [0, F.FLOAT])
def test_checkpoint_and_resume_continue_the_same_chain(flags, tmp_path):
    """A chain run in two calls -- the first writing a checkpoint, the second
    resuming from it (through a file) -- gives the trace of the chain run in
    one call, bit for bit: momentum keyed by the chain's iteration index, the
    host generator, tau, the trait precision and the step-size adaptation
    (its burn-in spans the split) all carry over."""
    from massivemds_gb300.hmc import load_checkpoint, save_checkpoint

    n, p, tau = 120, 2, 1.1
    delta, x0 = _problem(n, p, 8, clusters=3)
    kw = dict(leapfrog_steps=6, step_size=0.004, adapt_step_size=True, target_accept=0.8, burn_in=30,
              learn_precision=True, precision_half_width=0.05, learn_trait_precision=True, seed=99,
              traced_pairs=[[0, 1], [5, 77]], traced_locations=[3, 60])
    e = _engine(delta, p, tau, flags)
    whole = hmc(e, x0, iterations=50, **kw)
    e.setParameters([tau])
    first = hmc(e, x0, iterations=20, checkpoint=True, **kw)
    assert first.checkpoint is not None and len(first.checkpoint) > 16 * n * p
    path = str(tmp_path / "chain.ckpt")
    save_checkpoint(path, first.checkpoint)
    e.setParameters([3.0])  # resuming restores the chain's own precision
    rest = hmc(e, np.zeros_like(x0), iterations=30, resume=load_checkpoint(path), **kw)  # locations come from the checkpoint
    e.close()
    assert np.array_equal(np.vstack([first.trace, rest.trace]), whole.trace)
    assert np.array_equal(rest.final_locations, whole.final_locations)
    assert rest.precision == whole.precision and rest.step_size == whole.step_size


def test_resume_rejects_a_foreign_checkpoint():
    from massivemds_gb300 import MdsxError

    n, p = 60, 2
    delta, x0 = _problem(n, p, 9)
    e = _engine(delta, p, 1.0, 0)
    first = hmc(e, x0, iterations=3, step_size=0.003, seed=1, checkpoint=True)
    with pytest.raises(MdsxError):
        hmc(e, x0, iterations=3, step_size=0.003, seed=2, resume=first.checkpoint)  # another seed
    with pytest.raises(MdsxError):
        hmc(e, x0, iterations=3, step_size=0.003, seed=1, resume=first.checkpoint[:-5])  # truncated
    e.close()
    e3 = _engine(_problem(n, 3, 9)[0], 3, 1.0, 0)
    with pytest.raises(MdsxError):
        hmc(e3, np.zeros((n, 3)), iterations=3, step_size=0.003, seed=1, resume=first.checkpoint)  # P differs
    e3.close()


def test_precision_proposal_adapts_during_burn_in():
    """With adapt_precision_proposal the half-width of the tau proposal moves
    toward 44 % acceptance during burn-in and is then fixed (read back from the
    checkpoint header); without it the half-width stays the reference's."""
    import struct

    n, p = 150, 2
    delta, x0 = _problem(n, p, 12, clusters=3)
    out = {}
    for adapt in (False, True):
        e = _engine(delta, p, 0.2, 0)  # tau far from its posterior
        res = hmc(e, x0, iterations=400, burn_in=300, leapfrog_steps=5, step_size=0.003, adapt_step_size=True,
                  learn_precision=True, precision_half_width=0.01, seed=4, checkpoint=True,
                  adapt_precision_proposal=adapt)
        e.close()
        hw = struct.unpack_from("<d", res.checkpoint, 96)[0]
        tau = res.column("precision")
        moves = float(np.mean(tau[301:] != tau[300:-1]))
        out[adapt] = (hw, moves)
    assert out[False][0] == 0.01
    assert out[True][0] != 0.01
    assert 0.15 < out[True][1] < 0.8, out  # the adapted proposal accepts a fair share of moves
