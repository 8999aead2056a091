"""GPU parity tests of the batched multi-instance engine (batch.cu,
batch_kernel.cuh, batch_queue.cuh, batch_pairs.cuh) against the oracle,
instance by instance: every instance's sum of increments and gradient within
1e-5 relative of the FP64 oracle on its FP32-rounded delta (the FP32 bar of the
single-instance engine), for uneven N, mixed P, the three schedules and every
built tile shape, missing pairs, single-location updates and precision
changes; plus determinism and the autotuner."""
import numpy as np
import pytest

import oracle
from massivemds_gb300 import Engine, flags as F
from massivemds_gb300 import data as gen
from massivemds_gb300.batch import Batch

pytestmark = pytest.mark.gpu
TOL = 1e-5


def _rel(a, b):
    return abs(a - b) / max(abs(b), 1e-300)


def _grad_rel(g, ref):
    g = np.asarray(g).reshape(ref.shape)
    return np.abs(g - ref).max() / max(np.abs(ref).max(), 1e-300)


def _problems(spec, seed):
    rng = np.random.default_rng(seed)
    out = []
    for n, p in spec:
        delta = gen.euclidean_delta(n, dim=10, seed=int(rng.integers(1 << 30))).astype(np.float32)
        x = rng.standard_normal((n, p))
        tau = float(rng.gamma(2.0, 1.0)) + 0.05
        out.append((delta, x, tau))
    return out


def _fill(b, problems):
    for delta, x, tau in problems:
        k = b.add_instance(x.shape[1], x.shape[0])
        b.setPairwiseData(k, delta)
        b.updateLocations(k, -1, x)
        b.setParameters(k, [tau])


def _check(b, problems, trunc=True):
    for k, (delta, x, tau) in enumerate(problems):
        s_ref = oracle.sum_of_increments(delta, x, tau, trunc)
        g_ref = oracle.gradient(delta, x, tau, trunc)
        assert _rel(b.getSumOfIncrements(k), s_ref) < TOL, k
        assert _grad_rel(b.getLogLikelihoodGradient(k), g_ref) < TOL, k


SPEC = [(257, 2), (300, 3), (513, 6), (130, 2), (1024, 3), (777, 6), (64, 2), (999, 2)]


def test_mixed_instances_match_oracle():
    problems = _problems(SPEC, 1)
    with Batch() as b:
        _fill(b, problems)
        _check(b, problems)
        ll = b.getLogLikelihood(0)
        delta, x, tau = problems[0]
        assert _rel(ll, oracle.log_likelihood(oracle.sum_of_increments(delta, x, tau), x.shape[0], tau)) < TOL


def test_uneven_batch_at_full_scale_matches_oracle():
    """Sixteen instances from the 64-instance workload's generator
    (massivemds_gb300.batch_bench.make_instances: N ~ U{500..8000}, P cycling 2,
    3, 6, tau ~ Gamma(2, 1), delta = distances of N points iid N(0, I_10),
    FP32), the largest of them at N = 8000 so the top of the range is covered;
    every instance against the FP64 oracle, with the tuned shapes and with the
    default ones."""
    from massivemds_gb300.batch_bench import make_instances

    spec = make_instances(16, 3)
    top = int(np.argmax([n for n, _, _, _ in spec]))
    spec[top] = (8000,) + spec[top][1:]
    problems = []
    for n, p, tau, s in spec:
        delta = gen.pairwise_distances(gen.latent_points(n, 10, s), dtype=np.float32)
        x = np.random.default_rng(s + 1).standard_normal((n, p))
        problems.append((delta, x, tau))
    refs = [oracle.evaluate(delta, x, tau, True) for delta, x, tau in problems]
    for tuned in (False, True):
        with Batch() as b:
            _fill(b, problems)
            if tuned:
                b.tune(repetitions=2)
            for k, (s_ref, g_ref) in enumerate(refs):
                assert _rel(b.getSumOfIncrements(k), s_ref) < TOL, (tuned, k, spec[k][:2])
                assert _grad_rel(b.getLogLikelihoodGradient(k), g_ref) < TOL, (tuned, k, spec[k][:2])


SHAPES = [(2, 1, 2), (2, 2, 1), (2, 4, 2), (3, 1, 1), (3, 2, 2), (3, 4, 1), (6, 1, 2), (6, 2, 1)]


@pytest.mark.parametrize("schedule", [0, 1])
@pytest.mark.parametrize("p,rw,ctas", SHAPES)
def test_every_shape_matches_oracle(schedule, p, rw, ctas):
    problems = _problems([(257, p), (640, p), (129, p), (1000, p)], 10 + rw)
    with Batch() as b:
        _fill(b, problems)
        b.force_shape(p, rw, ctas, schedule)
        assert b.group_shape(p)[:3] == (schedule, rw, ctas)
        _check(b, problems)


@pytest.mark.parametrize("ctas", [1, 2])
@pytest.mark.parametrize("p", [1, 2, 3, 4, 5, 6])
def test_pair_schedule_matches_oracle(p, ctas):
    problems = _problems([(257, p), (640, p), (129, p), (1000, p), (33, p), (2, p)], 20 + p)
    with Batch() as b:
        _fill(b, problems)
        b.force_shape(p, 4, ctas, 2)
        sc, rw, c, _ = b.group_shape(p)
        assert (sc, rw) == (2, 4) and 1 <= c <= ctas  # P = 6 fits one CTA per SM: a forced 2 is clamped
        _check(b, problems)


def test_pair_schedule_mixed_groups_missing_pairs_and_updates():
    """Pair-schedule groups (P = 2, 3) beside a row-schedule group (P = 6) in one
    graph; asymmetric NaN pairs; precision and location updates."""
    problems = _problems([(300, 2), (700, 3), (260, 6), (1100, 2), (450, 3)], 21)
    d = problems[0][0].copy()
    rng = np.random.default_rng(3)
    for _ in range(30):
        i, j = rng.integers(0, 300, 2)
        d[i, j] = np.nan  # (j, i) stays observed
    d[17, :] = np.nan
    problems[0] = (d, problems[0][1], problems[0][2])
    with Batch() as b:
        _fill(b, problems)
        b.force_shape(2, 4, 2, 2)
        b.force_shape(3, 4, 2, 2)
        _check(b, problems)
        delta, x, tau = problems[3]
        x = x.copy()
        x[5] += 0.5
        b.updateLocations(3, 5, x[5])
        b.setParameters(4, [0.37])
        problems[3] = (delta, x, tau)
        problems[4] = (problems[4][0], problems[4][1], 0.37)
        _check(b, problems)
        b.makeDirty()
        b.evaluate()
        s1 = [b.getSumOfIncrements(k) for k in range(len(problems))]
        g1 = [b.getLogLikelihoodGradient(k).copy() for k in range(len(problems))]
        b.makeDirty()
        b.evaluate()
        assert [b.getSumOfIncrements(k) for k in range(len(problems))] == s1
        for k in range(len(problems)):
            assert np.array_equal(b.getLogLikelihoodGradient(k), g1[k])


def test_schedules_agree_and_gradients_concatenate_in_instance_order():
    torch = pytest.importorskip("torch")
    problems = _problems([(300, 6), (700, 2), (451, 3), (1200, 2)], 12)
    grads = {}
    for schedule in (0, 1, 2):
        with Batch() as b:
            _fill(b, problems)
            for p in (2, 3, 6):
                if schedule == 2:
                    b.force_shape(p, 4, 2, 2)
                else:
                    b.force_shape(p, 1, 2, schedule)
            total = sum(x.size for _, x, _ in problems)
            d_sums = torch.zeros(4 * len(problems), dtype=torch.float64, device="cuda")
            d_grads = torch.zeros(total, dtype=torch.float64, device="cuda")
            b.evaluate_device(d_sums.data_ptr(), d_grads.data_ptr())
            torch.cuda.synchronize()
            g = d_grads.cpu().numpy()
            off = 0
            for k, (_, x, _) in enumerate(problems):
                assert np.array_equal(g[off:off + x.size], b.getLogLikelihoodGradient(k))
                off += x.size
            grads[schedule] = g
    # the schedules sum the partials in different orders
    for schedule in (1, 2):
        assert np.abs(grads[0] - grads[schedule]).max() <= 1e-5 * np.abs(grads[0]).max()


def test_without_truncation():
    problems = _problems([(300, 2), (450, 3)], 3)
    with Batch(flags=F.FLOAT) as b:
        _fill(b, problems)
        _check(b, problems, trunc=False)


def test_missing_pairs():
    problems = _problems([(300, 2), (260, 3)], 4)
    d = problems[0][0].copy()
    rng = np.random.default_rng(0)
    i, j = rng.integers(0, 300, 40), rng.integers(0, 300, 40)
    d[i, j] = np.nan
    d[j, i] = np.nan
    problems[0] = (d, problems[0][1], problems[0][2])
    with Batch() as b:
        _fill(b, problems)
        _check(b, problems)


def test_updates_are_lazy_and_local():
    problems = _problems([(300, 2), (200, 6), (512, 3)], 5)
    with Batch() as b:
        _fill(b, problems)
        _check(b, problems)
        # one location of instance 1, the precision of instance 2
        delta, x, tau = problems[1]
        x = x.copy()
        x[17] += 0.25
        b.updateLocations(1, 17, x[17])
        problems[1] = (delta, x, tau)
        delta2, x2, _ = problems[2]
        b.setParameters(2, [3.5])
        problems[2] = (delta2, x2, 3.5)
        _check(b, problems)


def test_deterministic_and_same_as_single_engine():
    problems = _problems([(700, 2), (333, 3)], 6)
    with Batch() as b:
        _fill(b, problems)
        b.evaluate()
        first = [b.getLogLikelihoodGradient(k).copy() for k in range(2)]
        s1 = [b.getSumOfIncrements(k) for k in range(2)]
        b.makeDirty()
        b.evaluate()
        assert [b.getSumOfIncrements(k) for k in range(2)] == s1
        for k in range(2):
            assert np.array_equal(b.getLogLikelihoodGradient(k), first[k])
    for k, (delta, x, tau) in enumerate(problems):
        e = Engine(x.shape[1], x.shape[0], F.FLOAT | F.LEFT_TRUNCATION)
        e.setPairwiseData(delta)
        e.updateLocations(-1, x)
        e.setParameters([tau])
        assert _rel(e.getSumOfIncrements(), s1[k]) < 1e-6
        assert _grad_rel(e.getLogLikelihoodGradient(), first[k].reshape(x.shape)) < 1e-6
        e.close()


def test_tune_picks_a_built_shape_and_keeps_parity(tmp_path, monkeypatch):
    monkeypatch.setenv("MDSX_TUNE_CACHE", str(tmp_path / "tune.txt"))
    problems = _problems([(800, 2), (600, 2), (500, 3), (900, 6)], 7)
    with Batch() as b:
        _fill(b, problems)
        assert b.tune(repetitions=3) >= 3
        for p in (2, 3, 6):
            sc, rw, ctas, grid = b.group_shape(p)
            assert sc in (0, 1, 2) and ctas in (1, 2) and grid >= 1
            assert rw == 4 if sc == 2 else rw in ((1, 2, 4) if p <= 4 else (1, 2))
        _check(b, problems)


def test_location_updates_right_after_an_asynchronous_evaluation():
    """Location updates are staged in pinned host copies and uploaded with the
    next evaluation; an update issued while the previous evaluation (and its
    uploads) may still run must not change that evaluation's inputs, and the
    next evaluation sees the new locations."""
    torch = pytest.importorskip("torch")
    problems = _problems([(900, 2), (700, 3), (500, 6), (1200, 2)], 31)
    with Batch() as b:
        _fill(b, problems)
        total = sum(x.size for _, x, _ in problems)
        d_sums = torch.zeros(4 * len(problems), dtype=torch.float64, device="cuda")
        d_grads = torch.zeros(total, dtype=torch.float64, device="cuda")
        b.evaluate_device(d_sums.data_ptr(), d_grads.data_ptr())  # enqueued, not synchronised
        rng = np.random.default_rng(32)
        new = []
        for k, (delta, x, tau) in enumerate(problems):
            x2 = x + 0.3 * rng.standard_normal(x.shape)
            b.updateLocations(k, -1, x2)
            new.append((delta, x2, tau))
        torch.cuda.synchronize()
        first = d_sums.cpu().numpy().reshape(-1, 4)[:, 2]
        for k, (delta, x, tau) in enumerate(problems):
            assert _rel(first[k], oracle.sum_of_increments(delta, x, tau)) < TOL, k
        _check(b, new)
