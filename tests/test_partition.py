"""CPU tests of the row partition of one problem across ranks
(massivemds_gb300/partition.py): the row ranges cover every row, hence every
ordered pair, exactly once; and the exchange -- a scalar all-reduce of the
ranks' likelihood shares and an all-gather of their gradient rows -- rebuilds
the whole problem's sum of increments, log-likelihood and gradient. The ranks
are gloo processes on the CPU; each rank's engine over its rows is a stand-in
that evaluates those rows with the oracle (the CUDA engine over a row range is
tested against the whole-matrix engine in tests/test_partition_gpu.py)."""
import math
import os
import sys

import numpy as np
import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, REPO)

from massivemds_gb300.partition import RowPartitionedEngine, row_ranges  # noqa: E402


@pytest.mark.parametrize("n", [1, 2, 7, 64, 257, 1000, 20000])
@pytest.mark.parametrize("world", [1, 2, 3, 4, 8])
def test_row_ranges_cover_every_pair_once(n, world):
    if world > n:
        with pytest.raises(ValueError):
            row_ranges(n, world)
        return
    ranges = row_ranges(n, world)
    assert ranges[0][0] == 0 and ranges[-1][1] == n
    assert all(a[1] == b[0] for a, b in zip(ranges, ranges[1:]))
    sizes = [r1 - r0 for r0, r1 in ranges]
    assert min(sizes) >= 1 and max(sizes) - min(sizes) <= 1
    # every ordered pair (i, j) lies in exactly one rank's rows
    assert sum(s * n for s in sizes) == n * n


class OracleRows:
    """A rank's engine over rows [r0, r1), evaluated by the oracle (test stand-in)."""

    def __init__(self, p, n, rows, truncation):
        self.p, self.n, (self.r0, self.r1), self.trunc = p, n, rows, truncation
        self.delta = self.x = self.tau = None

    def setPairwiseData(self, rows_of_delta):
        a = np.asarray(rows_of_delta, dtype=np.float64)
        assert a.shape == (self.r1 - self.r0, self.n)
        self.delta = np.full((self.n, self.n), np.nan)
        self.delta[self.r0:self.r1] = a  # only this rank's rows are ever read

    def updateLocations(self, index, x):
        assert index == -1
        self.x = np.asarray(x, dtype=np.float64).reshape(self.n, self.p)

    def setParameters(self, parameters):
        self.tau = float(np.atleast_1d(parameters)[0])

    def _rows(self):
        import oracle

        return oracle.sweep_rows(self.delta, self.x, self.tau, self.trunc, self.r0, self.r1, threads=1)

    def getSumOfIncrements(self):
        half = math.fsum(self._rows()[0]) / 2.0
        return half if self.trunc else 0.5 * self.tau * half

    def getLogLikelihood(self):
        obs = (self.r1 - self.r0) * (self.n - 1) / 2.0
        return 0.5 * (math.log(self.tau) - math.log(2 * math.pi)) * obs - self.getSumOfIncrements()

    def getLogLikelihoodGradient(self):
        return self._rows()[1].reshape(-1)


def _problem(n, p, seed):
    rng = np.random.default_rng(seed)
    y = rng.standard_normal((n, 10))
    delta = np.sqrt(((y[:, None] - y[None]) ** 2).sum(-1))
    for _ in range(5):
        i, j = rng.choice(n, 2, replace=False)
        delta[i, j] = np.nan
    delta[n // 3, :] = np.nan
    return delta, rng.standard_normal((n, p))


def _rank_main(rank, world, port, n, p, truncation, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        delta, x = _problem(n, p, 5)
        rows = row_ranges(n, world)[rank]
        eng = RowPartitionedEngine(p, n, engine=OracleRows(p, n, rows, truncation))
        assert (eng.rowBegin, eng.rowEnd) == rows
        eng.setPairwiseData(delta)
        eng.updateLocations(-1, x)
        eng.setParameters([1.7])
        out[rank] = (eng.getSumOfIncrements(), eng.getLogLikelihood(), eng.getLogLikelihoodGradient())
    finally:
        dist.destroy_process_group()


def _free_port():
    import socket

    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


@pytest.mark.parametrize("world", [2, 3])
@pytest.mark.parametrize("truncation", [True, False])
def test_ranks_rebuild_the_whole_problem(world, truncation):
    import oracle

    n, p = 257, 3
    with mp.Manager() as manager:
        out = manager.dict()
        mp.spawn(_rank_main, args=(world, _free_port(), n, p, truncation, out), nprocs=world, join=True)
        results = dict(out)
    delta, x = _problem(n, p, 5)
    s_ref = oracle.sum_of_increments(delta, x, 1.7, truncation)
    g_ref = oracle.gradient(delta, x, 1.7, truncation)
    ll_ref = oracle.log_likelihood(s_ref, n, 1.7)
    for rank in range(world):
        s, ll, g = results[rank]
        assert s == pytest.approx(s_ref, rel=1e-13)
        assert ll == pytest.approx(ll_ref, rel=1e-13)
        np.testing.assert_allclose(g, g_ref, rtol=1e-13, atol=1e-13 * np.abs(g_ref).max())
