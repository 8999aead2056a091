"""One MDS problem's sweep split across ranks (one GPU each) by rows of delta.

The reference's own parallel split is over the rows i of delta: its TBB engine
runs both passes as parallel_reduce / parallel_for over i
(src/NewMultiDimensionalScaling.hpp:708-744). Row i of the gradient reads only
row i of delta (:421-461) and the sum of increments is a sum of row sums
(:524-561), so the rows can be split across devices with no exchange inside
the sweep:

* rank r of G holds rows [r0, r1) of delta (``row_ranges``: equal shares of
  rows, i.e. of the N^2 pairs) in an engine over those rows only
  (``Engine(..., rows=(r0, r1))``, mdsx_create_rows): (r1 - r0) * N * s_delta
  bytes of HBM per rank;
* every rank holds all N locations (the caller replicates its state, as a
  sampler whose ranks draw the same proposal does);
* per evaluation, one scalar all-reduce (the sum of increments, or the
  log-likelihood) and one all-gather of the gradient rows (N * P doubles).

Collectives go through ``torch.distributed``: NCCL with device tensors on GPUs,
gloo with host tensors on the CPU. There is no peer memory access, no TMA
multicast and nothing inside the kernels that waits on another rank.
"""
from __future__ import annotations

import numpy as np

from .engine import Engine


def row_ranges(n: int, world: int) -> list[tuple[int, int]]:
    """[r0, r1) per rank: contiguous, covering [0, n) once, sizes differing by at most one."""
    if world < 1 or n < world:
        raise ValueError("need 1 <= world <= n")
    bounds = [(r * n) // world for r in range(world + 1)]
    return [(bounds[r], bounds[r + 1]) for r in range(world)]


def _dist():
    import torch.distributed as dist

    return dist if dist.is_available() and dist.is_initialized() else None


class RowPartitionedEngine:
    """``mds::AbstractMultiDimensionalScaling`` for one rank's share of a problem.

    Same method names and argument meaning as :class:`Engine`; the results of
    getSumOfIncrements, getLogLikelihood and getLogLikelihoodGradient are the
    whole problem's on every rank (after the collectives). ``engine`` replaces
    the rank's CUDA engine over its rows by any object with the engine's
    methods (tests use it to run the exchange on CPU ranks).
    """

    def __init__(self, embeddingDimension: int, locationCount: int, flags: int = 0, device: int = -1,
                 group=None, engine=None):
        dist = _dist()
        self.group = group
        self.rank = dist.get_rank(group) if dist else 0
        self.world = dist.get_world_size(group) if dist else 1
        self.embeddingDimension = int(embeddingDimension)
        self.locationCount = int(locationCount)
        self.ranges = row_ranges(self.locationCount, self.world)
        self.rowBegin, self.rowEnd = self.ranges[self.rank]
        self.engine = engine if engine is not None else Engine(embeddingDimension, locationCount, flags, device,
                                                               rows=(self.rowBegin, self.rowEnd))
        self._device = None
        if dist:
            import torch

            backend = dist.get_backend(group)
            self._device = torch.device("cuda", torch.cuda.current_device()) if backend == "nccl" else \
                torch.device("cpu")

    def close(self) -> None:
        if hasattr(self.engine, "close"):
            self.engine.close()

    # -- collectives
    def _all_reduce_sum(self, value: float) -> float:
        dist = _dist()
        if not dist or self.world == 1:
            return value
        import torch

        t = torch.tensor([value], dtype=torch.float64, device=self._device)
        dist.all_reduce(t, op=dist.ReduceOp.SUM, group=self.group)
        return float(t.item())

    def _all_gather_rows(self, local: np.ndarray) -> np.ndarray:
        p = self.embeddingDimension
        dist = _dist()
        if not dist or self.world == 1:
            return local.reshape(-1, p)
        import torch

        width = max(r1 - r0 for r0, r1 in self.ranges) * p
        buf = torch.zeros(width, dtype=torch.float64, device=self._device)
        buf[:local.size] = torch.from_numpy(np.ascontiguousarray(local).reshape(-1)).to(self._device)
        parts = [torch.empty_like(buf) for _ in range(self.world)]
        dist.all_gather(parts, buf, group=self.group)
        rows = [parts[r][:(r1 - r0) * p].cpu().numpy() for r, (r0, r1) in enumerate(self.ranges)]
        return np.concatenate(rows).reshape(self.locationCount, p)

    # -- AbstractMultiDimensionalScaling
    def setPairwiseData(self, data) -> None:
        """The full N x N delta (this rank keeps its rows) or this rank's rows alone."""
        a = np.asarray(data)
        n = self.locationCount
        if a.size == n * n:
            a = a.reshape(n, n)[self.rowBegin:self.rowEnd]
        self.engine.setPairwiseData(np.ascontiguousarray(a))

    def updateLocations(self, locationIndex: int, locations) -> None:
        self.engine.updateLocations(locationIndex, locations)

    def setParameters(self, parameters) -> None:
        self.engine.setParameters(parameters)

    def getSumOfIncrements(self) -> float:
        return self._all_reduce_sum(self.engine.getSumOfIncrements())

    def getLogLikelihood(self) -> float:
        return self._all_reduce_sum(self.engine.getLogLikelihood())

    def getLogLikelihoodGradient(self) -> np.ndarray:
        return self._all_gather_rows(np.asarray(self.engine.getLogLikelihoodGradient()))

    def storeState(self) -> None:
        self.engine.storeState()

    def restoreState(self) -> None:
        self.engine.restoreState()

    def acceptState(self) -> None:
        self.engine.acceptState()

    def makeDirty(self) -> None:
        self.engine.makeDirty()

    def getInternalDimension(self) -> int:
        return self.embeddingDimension
