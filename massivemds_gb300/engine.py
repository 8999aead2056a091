"""Python mirror of the MassiveMDS engine interface over the CUDA C ABI.

:class:`Engine` has the methods of ``mds::AbstractMultiDimensionalScaling``
(src/AbstractMultiDimensionalScaling.hpp:48-59) with the reference's names and
argument meaning; :func:`factory` mirrors ``mds::factory``
(src/factory.cpp:32-118) for the GPU branch. The module-level functions
``createEngine``, ``setPairwiseData``, ``updateLocations``, ``setPrecision``,
``getLogLikelihood`` and ``getGradient`` mirror the R package's user API
(R/mds.R:10-111, src/MassiveMDS.cpp:60-113), including its error messages.

Where the reference asserts (wrong lengths, src/NewMultiDimensionalScaling.hpp:140,148,258,263,283)
or exits, this engine raises :class:`massivemds_gb300._lib.MdsxError`.
"""
from __future__ import annotations

import ctypes
import math

import numpy as np

from . import flags as F
from ._lib import check, load

_dp = ctypes.POINTER(ctypes.c_double)


class Engine:
    """A GPU MDS engine: ``mds::AbstractMultiDimensionalScaling`` through libmdsx.so."""

    def __init__(self, embeddingDimension: int, locationCount: int, flags: int = 0, device: int = -1,
                 rows: tuple[int, int] | None = None):
        """``rows=(row_begin, row_end)`` makes an engine over those rows of delta
        only (mdsx_create_rows): setPairwiseData then takes the rows' (row_end -
        row_begin) x N values, getSumOfIncrements / getLogLikelihood return the
        rows' share and getLogLikelihoodGradient their gradient rows."""
        self._lib = load()
        h = ctypes.c_void_p()
        if rows is None:
            check(self._lib.mdsx_create(int(embeddingDimension), int(locationCount), int(flags), int(device),
                                        ctypes.byref(h)))
            rows = (0, int(locationCount))
        else:
            check(self._lib.mdsx_create_rows(int(embeddingDimension), int(locationCount), int(flags), int(device),
                                             int(rows[0]), int(rows[1]), ctypes.byref(h)))
        self._h = h
        self.embeddingDimension = int(embeddingDimension)
        self.locationCount = int(locationCount)
        self.flags = int(flags)
        self.rowBegin, self.rowEnd = int(rows[0]), int(rows[1])

    # -- lifetime
    def close(self) -> None:
        if getattr(self, "_h", None):
            self._lib.mdsx_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def _check(self, status: int) -> None:
        check(status, self._h)

    # -- AbstractMultiDimensionalScaling
    def updateLocations(self, locationIndex: int, locations) -> None:
        v = np.ascontiguousarray(locations, dtype=np.float64).ravel()
        self._check(self._lib.mdsx_update_locations(self._h, int(locationIndex), v.ctypes.data_as(_dp), v.size))

    def getSumOfIncrements(self) -> float:
        out = ctypes.c_double()
        self._check(self._lib.mdsx_get_sum_of_increments(self._h, ctypes.byref(out)))
        return out.value

    def getLogLikelihoodGradient(self, out: np.ndarray | None = None) -> np.ndarray:
        n = (self.rowEnd - self.rowBegin) * self.embeddingDimension
        if out is None:
            out = np.empty(n, dtype=np.float64)
        if out.dtype != np.float64 or not out.flags.c_contiguous or out.size != n:
            raise ValueError("gradient buffer must be a contiguous float64 array of N*P entries (rows*P for a row range)")
        self._check(self._lib.mdsx_get_log_likelihood_gradient(self._h, out.ctypes.data_as(_dp), out.size))
        return out

    def storeState(self) -> None:
        self._check(self._lib.mdsx_store_state(self._h))

    def restoreState(self) -> None:
        self._check(self._lib.mdsx_restore_state(self._h))

    def acceptState(self) -> None:
        self._check(self._lib.mdsx_accept_state(self._h))

    def setPairwiseData(self, data) -> None:
        arr = np.asarray(data)
        if arr.dtype == np.float32:
            v = np.ascontiguousarray(arr).ravel()
            self._check(self._lib.mdsx_set_pairwise_data_f32(
                self._h, v.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), v.size))
        else:
            v = np.ascontiguousarray(arr, dtype=np.float64).ravel()
            self._check(self._lib.mdsx_set_pairwise_data(self._h, v.ctypes.data_as(_dp), v.size))

    def setParameters(self, parameters) -> None:
        v = np.ascontiguousarray(np.atleast_1d(parameters), dtype=np.float64)
        self._check(self._lib.mdsx_set_parameters(self._h, v.ctypes.data_as(_dp), v.size))

    def makeDirty(self) -> None:
        self._check(self._lib.mdsx_make_dirty(self._h))

    def getInternalDimension(self) -> int:
        out = ctypes.c_int()
        self._check(self._lib.mdsx_get_internal_dimension(self._h, ctypes.byref(out)))
        return out.value

    # -- conveniences
    def getLogLikelihood(self) -> float:
        """0.5*(log tau - log 2pi)*N(N-1)/2 - sumOfIncrements (R/mds.R:24-28)."""
        out = ctypes.c_double()
        self._check(self._lib.mdsx_get_log_likelihood(self._h, ctypes.byref(out)))
        return out.value

    # -- device-resident API (pointers are integers: device addresses / cudaStream_t)
    def set_stream(self, stream: int | None) -> None:
        self._check(self._lib.mdsx_set_stream(self._h, ctypes.c_void_p(stream or 0)))

    def update_locations_device(self, d_locations: int) -> None:
        n = self.locationCount * self.embeddingDimension
        self._check(self._lib.mdsx_update_locations_device(self._h, ctypes.c_void_p(d_locations), n))

    def evaluate_device(self, d_sum: int | None, d_gradient: int | None) -> None:
        self._check(self._lib.mdsx_evaluate_device(self._h, ctypes.c_void_p(d_sum or 0),
                                                   ctypes.c_void_p(d_gradient or 0)))

    def set_sweep_schedule(self, schedule: int) -> None:
        """flags.SWEEP_ROWS or flags.SWEEP_PAIRS (mdsx_set_sweep_schedule)."""
        self._check(self._lib.mdsx_set_sweep_schedule(self._h, int(schedule)))

    def sweep_schedule(self) -> int:
        out = ctypes.c_int()
        self._check(self._lib.mdsx_get_sweep_schedule(self._h, ctypes.byref(out)))
        return out.value

    def last_launch_count(self) -> int:
        out = ctypes.c_int()
        self._check(self._lib.mdsx_last_launch_count(self._h, ctypes.byref(out)))
        return out.value


def factory(dim1: int, dim2: int, flags: int, device: int = -1, threads: int = 0) -> Engine:
    """``mds::factory`` for the GPU branch: OPENCL or CUDA flags select this engine.

    The reference's CPU engines (no OPENCL/CUDA bit) are not part of this
    package; asking for one raises.
    """
    if not flags & (F.OPENCL | F.CUDA):
        raise ValueError("factory: only GPU engines (OPENCL or CUDA flag) are provided by massivemds_gb300")
    return Engine(dim1, dim2, flags, device)


# ---------------------------------------------------------------- R-level API

class MdsEngine(dict):
    """The list ``createEngine`` returns in R (src/MassiveMDS.cpp:101-111), as a dict
    with attribute access."""

    __getattr__ = dict.__getitem__

    def __setattr__(self, key, value):
        self[key] = value


def createEngine(embeddingDimension: int, locationCount: int, truncation: bool, tbb: int = 0, simd: int = 0,
                 gpu: int = 1, single: bool = False) -> MdsEngine:
    """src/MassiveMDS.cpp:60-113. ``gpu > 0`` selects the CUDA engine on device ``gpu - 1``
    (the benchmark's numbering, src/benchmark.cpp:92); ``single`` selects FP32."""
    flags = 0
    if truncation:
        flags |= F.LEFT_TRUNCATION
    if gpu <= 0:
        raise ValueError("createEngine: this package provides the GPU engine only (gpu must be > 0)")
    flags |= F.OPENCL
    if single:
        flags |= F.FLOAT
    eng = Engine(embeddingDimension, locationCount, flags, gpu - 1)
    return MdsEngine(engine=eng, embeddingDimension=embeddingDimension, locationCount=locationCount,
                     dataInitialized=False, locationsInitialized=False, truncation=truncation, threads=0,
                     deviceNumber=gpu - 1, flags=flags, precision=None)


def setPairwiseData(engine: MdsEngine, data) -> MdsEngine:
    """R/mds.R:84-92."""
    data = np.asarray(data)
    if data.size != engine.locationCount * engine.locationCount:
        raise ValueError("Invalid data size")
    engine.engine.setPairwiseData(data)
    engine.dataInitialized = True
    return engine


def updateLocations(engine: MdsEngine, locations) -> MdsEngine:
    """R/mds.R:103-111: locations is an N x P matrix (row i = location i)."""
    loc = np.asarray(locations, dtype=np.float64)
    if loc.size != engine.locationCount * engine.embeddingDimension:
        raise ValueError("Invalid data size")
    engine.engine.updateLocations(-1, loc.reshape(engine.locationCount, engine.embeddingDimension))
    engine.locationsInitialized = True
    return engine


def setPrecision(engine: MdsEngine, precision: float) -> MdsEngine:
    """R/mds.R:68-72."""
    engine.engine.setParameters([precision])
    engine.precision = float(precision)
    return engine


def _require(engine: MdsEngine) -> None:
    if not engine.dataInitialized:
        raise RuntimeError("data are not set")
    if not engine.locationsInitialized:
        raise RuntimeError("locations are not set")
    if engine.precision is None:
        raise RuntimeError("precision is not set")


def getLogLikelihood(engine: MdsEngine) -> float:
    """R/mds.R:10-31."""
    _require(engine)
    s = engine.engine.getSumOfIncrements()
    observation_count = engine.locationCount * (engine.locationCount - 1) / 2
    return 0.5 * (math.log(engine.precision) - math.log(2 * math.pi)) * observation_count - s


def getGradient(engine: MdsEngine) -> np.ndarray:
    """R/mds.R:41-57: the gradient as an N x P matrix."""
    _require(engine)
    g = engine.engine.getLogLikelihoodGradient()
    return g.reshape(engine.locationCount, engine.embeddingDimension)
