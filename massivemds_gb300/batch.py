"""Batched multi-instance engine (mdsx_batch_* of the C ABI).

The reference drives many MDS problems through a process-wide vector of
engines addressed by an instance index (its JNI singleton,
src/jni/dr_inference_multidimensionalscaling_NativeMDSSingleton.cpp:10-100).
``Batch`` keeps that call surface (initialize -> add_instance, then
updateLocations / setPairwiseData / setParameters / getSumOfIncrements /
getLogLikelihoodGradient / makeDirty by index) but evaluates all instances
together: one persistent launch per embedding dimension on one GPU, captured
as a CUDA graph, with the schedule (stream-K units or a queue of whole row
blocks) and tile shape from the autotuner (``tune``).
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import flags as F
from ._lib import MdsxError, load

_dp = ctypes.POINTER(ctypes.c_double)
_fp = ctypes.POINTER(ctypes.c_float)


class Batch:
    def __init__(self, flags: int = F.FLOAT | F.LEFT_TRUNCATION, device: int = -1):
        self._lib = load()
        h = ctypes.c_void_p()
        st = self._lib.mdsx_batch_create(int(flags), int(device), ctypes.byref(h))
        if st != 0:
            raise MdsxError(st, "mdsx_batch_create failed (the batched path needs MDSX_FLAG_FLOAT)")
        self._h = h
        self._shapes: list[tuple[int, int]] = []

    def _check(self, status: int) -> None:
        if status != 0:
            msg = self._lib.mdsx_batch_last_error(self._h)
            raise MdsxError(status, msg.decode() if msg else "")

    def close(self) -> None:
        if getattr(self, "_h", None):
            self._lib.mdsx_batch_destroy(self._h)
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

    def __len__(self) -> int:
        return self._lib.mdsx_batch_instance_count(self._h)

    # -- the JNI singleton's surface, by instance index
    def add_instance(self, embeddingDimension: int, locationCount: int) -> int:
        k = ctypes.c_int()
        self._check(self._lib.mdsx_batch_add_instance(self._h, int(embeddingDimension), int(locationCount),
                                                      ctypes.byref(k)))
        self._shapes.append((int(locationCount), int(embeddingDimension)))
        return k.value

    initialize = add_instance

    def setPairwiseData(self, instance: int, data) -> None:
        n = self._shapes[instance][0]
        a = np.asarray(data)
        if a.dtype == np.float32:
            v = np.ascontiguousarray(a).reshape(-1)
            self._check(self._lib.mdsx_batch_set_pairwise_data_f32(self._h, int(instance), v.ctypes.data_as(_fp),
                                                                   v.size))
        else:
            v = np.ascontiguousarray(a, dtype=np.float64).reshape(-1)
            self._check(self._lib.mdsx_batch_set_pairwise_data(self._h, int(instance), v.ctypes.data_as(_dp),
                                                               v.size))
        assert v.size == n * n

    def setParameters(self, instance: int, parameters) -> None:
        v = np.ascontiguousarray(parameters, dtype=np.float64).reshape(-1)
        self._check(self._lib.mdsx_batch_set_parameters(self._h, int(instance), v.ctypes.data_as(_dp), v.size))

    def updateLocations(self, instance: int, locationIndex: int, locations) -> None:
        v = np.ascontiguousarray(locations, dtype=np.float64).reshape(-1)
        self._check(self._lib.mdsx_batch_update_locations(self._h, int(instance), int(locationIndex),
                                                          v.ctypes.data_as(_dp), v.size))

    def makeDirty(self) -> None:
        self._check(self._lib.mdsx_batch_make_dirty(self._h))

    def getSumOfIncrements(self, instance: int) -> float:
        out = ctypes.c_double()
        self._check(self._lib.mdsx_batch_get_sum_of_increments(self._h, int(instance), ctypes.byref(out)))
        return out.value

    def getLogLikelihood(self, instance: int) -> float:
        out = ctypes.c_double()
        self._check(self._lib.mdsx_batch_get_log_likelihood(self._h, int(instance), ctypes.byref(out)))
        return out.value

    def getLogLikelihoodGradient(self, instance: int) -> np.ndarray:
        n, p = self._shapes[instance]
        out = np.empty(n * p, dtype=np.float64)
        self._check(self._lib.mdsx_batch_get_log_likelihood_gradient(self._h, int(instance), out.ctypes.data_as(_dp),
                                                                     out.size))
        return out

    # -- batch-level calls
    def evaluate(self) -> None:
        self._check(self._lib.mdsx_batch_evaluate(self._h))

    def evaluate_device(self, d_sums: int | None = None, d_gradients: int | None = None) -> None:
        self._check(self._lib.mdsx_batch_evaluate_device(self._h, d_sums, d_gradients))

    def tune(self, repetitions: int = 5) -> int:
        c = ctypes.c_int()
        self._check(self._lib.mdsx_batch_tune(self._h, int(repetitions), ctypes.byref(c)))
        return c.value

    def group_shape(self, p: int) -> tuple[int, int, int, int]:
        """(schedule, rows per warp, CTAs per SM, grid) of dimension p's group;
        schedule 0 = stream-K units, 1 = row-block queue, 2 = unordered pairs."""
        sc, rw, ctas, grid = ctypes.c_int(), ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        self._check(self._lib.mdsx_batch_group_shape(self._h, int(p), ctypes.byref(sc), ctypes.byref(rw),
                                                     ctypes.byref(ctas), ctypes.byref(grid)))
        return sc.value, rw.value, ctas.value, grid.value

    def force_shape(self, p: int, rows_per_warp: int, ctas_per_sm: int = 2, schedule: int = 1) -> None:
        """Fixes dimension p's shape (schedule 2 needs P <= 6 and rows_per_warp 4);
        rows_per_warp 0 removes the override."""
        self._check(self._lib.mdsx_batch_force_shape(self._h, int(p), int(schedule), int(rows_per_warp),
                                                     int(ctas_per_sm)))
