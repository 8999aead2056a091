"""ctypes bindings for the oracle libraries (test infrastructure, not product).

``liboracle.so`` is the C restatement (``mds_oracle.c``); ``_ref/libmdsref.so``
is the reference engine built from its own sources by ``oracle/Makefile``.
"""
from __future__ import annotations

import ctypes
import math
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_ORACLE_SO = os.path.join(_HERE, "liboracle.so")
_REF_SO = os.path.join(_HERE, "_ref", "libmdsref.so")


def reference_root() -> str | None:
    """Root of a MassiveMDS reference checkout (its ``src/`` and ``inst/extdata``):
    ``$MDSX_REFERENCE_ROOT`` when set, else a sibling directory named
    ``reference`` beside this repository; None when neither holds the sources."""
    env = os.environ.get("MDSX_REFERENCE_ROOT")
    cands = [env] if env else [os.path.join(os.path.dirname(os.path.dirname(_HERE)), "reference")]
    for c in cands:
        if c and os.path.isfile(os.path.join(c, "src", "NewMultiDimensionalScaling.hpp")):
            return os.path.abspath(c)
    return None


REFERENCE_ROOT = reference_root()

_dbl_p = ctypes.POINTER(ctypes.c_double)


def build(reference: bool | None = None) -> None:
    """Compile liboracle.so (and the reference engine when its sources exist)."""
    targets = ["oracle"]
    if reference is None:
        reference = REFERENCE_ROOT is not None
    args = ["make", "-s", "-C", _HERE]
    if reference:
        if REFERENCE_ROOT is None:
            raise RuntimeError("no reference checkout: set MDSX_REFERENCE_ROOT")
        targets.append("ref")
        args.append(f"REF={REFERENCE_ROOT}")
    subprocess.run([*args, *targets], check=True)


_lib = None


def _oracle():
    global _lib
    if _lib is None:
        if not os.path.exists(_ORACLE_SO):
            build(reference=False)
        lib = ctypes.CDLL(_ORACLE_SO)
        lib.mdso_sweep_rows.restype = ctypes.c_int
        lib.mdso_sweep_rows.argtypes = [
            ctypes.c_void_p, ctypes.c_int, _dbl_p, ctypes.c_int64, ctypes.c_int, ctypes.c_double,
            ctypes.c_int, ctypes.c_int64, ctypes.c_int64, _dbl_p, _dbl_p, ctypes.c_int,
        ]
        lib.mdso_sum_of_increments.restype = ctypes.c_double
        lib.mdso_sum_of_increments.argtypes = [
            ctypes.c_void_p, ctypes.c_int, _dbl_p, ctypes.c_int64, ctypes.c_int, ctypes.c_double,
            ctypes.c_int, ctypes.c_int,
        ]
        lib.mdso_gradient.restype = ctypes.c_int
        lib.mdso_gradient.argtypes = [
            ctypes.c_void_p, ctypes.c_int, _dbl_p, ctypes.c_int64, ctypes.c_int, ctypes.c_double,
            ctypes.c_int, _dbl_p, ctypes.c_int,
        ]
        lib.mdso_log_likelihood.restype = ctypes.c_double
        lib.mdso_log_likelihood.argtypes = [ctypes.c_double, ctypes.c_int64, ctypes.c_double]
        lib.mdso_port_eval_rows_f32.restype = ctypes.c_double
        lib.mdso_port_eval_rows_f32.argtypes = [
            ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_int, ctypes.c_float, ctypes.c_int,
            ctypes.c_int64, ctypes.c_int64, ctypes.c_void_p, ctypes.c_int,
        ]
        lib.mdso_port_eval_rows.restype = ctypes.c_double
        lib.mdso_port_eval_rows.argtypes = [
            ctypes.c_void_p, ctypes.c_int, _dbl_p, ctypes.c_int64, ctypes.c_int, ctypes.c_double,
            ctypes.c_int, ctypes.c_int64, ctypes.c_int64, _dbl_p, ctypes.c_int,
        ]
        _lib = lib
    return _lib


def _delta_args(delta):
    if delta.dtype == np.float32:
        d = np.ascontiguousarray(delta, dtype=np.float32)
        return d, 1
    d = np.ascontiguousarray(delta, dtype=np.float64)
    return d, 0


def _threads(threads):
    return int(threads) if threads else (os.cpu_count() or 1)


def sum_of_increments(delta, x, tau, truncation=True, threads=None) -> float:
    """Reference ``getSumOfIncrements()`` on a full N x N ``delta`` (float64 or float32)."""
    d, is32 = _delta_args(delta)
    x = np.ascontiguousarray(x, dtype=np.float64)
    n, p = x.shape
    assert d.shape == (n, n)
    return _oracle().mdso_sum_of_increments(
        d.ctypes.data, is32, x.ctypes.data_as(_dbl_p), n, p, float(tau), int(bool(truncation)),
        _threads(threads))


def gradient(delta, x, tau, truncation=True, threads=None) -> np.ndarray:
    """Reference ``getLogLikelihoodGradient()``; returns an (N, P) array."""
    d, is32 = _delta_args(delta)
    x = np.ascontiguousarray(x, dtype=np.float64)
    n, p = x.shape
    out = np.empty((n, p), dtype=np.float64)
    rc = _oracle().mdso_gradient(d.ctypes.data, is32, x.ctypes.data_as(_dbl_p), n, p, float(tau),
                                 int(bool(truncation)), out.ctypes.data_as(_dbl_p), _threads(threads))
    if rc != 0:
        raise RuntimeError("oracle gradient failed")
    return out


def sweep_rows(delta, x, tau, truncation, row_begin, row_end, threads=None):
    """Per-row (unhalved) increment sums and gradient rows for rows [row_begin, row_end)."""
    d, is32 = _delta_args(delta)
    x = np.ascontiguousarray(x, dtype=np.float64)
    n, p = x.shape
    rows = row_end - row_begin
    row_sum = np.empty(rows, dtype=np.float64)
    grad = np.empty((rows, p), dtype=np.float64)
    rc = _oracle().mdso_sweep_rows(d.ctypes.data, is32, x.ctypes.data_as(_dbl_p), n, p, float(tau),
                                   int(bool(truncation)), row_begin, row_end,
                                   row_sum.ctypes.data_as(_dbl_p), grad.ctypes.data_as(_dbl_p),
                                   _threads(threads))
    if rc != 0:
        raise RuntimeError("oracle sweep failed")
    return row_sum, grad


def evaluate(delta, x, tau, truncation=True, threads=None):
    """getSumOfIncrements() and getLogLikelihoodGradient() from one pass over
    delta (the two calls above each sweep the whole matrix)."""
    n = x.shape[0]
    row_sum, grad = sweep_rows(delta, x, tau, truncation, 0, n, threads)
    half = math.fsum(row_sum) / 2.0
    return (half if truncation else 0.5 * tau * half), grad


def log_likelihood(sum_of_incs: float, n: int, tau: float) -> float:
    """R/mds.R:24-28."""
    return _oracle().mdso_log_likelihood(float(sum_of_incs), int(n), float(tau))


def port_eval_rows(delta, x, tau, truncation, row_begin, row_end, threads=1):
    """The reference's per-evaluation work order over a row range (CPU baseline timing)."""
    d, is32 = _delta_args(delta) if delta.dtype in (np.float32, np.float64) else (delta, 0)
    x = np.ascontiguousarray(x, dtype=np.float64)
    n, p = x.shape
    grad = np.empty((row_end - row_begin, p), dtype=np.float64)
    s = _oracle().mdso_port_eval_rows(d.ctypes.data, is32, x.ctypes.data_as(_dbl_p), n, p,
                                      float(tau), int(bool(truncation)), row_begin, row_end,
                                      grad.ctypes.data_as(_dbl_p), int(threads))
    return s, grad


def port_eval_rows_f32(delta32, x, tau, truncation, row_begin, row_end, threads=1):
    """The reference FLOAT engine's per-evaluation work order over a row range
    (single-precision CPU baseline timing); delta32 must be float32."""
    d = np.ascontiguousarray(delta32, dtype=np.float32)
    x32 = np.ascontiguousarray(x, dtype=np.float32)
    n, p = x32.shape
    grad = np.empty((row_end - row_begin, p), dtype=np.float32)
    s = _oracle().mdso_port_eval_rows_f32(d.ctypes.data, x32.ctypes.data, n, p, float(tau), int(bool(truncation)),
                                          row_begin, row_end, grad.ctypes.data, int(threads))
    return s, grad


def reference_available() -> bool:
    if os.path.exists(_REF_SO):
        return True
    if REFERENCE_ROOT is not None:
        try:
            build(reference=True)
        except (subprocess.CalledProcessError, OSError):
            return False
        return os.path.exists(_REF_SO)
    return False


# Reference flag bits (src/flags.h:6-14).
FLOAT, TBB, OPENCL, LEFT_TRUNCATION = 1 << 2, 1 << 3, 1 << 4, 1 << 5


class ReferenceEngine:
    """The reference's own CPU engine through mds::factory (src/factory.cpp:32-118)."""

    _ref = None

    @classmethod
    def _load(cls):
        if cls._ref is None:
            if not reference_available():
                raise RuntimeError("reference engine unavailable (sources not present)")
            lib = ctypes.CDLL(_REF_SO)
            vp = ctypes.c_void_p
            lib.mdsref_create.restype = vp
            lib.mdsref_create.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_long, ctypes.c_int]
            for name in ("mdsref_destroy", "mdsref_store_state", "mdsref_restore_state",
                         "mdsref_accept_state", "mdsref_make_dirty"):
                getattr(lib, name).argtypes = [vp]
                getattr(lib, name).restype = None
            lib.mdsref_set_pairwise_data.argtypes = [vp, _dbl_p, ctypes.c_size_t]
            lib.mdsref_set_pairwise_data.restype = None
            lib.mdsref_update_locations.argtypes = [vp, ctypes.c_int, _dbl_p, ctypes.c_size_t]
            lib.mdsref_update_locations.restype = None
            lib.mdsref_set_parameters.argtypes = [vp, _dbl_p, ctypes.c_size_t]
            lib.mdsref_set_parameters.restype = None
            lib.mdsref_get_sum_of_increments.argtypes = [vp]
            lib.mdsref_get_sum_of_increments.restype = ctypes.c_double
            lib.mdsref_get_log_likelihood_gradient.argtypes = [vp, _dbl_p, ctypes.c_size_t]
            lib.mdsref_get_log_likelihood_gradient.restype = None
            lib.mdsref_get_internal_dimension.argtypes = [vp]
            lib.mdsref_get_internal_dimension.restype = ctypes.c_int
            cls._ref = lib
        return cls._ref

    def __init__(self, embedding_dimension, location_count, flags=0, threads=0):
        self._lib = self._load()
        self.p, self.n = int(embedding_dimension), int(location_count)
        self._h = self._lib.mdsref_create(self.p, self.n, int(flags), int(threads))
        if not self._h:
            raise RuntimeError("mdsref_create failed")

    def close(self):
        if self._h:
            self._lib.mdsref_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def setPairwiseData(self, delta):
        d = np.ascontiguousarray(delta, dtype=np.float64).ravel()
        self._lib.mdsref_set_pairwise_data(self._h, d.ctypes.data_as(_dbl_p), d.size)

    def updateLocations(self, index, x):
        v = np.ascontiguousarray(x, dtype=np.float64).ravel()
        self._lib.mdsref_update_locations(self._h, int(index), v.ctypes.data_as(_dbl_p), v.size)

    def setParameters(self, tau):
        v = np.array([tau], dtype=np.float64)
        self._lib.mdsref_set_parameters(self._h, v.ctypes.data_as(_dbl_p), 1)

    def getSumOfIncrements(self):
        return self._lib.mdsref_get_sum_of_increments(self._h)

    def getLogLikelihoodGradient(self):
        out = np.empty(self.n * self.p, dtype=np.float64)
        self._lib.mdsref_get_log_likelihood_gradient(self._h, out.ctypes.data_as(_dbl_p), out.size)
        return out.reshape(self.n, self.p)

    def storeState(self):
        self._lib.mdsref_store_state(self._h)

    def restoreState(self):
        self._lib.mdsref_restore_state(self._h)

    def acceptState(self):
        self._lib.mdsref_accept_state(self._h)

    def makeDirty(self):
        self._lib.mdsref_make_dirty(self._h)

    def getInternalDimension(self):
        return self._lib.mdsref_get_internal_dimension(self._h)
