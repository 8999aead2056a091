"""Learned gradient surrogate (mdsx_surrogate_* of the C ABI).

No counterpart in the reference. The surrogate approximates the exact
log-likelihood gradient of an engine's state,

    g_i ~= s * sum_k alpha_ik(f_i) (x_i - x_{l_k}),

over K landmark locations (a seeded random subset of the N locations), where
f_i holds the scaled residuals d(x_i, x_{l_k}) - delta_{i, l_k} (computed in
FP32 before the BF16 rounding) and the standardised dissimilarities
delta_{i, l_k}, and alpha_i is the output of an MLP
(2K -> width x layers, SiLU -> K). Forward and backward passes run on BF16
tensor cores with FP32 accumulation; Adam keeps FP32 master weights. The HMC
driver (``hmc(..., surrogate=...)``) harvests training rows from exact
trajectories, trains, and then uses the surrogate for the leapfrog kicks while
the exact potential decides every accept.
"""
from __future__ import annotations

import ctypes

import numpy as np

from ._lib import MdsxError, load
from .engine import Engine

_dp = ctypes.POINTER(ctypes.c_double)
_fp = ctypes.POINTER(ctypes.c_float)
_ip = ctypes.POINTER(ctypes.c_int)


class Surrogate:
    """A gradient surrogate bound to one engine (its delta, GPU and stream)."""

    def __init__(self, engine: Engine, landmarks: int = 256, width: int = 256, layers: int = 2,
                 max_training_rows: int = 50_000, seed: int = 0):
        self._lib = load()
        self.engine = engine
        h = ctypes.c_void_p()
        st = self._lib.mdsx_surrogate_create(engine._h, int(landmarks), int(width), int(layers),
                                             int(max_training_rows), int(seed), ctypes.byref(h))
        if st != 0:
            msg = self._lib.mdsx_last_error(engine._h)
            raise MdsxError(st, msg.decode() if msg else "")
        self._h = h

    def _check(self, status: int) -> None:
        if status != 0:
            msg = self._lib.mdsx_surrogate_last_error(self._h)
            raise MdsxError(status, msg.decode() if msg else "")

    def close(self) -> None:
        if getattr(self, "_h", None):
            self._lib.mdsx_surrogate_destroy(self._h)
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

    # ---------------------------------------------------------------- info
    def info(self) -> dict:
        ints = (ctypes.c_int * 8)()
        reals = (ctypes.c_double * 5)()
        self._check(self._lib.mdsx_surrogate_info(self._h, ints, reals))
        keys = ("n", "p", "landmarks", "width", "layers", "rows", "max_rows", "adam_steps")
        out = dict(zip(keys, list(ints)))
        out.update(zip(("mu", "inv_sigma", "scale", "target_scale", "inv_sigma_r"), list(reals)))
        return out

    @property
    def n(self) -> int:
        return self.info()["n"]

    def landmarks(self) -> np.ndarray:
        k = self.info()["landmarks"]
        out = np.empty(k, dtype=np.int32)
        self._check(self._lib.mdsx_surrogate_landmarks(self._h, out.ctypes.data_as(_ip)))
        return out

    def layer_shapes(self) -> list[tuple[int, int]]:
        inf = self.info()
        k, w, layers = inf["landmarks"], inf["width"], inf["layers"]
        fan_in = [2 * k] + [w] * layers
        fan_out = [w] * layers + [k]
        return list(zip(fan_out, fan_in))

    def _params(self, layer: int, which: int, w=None, b=None):
        fo, fi = self.layer_shapes()[layer]
        if w is None:
            w = np.empty((fo, fi), dtype=np.float32)
            b = np.empty(fo, dtype=np.float32)
        else:
            w = np.ascontiguousarray(w, dtype=np.float32).reshape(fo, fi)
            b = np.ascontiguousarray(b, dtype=np.float32).reshape(fo)
        self._check(self._lib.mdsx_surrogate_parameters(self._h, int(layer), which, w.ctypes.data_as(_fp),
                                                        b.ctypes.data_as(_fp)))
        return w, b

    def parameters(self, layer: int):
        """FP32 master weight [out][in] and bias of `layer` (the last is the output layer)."""
        return self._params(layer, 0)

    def set_parameters(self, layer: int, weight, bias) -> None:
        self._params(layer, 1, weight, bias)

    def parameter_gradients(self, layer: int):
        return self._params(layer, 2)

    # ------------------------------------------------------------- training
    def add_state(self, locations, gradient, rows: int, seed: int = 0) -> None:
        """Harvest `rows` rows at random locations of one exact state."""
        n, p = self.engine.locationCount, self.engine.embeddingDimension
        x = np.ascontiguousarray(locations, dtype=np.float64).reshape(n, p)
        g = np.ascontiguousarray(gradient, dtype=np.float64).reshape(n, p)
        self._check(self._lib.mdsx_surrogate_add_state(self._h, x.ctypes.data_as(_dp), g.ctypes.data_as(_dp),
                                                       int(rows), int(seed)))

    def training_rows(self, first: int, count: int):
        """(features [count, 2K], directions [count, K, P], targets [count, P]) as float32."""
        inf = self.info()
        k, p = inf["landmarks"], inf["p"]
        feat = np.empty((count, 2 * k), dtype=np.float32)
        dirs = np.empty((count, k, p), dtype=np.float32)
        tgt = np.empty((count, p), dtype=np.float32)
        self._check(self._lib.mdsx_surrogate_training_rows(self._h, int(first), int(count), feat.ctypes.data_as(_fp),
                                                           dirs.ctypes.data_as(_fp), tgt.ctypes.data_as(_fp)))
        return feat, dirs, tgt

    def train(self, steps: int, batch: int = 512, learning_rate: float = 1e-3, seed: int = 0) -> np.ndarray:
        """Adam steps on seeded uniform batches; returns the per-step loss."""
        losses = np.empty(max(1, steps), dtype=np.float64)
        self._check(self._lib.mdsx_surrogate_train(self._h, int(steps), int(batch), float(learning_rate), int(seed),
                                                   losses.ctypes.data_as(_dp)))
        return losses[:steps]

    def batch_gradient(self, rows) -> float:
        """Loss of the given training rows; their parameter gradients are left
        for parameter_gradients()."""
        r = np.ascontiguousarray(rows, dtype=np.int32)
        loss = ctypes.c_double()
        self._check(self._lib.mdsx_surrogate_batch_gradient(self._h, r.ctypes.data_as(_ip), len(r),
                                                            ctypes.byref(loss)))
        return loss.value

    # ------------------------------------------------------------ inference
    def gradient(self, locations) -> np.ndarray:
        """Surrogate log-likelihood gradient (N x P) at the given locations."""
        n, p = self.engine.locationCount, self.engine.embeddingDimension
        x = np.ascontiguousarray(locations, dtype=np.float64).reshape(n, p)
        out = np.empty((n, p), dtype=np.float64)
        self._check(self._lib.mdsx_surrogate_gradient(self._h, x.ctypes.data_as(_dp), out.ctypes.data_as(_dp)))
        return out


def gemm_bf16(a_bits: np.ndarray, b_bits: np.ndarray, a_t: bool, b_t: bool, m: int, n: int, k: int) -> np.ndarray:
    """The MLP's tensor-core GEMM on BF16 bit patterns (uint16), FP32 result [m, n]."""
    lib = load()
    a = np.ascontiguousarray(a_bits, dtype=np.uint16)
    b = np.ascontiguousarray(b_bits, dtype=np.uint16)
    c = np.empty((m, n), dtype=np.float32)
    up = ctypes.POINTER(ctypes.c_ushort)
    st = lib.mdsx_test_gemm_bf16(int(a_t), int(b_t), m, n, k, a.ctypes.data_as(up), b.ctypes.data_as(up),
                                 c.ctypes.data_as(_fp))
    if st != 0:
        raise MdsxError(st, "mdsx_test_gemm_bf16 failed")
    return c
