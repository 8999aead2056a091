"""Hamiltonian Monte Carlo for the MDS posterior on the GPU (mdsx_hmc_run).

Restates the reference's R sampler ``hmcsampler`` (R/Untitled.R:477-729):
leapfrog HMC on the latent locations with a matrix-normal prior, optional
Metropolis steps on the precision tau and Gibbs draws of the trait precision.
The whole chain runs in one call of the C ABI; this module packs the
configuration and unpacks the trace.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass

import numpy as np

from ._lib import check, load
from .engine import Engine

TRACE_BASE = 8
TRACE_COLUMNS = ("log_likelihood", "log_prior", "potential", "precision", "accepted", "step_size", "delta_h",
                 "surrogate")


class _Config(ctypes.Structure):
    _fields_ = [
        ("iterations", ctypes.c_int),
        ("burn_in", ctypes.c_int),
        ("leapfrog_steps", ctypes.c_int),
        ("step_size", ctypes.c_double),
        ("adapt_step_size", ctypes.c_int),
        ("target_accept", ctypes.c_double),
        ("learn_precision", ctypes.c_int),
        ("precision_half_width", ctypes.c_double),
        ("learn_trait_precision", ctypes.c_int),
        ("seed", ctypes.c_ulonglong),
        ("n_traced_pairs", ctypes.c_int),
        ("traced_pairs", ctypes.POINTER(ctypes.c_int)),
        ("n_traced_locations", ctypes.c_int),
        ("traced_locations", ctypes.POINTER(ctypes.c_int)),
        ("use_graph", ctypes.c_int),
        ("surrogate", ctypes.c_void_p),
        ("harvest_iterations", ctypes.c_int),
        ("harvest_start", ctypes.c_int),
        ("harvest_rows", ctypes.c_int),
        ("train_steps", ctypes.c_int),
        ("train_batch", ctypes.c_int),
        ("train_learning_rate", ctypes.c_double),
        ("fallback_accept", ctypes.c_double),
        ("fallback_window", ctypes.c_int),
        ("resume", ctypes.c_void_p),
        ("resume_bytes", ctypes.c_size_t),
        ("checkpoint", ctypes.c_void_p),
        ("checkpoint_capacity", ctypes.c_size_t),
        ("adapt_precision_proposal", ctypes.c_int),
    ]


class _Stats(ctypes.Structure):
    _fields_ = [
        ("accept_rate", ctypes.c_double),
        ("step_size", ctypes.c_double),
        ("seconds", ctypes.c_double),
        ("gradient_evaluations", ctypes.c_longlong),
        ("precision", ctypes.c_double),
        ("surrogate_evaluations", ctypes.c_longlong),
        ("fallback_iteration", ctypes.c_int),
        ("train_seconds", ctypes.c_double),
        ("train_loss", ctypes.c_double),
        ("checkpoint_bytes", ctypes.c_longlong),
    ]


@dataclass
class HmcResult:
    trace: np.ndarray            # iterations x (TRACE_BASE + pairs + locations)
    final_locations: np.ndarray  # N x P
    accept_rate: float
    step_size: float
    seconds: float
    gradient_evaluations: int
    precision: float
    n_pairs: int
    n_locations: int
    surrogate_evaluations: int = 0
    fallback_iteration: int = -1
    train_seconds: float = 0.0
    train_loss: float = float("nan")
    checkpoint: bytes | None = None  # the chain's state after its last iteration (``checkpoint=True``)

    def column(self, name: str) -> np.ndarray:
        return self.trace[:, TRACE_COLUMNS.index(name)]

    @property
    def pair_distances(self) -> np.ndarray:
        return self.trace[:, TRACE_BASE:TRACE_BASE + self.n_pairs]

    @property
    def location_norms(self) -> np.ndarray:
        return self.trace[:, TRACE_BASE + self.n_pairs:]


def hmc(engine: Engine, initial_locations, iterations: int, burn_in: int = 0, leapfrog_steps: int = 20,
        step_size: float = 0.01, adapt_step_size: bool = False, target_accept: float = 0.8,
        learn_precision: bool = False, precision_half_width: float = 0.01, learn_trait_precision: bool = False,
        seed: int = 666, traced_pairs=None, traced_locations=None, use_graph: bool = True, surrogate=None,
        harvest_iterations: int = 0, harvest_start: int | None = None, harvest_rows: int = 100, train_steps: int = 2000, train_batch: int = 512,
        train_learning_rate: float = 1e-3, fallback_accept: float = 0.6, fallback_window: int = 50,
        checkpoint: bool = False, resume: bytes | None = None, adapt_precision_proposal: bool = False) -> HmcResult:
    """Runs one chain on the engine's GPU; the engine must hold delta and tau.

    Defaults follow the reference: 20 leapfrog steps of 0.01 (trajectory 0.2,
    R/Untitled.R:509-510), precision proposal half-width 0.01 (:670).

    With a ``Surrogate``: the first ``harvest_iterations`` iterations use exact
    gradients, and those from ``harvest_start`` (default: half-way) harvest
    ``harvest_rows`` rows from the chain's state after each accept step; the
    surrogate is then trained (``train_*``) and drives the leapfrog kicks,
    with the exact potential deciding every accept, until the acceptance over
    the last ``fallback_window`` surrogate iterations drops below
    ``fallback_accept`` (exact gradients from then on).

    ``adapt_precision_proposal=True`` adapts the precision proposal's
    half-width toward 44 % acceptance during burn-in (the reference keeps
    ``precision_half_width`` fixed).

    ``checkpoint=True`` returns the chain's state after its last iteration in
    ``HmcResult.checkpoint``; ``resume=<those bytes>`` (same engine, delta and
    seed) continues that chain for ``iterations`` more iterations, ignoring
    ``initial_locations``, with ``burn_in`` still counted from the chain's
    first iteration. Exact-gradient chains only. See :func:`save_checkpoint`.
    """
    lib = load()
    n, p = engine.locationCount, engine.embeddingDimension
    x0 = np.ascontiguousarray(initial_locations, dtype=np.float64).reshape(n, p)
    pairs = np.ascontiguousarray(np.zeros((0, 2)) if traced_pairs is None else traced_pairs, dtype=np.int32)
    pairs = pairs.reshape(-1, 2)
    locs = np.ascontiguousarray(np.zeros(0) if traced_locations is None else traced_locations, dtype=np.int32)
    ip = ctypes.POINTER(ctypes.c_int)
    cfg = _Config(int(iterations), int(burn_in), int(leapfrog_steps), float(step_size), int(adapt_step_size),
                  float(target_accept), int(learn_precision), float(precision_half_width),
                  int(learn_trait_precision), int(seed), len(pairs), pairs.ctypes.data_as(ip), len(locs),
                  locs.ctypes.data_as(ip), int(use_graph), surrogate._h.value if surrogate is not None else None,
                  int(harvest_iterations), int(harvest_iterations // 2 if harvest_start is None else harvest_start),
                  int(harvest_rows), int(train_steps), int(train_batch),
                  float(train_learning_rate), float(fallback_accept), int(fallback_window))
    resume_buf = ctypes.create_string_buffer(bytes(resume), len(resume)) if resume is not None else None
    cap = lib_checkpoint_bytes(n, p) if checkpoint else 0
    ckpt_buf = ctypes.create_string_buffer(cap) if checkpoint else None
    cfg.resume = ctypes.cast(resume_buf, ctypes.c_void_p) if resume_buf is not None else None
    cfg.resume_bytes = len(resume) if resume is not None else 0
    cfg.checkpoint = ctypes.cast(ckpt_buf, ctypes.c_void_p) if ckpt_buf is not None else None
    cfg.checkpoint_capacity = cap
    cfg.adapt_precision_proposal = int(adapt_precision_proposal)
    cols = TRACE_BASE + len(pairs) + len(locs)
    trace = np.empty((iterations, cols), dtype=np.float64)
    final = np.empty((n, p), dtype=np.float64)
    stats = _Stats()
    dp = ctypes.POINTER(ctypes.c_double)
    check(lib.mdsx_hmc_run(engine._h, ctypes.c_void_p(ctypes.addressof(cfg)), x0.ctypes.data_as(dp),
                           trace.ctypes.data_as(dp), final.ctypes.data_as(dp),
                           ctypes.c_void_p(ctypes.addressof(stats))), engine._h)
    ckpt = ckpt_buf.raw[:stats.checkpoint_bytes] if checkpoint else None
    return HmcResult(trace, final, stats.accept_rate, stats.step_size, stats.seconds, stats.gradient_evaluations,
                     stats.precision, len(pairs), len(locs), stats.surrogate_evaluations, stats.fallback_iteration,
                     stats.train_seconds, stats.train_loss, ckpt)


def lib_checkpoint_bytes(n: int, p: int) -> int:
    """MDSX_HMC_CHECKPOINT_BYTES(N, P): the buffer a chain checkpoint needs."""
    return 112 + 16 * p * p + 16 * n * p + 8192


def save_checkpoint(path: str, data: bytes) -> None:
    """Writes a chain checkpoint to a file (atomically: a temporary file, then a rename)."""
    import os

    tmp = path + ".tmp"
    with open(tmp, "wb") as f:
        f.write(data)
        f.flush()
        os.fsync(f.fileno())
    os.replace(tmp, path)


def load_checkpoint(path: str) -> bytes:
    with open(path, "rb") as f:
        return f.read()
