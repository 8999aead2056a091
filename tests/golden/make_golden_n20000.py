"""Generates tests/golden/golden_n20000.npz: the reference engine on the full
N = 20 000 workload.

Workload: N = 20 000, P = 2, tau = 2, truncation on; delta = distances of
20 000 points iid N(0, I_10) plus iid N(0, 0.05^2) noise drawn once per
unordered pair, mirrored and clipped at 0, stored FP32 (massivemds_gb300.data
.noisy_delta with seed 666, the matrix bench.py times). delta itself is not
stored: the tests regenerate it from the seed and check its fingerprint (the
FP64 sum of its entries and of their squares) before comparing.

For each of three location states x ~ N(0, 1) (drawn in FP32, so they are
stored exactly in FP32), the reference's own CPU engine
(NewMultiDimensionalScaling through mds::factory, compiled from its sources by
oracle/Makefile; the TBB code path on the std::thread stand-in scheduler)
computes getSumOfIncrements() and getLogLikelihoodGradient() twice:

* the double engine on the FP32-rounded delta promoted to double -- the
  values the engine's FP64 modes (FP64 over FP32-stored delta, and FP64-stored
  delta holding the same values) must match within 1e-10 / 1e-9, and the FP32
  mode within 1e-5;
* the FLOAT engine (flags FLOAT) on the same delta -- the reference's own
  single-precision answer, kept to show how far it lies from the double one.

Run from the repository root where the reference sources are available:
    python tests/golden/make_golden_n20000.py
"""
from __future__ import annotations

import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

import oracle  # noqa: E402
from massivemds_gb300 import data as gen  # noqa: E402
from oracle.oracle import FLOAT, LEFT_TRUNCATION, TBB, ReferenceEngine  # noqa: E402

N, P, TAU = 20000, 2, 2.0
STATES = 3
DELTA_SEED = 666
X_SEED = 20000
OUT = os.path.join(HERE, "golden_n20000.npz")


def workload_delta():
    return gen.noisy_delta(N, dim=10, noise_sd=0.05, seed=DELTA_SEED, dtype=np.float32)


def fingerprint(delta32):
    """FP64 sum of the entries and of their squares, accumulated row by row."""
    s = s2 = 0.0
    for r0 in range(0, delta32.shape[0], 1000):
        blk = delta32[r0:r0 + 1000].astype(np.float64)
        s += float(blk.sum())
        s2 += float(np.square(blk).sum())
    return np.array([s, s2])


def states():
    rng = np.random.default_rng(X_SEED)
    return [rng.standard_normal((N, P), dtype=np.float32) for _ in range(STATES)]


def run_engine(delta64, xs, flags, threads):
    eng = ReferenceEngine(P, N, flags | TBB | LEFT_TRUNCATION, threads)
    eng.setPairwiseData(delta64)
    eng.setParameters(TAU)
    sums, grads = [], []
    for x in xs:
        t = time.time()
        eng.updateLocations(-1, x.astype(np.float64))
        sums.append(eng.getSumOfIncrements())
        grads.append(eng.getLogLikelihoodGradient())
        print(f"  flags {flags:#x}: sum {sums[-1]!r} ({time.time() - t:.1f} s)", flush=True)
    eng.close()
    return np.array(sums), np.array(grads)


def main():
    if not oracle.reference_available():
        raise SystemExit("reference engine not available: the reference sources are needed")
    threads = os.cpu_count() or 1
    delta32 = workload_delta()
    fp = fingerprint(delta32)
    xs = states()
    delta64 = delta32.astype(np.float64)
    del delta32
    print("double engine", flush=True)
    s64, g64 = run_engine(delta64, xs, 0, threads)
    print("FLOAT engine", flush=True)
    s32, g32 = run_engine(delta64, xs, FLOAT, threads)
    # the FLOAT engine's gradient is float internally: stored exactly in FP32
    assert np.array_equal(g32.astype(np.float32).astype(np.float64), g32)
    np.savez_compressed(OUT, x=np.array(xs), delta_fingerprint=fp,
                        meta=np.array([N, P, TAU, DELTA_SEED, 0.05]),
                        sum_f64=s64, grad_f64=g64, sum_float=s32, grad_float=g32.astype(np.float32))
    print(f"wrote {OUT}")


if __name__ == "__main__":
    main()
