"""Generates tests/golden/golden.npz from the MassiveMDS reference engine itself.

The reference's serial CPU engine (NewMultiDimensionalScaling, double and float
instantiations) is compiled from its own sources by oracle/Makefile into
oracle/_ref/libmdsref.so; this script drives it through mds::factory on seeded
inputs and stores inputs and outputs. The GPU machine has no reference tree, so the
parity tests read these fixtures instead.

Run from the repository root, where the reference sources are available:
    python tests/golden/make_golden.py
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

import oracle  # noqa: E402
from oracle.oracle import FLOAT, LEFT_TRUNCATION, ReferenceEngine  # noqa: E402

# (name, N, P, truncation, tau, float engine, nan pairs, seed)
CASES = [
    ("n5_p1_trunc", 5, 1, True, 1.0, False, 0, 11),
    ("n17_p2_trunc_nan", 17, 2, True, 1.0, False, 2, 12),
    ("n33_p3_plain", 33, 3, False, 1.7, False, 0, 13),
    ("n64_p2_trunc_float", 64, 2, True, 2.0, True, 0, 14),
    ("n129_p6_trunc", 129, 6, True, 0.5, False, 3, 15),
    ("n200_p2_trunc", 200, 2, True, 1.0, False, 0, 16),
    ("n150_p10_plain_float", 150, 10, False, 1.3, True, 0, 17),
]


def make_inputs(n, p, nan_pairs, seed):
    rng = np.random.default_rng(seed)
    y = rng.standard_normal((n, 10))
    diff = y[:, None, :] - y[None, :, :]
    delta = np.sqrt((diff * diff).sum(-1))
    np.fill_diagonal(delta, 0.0)
    for _ in range(nan_pairs):
        i, j = rng.choice(n, 2, replace=False)
        delta[i, j] = delta[j, i] = np.nan
    x = rng.standard_normal((n, p))
    return delta, x


def sequence(delta, x0, tau, flags, iters, seed):
    """The reference benchmark's loop (src/benchmark.cpp:250-309) on a small case:
    storeState, updateLocations(-1), getSumOfIncrements, restore (p = 0.75) or
    accept, getLogLikelihoodGradient. Returns every location set, restore draw,
    sum and gradient."""
    n, p = x0.shape
    rng = np.random.default_rng(seed)
    eng = ReferenceEngine(p, n, flags)
    eng.setPairwiseData(delta)
    eng.updateLocations(-1, x0)
    eng.setParameters(tau)
    eng.makeDirty()
    sums = [eng.getSumOfIncrements()]
    grads = [eng.getLogLikelihoodGradient()]
    xs, restores = [], []
    for _ in range(iters):
        eng.storeState()
        x = rng.standard_normal((n, p))
        xs.append(x)
        eng.updateLocations(-1, x)
        sums.append(eng.getSumOfIncrements())
        r = bool(rng.random() < 0.75)
        restores.append(r)
        if r:
            eng.restoreState()
        else:
            eng.acceptState()
        grads.append(eng.getLogLikelihoodGradient())
    eng.close()
    return np.array(xs), np.array(restores), np.array(sums), np.array(grads)


def main():
    if not oracle.reference_available():
        raise SystemExit("reference engine not available: the reference sources are needed")
    out = {}
    for name, n, p, trunc, tau, use_float, nans, seed in CASES:
        delta, x = make_inputs(n, p, nans, seed)
        flags = (LEFT_TRUNCATION if trunc else 0) | (FLOAT if use_float else 0)
        eng = ReferenceEngine(p, n, flags)
        eng.setPairwiseData(delta)
        eng.updateLocations(-1, x)
        eng.setParameters(tau)
        eng.makeDirty()
        s = eng.getSumOfIncrements()
        g = eng.getLogLikelihoodGradient()
        eng.close()
        out[f"{name}.delta"] = delta
        out[f"{name}.x"] = x
        out[f"{name}.meta"] = np.array([n, p, int(trunc), tau, int(use_float)], dtype=np.float64)
        out[f"{name}.sum"] = np.array(s)
        out[f"{name}.grad"] = g
        print(f"{name}: sum={s!r}")
    # state-machine sequence
    delta, x0 = make_inputs(40, 2, 1, 21)
    xs, restores, sums, grads = sequence(delta, x0, 1.5, LEFT_TRUNCATION, 8, 22)
    out.update({"seq.delta": delta, "seq.x0": x0, "seq.xs": xs, "seq.restores": restores, "seq.sums": sums,
                "seq.grads": grads, "seq.tau": np.array(1.5)})
    np.savez_compressed(os.path.join(HERE, "golden.npz"), **out)
    names = ", ".join(c[0] for c in CASES)
    print(f"wrote golden.npz: {names}, seq")


if __name__ == "__main__":
    main()
