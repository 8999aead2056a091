"""Why a per-location landmark surrogate cannot carry the leapfrog: how much of
the change of the exact gradient along a chain is explained locally.

For states x* and x = x* + dx a few iterations apart on an exact HMC chain at
equilibrium (clustered workload, tau = 1, started at classical MDS), the change
dg = g(x) - g(x*) of the exact log-likelihood gradient is compared with its
linearisation through the exact Hessian H = d g / d x (by central differences
of the engine's gradient at x*), truncated three ways:
  own        dg_i ~ H_ii dx_i                        (the location's own block)
  landmarks  own + sum_k H_{i,l_k} dx_{l_k}           (K landmark locations)
  scaled     own + (N - 1) / K * sum_k H_{i,l_k} dx_{l_k}  (landmarks standing in for all)
  full       sum_j H_ij dx_j                          (every location: the linearisation itself)
and the relative error ||dg - prediction|| / ||dg|| of each is reported. A
surrogate that sees location i and K landmarks (O(N K) work) can at best
reproduce the "landmarks" or "scaled" predictions; if those leave most of dg
unexplained while "full" explains it, the gradient's change is carried by the
coupling to all N - 1 other locations and no such surrogate can track it.

Prints one JSON line. Runs on the GPU through the engine (about a minute).
"""
from __future__ import annotations

import argparse
import json

import numpy as np

from . import Engine, data, flags as F
from .hmc import hmc


def hessian(e: Engine, x: np.ndarray, h: float = 1e-4) -> np.ndarray:
    """H[i, a, j, b] = d g_{i,a} / d x_{j,b} by central differences of the exact gradient."""
    n, p = x.shape
    hess = np.empty((n, p, n, p))
    for j in range(n):
        for b in range(p):
            xp = x.copy()
            xp[j, b] += h
            e.updateLocations(-1, xp)
            gp = np.asarray(e.getLogLikelihoodGradient()).reshape(n, p)
            xp[j, b] -= 2 * h
            e.updateLocations(-1, xp)
            gm = np.asarray(e.getLogLikelihoodGradient()).reshape(n, p)
            hess[:, :, j, b] = (gp - gm) / (2 * h)
    return hess


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--n", type=int, default=600)
    ap.add_argument("--landmarks", type=int, default=64)
    ap.add_argument("--iterations", type=int, default=1500)
    ap.add_argument("--gap", type=int, default=1, help="iterations between x* and x")
    ap.add_argument("--pairs", type=int, default=5, help="(x*, x) pairs evaluated")
    ap.add_argument("--seed", type=int, default=3)
    args = ap.parse_args(argv)

    n, p, k = args.n, 2, args.landmarks
    delta = data.clustered_delta(n, dim=10, clusters=5, noise_sd=0.1, seed=5).astype(np.float64)
    x0 = data.classical_mds(delta, p)
    e = Engine(p, n, F.LEFT_TRUNCATION)  # FP64 gradients for the differences
    e.setPairwiseData(delta)
    e.setParameters([1.0])
    rng = np.random.default_rng(args.seed)
    landmarks = rng.choice(n, k, replace=False)
    # an exact chain; keep its states at the chosen iterations
    burn = args.iterations // 2
    res = hmc(e, x0, iterations=burn, burn_in=burn, leapfrog_steps=20, step_size=0.003, adapt_step_size=True,
              target_accept=0.8, seed=args.seed)
    x = res.final_locations
    errs = {"own": [], "landmarks": [], "scaled": [], "full": []}
    norms = []
    for m in range(args.pairs):
        step = hmc(e, x, iterations=max(1, args.gap), leapfrog_steps=20, step_size=res.step_size,
                   seed=args.seed + 100 + m)
        x_new = step.final_locations
        if np.array_equal(x_new, x):  # rejected: move on
            x = x_new
            continue
        hess = hessian(e, x)
        e.updateLocations(-1, x)
        g0 = np.asarray(e.getLogLikelihoodGradient()).reshape(n, p)
        e.updateLocations(-1, x_new)
        g1 = np.asarray(e.getLogLikelihoodGradient()).reshape(n, p)
        dg, dx = g1 - g0, x_new - x
        own = np.einsum("iaib,ib->ia", hess, dx)
        land = np.einsum("iajb,jb->ia", hess[:, :, landmarks, :], dx[landmarks])
        own_in_land = np.zeros_like(own)  # a landmark's own block is already in `own`
        own_in_land[landmarks] = own[landmarks]
        full = np.einsum("iajb,jb->ia", hess, dx)
        preds = {"own": own, "landmarks": own + land - own_in_land,
                 "scaled": own + (n - 1) / k * (land - own_in_land), "full": full}
        den = np.linalg.norm(dg)
        for key, pred in preds.items():
            errs[key].append(float(np.linalg.norm(dg - pred) / den))
        norms.append(float(den / np.linalg.norm(g0)))
        x = x_new
    e.close()
    out = {"metric": "relative error of truncated linearisations of the gradient change along an exact chain",
           "workload": {"n": n, "p": p, "tau": 1.0, "landmarks": k, "gap_iterations": args.gap,
                        "pairs": len(norms), "chain_accept": res.accept_rate, "step_size": res.step_size},
           "relative_error": {key: (float(np.mean(v)) if v else None) for key, v in errs.items()},
           "relative_change_of_gradient": float(np.mean(norms)) if norms else None}
    print(json.dumps(out))


if __name__ == "__main__":
    main()
