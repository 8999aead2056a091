"""Plain versus surrogate-gradient HMC on one GPU: minimum ESS per second over
invariant functionals at matched posterior means.

Workload (clustered MDS posterior): N = 5000 locations, P = 2; latent points
from 5 cluster centres ~ N(0, 9 I_10), 1000 points each, within-cluster
N(0, I_10); delta = Euclidean distance + N(0, 0.1^2) noise per pair, clipped at
0 and mirrored; tau = 1 fixed; prior iid N(0, 1) (identity tree and trait
covariance). Both chains: 2000 iterations of 20 leapfrog steps from the same
classical-MDS start, the step size tuned by dual averaging to 0.8 acceptance
during the first 500 (burn-in) iterations. The surrogate chain harvests 200
(state, exact gradient) rows from each of iterations 250..499 (50 000 rows;
each row is one location of one harvested state), trains the 2 x 256 BF16 MLP
over K = 256 landmarks, then drives its leapfrog steps with the surrogate;
the exact potential decides every accept and the chain returns to exact
gradients if the acceptance over 50 surrogate iterations drops below 0.6.

ESS: Geyer initial monotone sequence over the 1500 kept draws of the
log-likelihood, 50 fixed pair distances and 50 fixed location norms; time:
wall time of the kept iterations (training time reported separately).
Prints one JSON line.
"""
from __future__ import annotations

import argparse
import json
import time

import numpy as np

from . import Engine, data, diagnostics, flags as F
from .hmc import hmc
from .surrogate import Surrogate


def summarise(res, kept_from):
    cols = diagnostics.invariant_functionals(res)[kept_from:]
    mess, k = diagnostics.min_ess(cols)
    means = cols.mean(0)
    mcse = np.array([diagnostics.mcse_mean(cols[:, j]) for j in range(cols.shape[1])])
    return cols, mess, k, means, mcse


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--n", type=int, default=5000)
    ap.add_argument("--iterations", type=int, default=2000)
    ap.add_argument("--burn-in", type=int, default=500)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--landmarks", type=int, default=256)
    ap.add_argument("--width", type=int, default=256)
    ap.add_argument("--layers", type=int, default=2)
    ap.add_argument("--harvest-rows", type=int, default=200)
    ap.add_argument("--train-steps", type=int, default=4000)
    ap.add_argument("--train-batch", type=int, default=512)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--seed", type=int, default=1)
    args = ap.parse_args(argv)

    n, p, tau = args.n, 2, 1.0
    delta = data.clustered_delta(n, dim=10, clusters=5, noise_sd=0.1, seed=5)
    x0 = data.classical_mds(delta, p)
    rng = np.random.default_rng(args.seed)
    pairs = rng.integers(0, n, (50, 2))
    pairs = pairs[pairs[:, 0] != pairs[:, 1]]
    locs = rng.choice(n, 50, replace=False)

    e = Engine(p, n, F.FLOAT | F.LEFT_TRUNCATION)
    e.setPairwiseData(delta)
    e.setParameters([tau])
    common = dict(iterations=args.iterations, burn_in=args.burn_in, leapfrog_steps=args.steps, step_size=0.003,
                  adapt_step_size=True, target_accept=0.8, seed=args.seed, traced_pairs=pairs,
                  traced_locations=locs)
    t = time.time()
    plain = hmc(e, x0, **common)
    plain_wall = time.time() - t
    s = Surrogate(e, landmarks=args.landmarks, width=args.width, layers=args.layers,
                  max_training_rows=(args.burn_in - args.burn_in // 2) * args.harvest_rows, seed=args.seed)
    t = time.time()
    sur = hmc(e, x0, surrogate=s, harvest_iterations=args.burn_in, harvest_start=args.burn_in // 2,
              harvest_rows=args.harvest_rows, train_steps=args.train_steps, train_batch=args.train_batch,
              train_learning_rate=args.lr, fallback_accept=0.6, fallback_window=50, **common)
    sur_wall = time.time() - t
    g_exact = (e.updateLocations(-1, sur.final_locations), np.asarray(e.getLogLikelihoodGradient()).reshape(n, p))[1]
    g_sur = s.gradient(sur.final_locations)
    # the trained surrogate alone (no fallback) from the plain chain's end: its
    # acceptance and the cost of a surrogate iteration
    only_iters = 300
    only = hmc(e, plain.final_locations, iterations=only_iters, leapfrog_steps=args.steps, step_size=plain.step_size,
               seed=args.seed + 1, surrogate=s, harvest_iterations=0, train_steps=0, fallback_accept=0.0)
    s.close()
    e.close()

    kb = args.burn_in
    _, ess_p, kp, mean_p, mcse_p = summarise(plain, kb)
    _, ess_s, ks, mean_s, mcse_s = summarise(sur, kb)
    z = np.abs(mean_p - mean_s) / np.sqrt(mcse_p ** 2 + mcse_s ** 2)
    out = {
        "metric": "min ESS/s, surrogate vs plain HMC",
        "workload": {"n": n, "p": p, "tau": tau, "iterations": args.iterations, "burn_in": kb,
                     "leapfrog_steps": args.steps, "landmarks": args.landmarks, "mlp": [args.width] * args.layers,
                     "harvest_rows": (kb - kb // 2) * args.harvest_rows},
        "plain": {"min_ess": ess_p, "seconds": plain.seconds, "min_ess_per_s": ess_p / plain.seconds,
                  "accept": plain.accept_rate, "step_size": plain.step_size,
                  "gradient_evaluations": plain.gradient_evaluations, "wall": plain_wall},
        "surrogate": {"min_ess": ess_s, "seconds": sur.seconds, "min_ess_per_s": ess_s / sur.seconds,
                      "min_ess_per_s_with_training": ess_s / (sur.seconds + sur.train_seconds),
                      "accept": sur.accept_rate, "fallback_iteration": sur.fallback_iteration,
                      "train_seconds": sur.train_seconds, "train_loss": sur.train_loss,
                      "surrogate_evaluations": sur.surrogate_evaluations,
                      "gradient_evaluations": sur.gradient_evaluations, "wall": sur_wall,
                      "relative_gradient_error": float(np.linalg.norm(g_sur - g_exact) / np.linalg.norm(g_exact))},
        "surrogate_only": {"iterations": only_iters, "accept": only.accept_rate,
                           "ms_per_iteration": 1e3 * only.seconds / only_iters,
                           "plain_ms_per_iteration": 1e3 * plain.seconds / (args.iterations - kb)},
        "ratio": (ess_s / sur.seconds) / (ess_p / plain.seconds),
        "means_within_2_mcse": float(np.mean(z <= 2.0)),
        "max_mean_z": float(np.max(z)),
    }
    print(json.dumps(out))


if __name__ == "__main__":
    main()
