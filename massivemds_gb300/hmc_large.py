"""HMC at scale: the full MDS posterior with learned precision and trait
precision on one GPU.

Workload: N = 50 000 locations, P = 3; latent points Y ~ N(0, I_20), delta =
||Y_i - Y_j|| + N(0, 0.05^2) noise per pair, mirrored, clipped at 0, stored
FP32 (10 GB); truncation on. The chain learns tau (Metropolis with the
reflected uniform proposal, R/Untitled.R:668-691) and the trait precision
(Wishart Gibbs draw, :694-700); 1000 iterations of 30 leapfrog steps from a
classical-MDS start, the step size tuned toward 0.8 acceptance over the first
200 (burn-in) iterations. Every accept uses the exact FP32-compensated
potential. The synthetic delta and the start are built on the GPU with torch
(host copies only for the engine's setPairwiseData).

By default the half-width of the tau proposal adapts toward 44 % acceptance
during burn-in (the reference's fixed 0.01 moves tau too slowly at this N;
--fixed-precision-proposal keeps it). With --surrogate a second chain from the
same start runs with the learned gradient surrogate (K = 512 landmarks, MLP of
3 hidden layers of width 512, trained on rows harvested during burn-in; exact
potential at every accept; fallback to exact gradients below 0.6 acceptance),
and both chains' min ESS/s are reported side by side.

Prints one JSON line: seconds per iteration, fused sweeps per second and the
bytes they read, acceptance, the learned tau, min ESS over invariant
functionals (tau included) and min ESS/s.
"""
from __future__ import annotations

import argparse
import json
import time

import numpy as np
import torch

from . import Engine, diagnostics, flags as F
from .hmc import hmc
from .surrogate import Surrogate


def make_delta(n: int, dim: int, noise_sd: float, seed: int, dev) -> torch.Tensor:
    g = torch.Generator(device=dev)
    g.manual_seed(seed)
    y = torch.randn(n, dim, generator=g, device=dev, dtype=torch.float64)
    d = torch.empty(n, n, dtype=torch.float32, device=dev)
    block = 4096
    for r0 in range(0, n, block):
        r1 = min(n, r0 + block)
        d[r0:r1] = torch.cdist(y[r0:r1], y, compute_mode="donot_use_mm_for_euclid_dist").float()
    # one noise draw per unordered pair, mirrored
    for r0 in range(0, n, block):
        r1 = min(n, r0 + block)
        e = torch.randn(r1 - r0, n, generator=g, device=dev, dtype=torch.float32) * noise_sd
        rows = torch.arange(r0, r1, device=dev)[:, None]
        cols = torch.arange(n, device=dev)[None, :]
        e = torch.where(cols > rows, e, torch.zeros((), device=dev))
        d[r0:r1] += e
    for r0 in range(0, n, block):  # lower triangle from the upper one
        r1 = min(n, r0 + block)
        upper = d[:, r0:r1].T.contiguous()  # rows r0..r1 of the transposed matrix
        rows = torch.arange(r0, r1, device=dev)[:, None]
        cols = torch.arange(n, device=dev)[None, :]
        d[r0:r1] = torch.where(cols < rows, upper, d[r0:r1])
    d.clamp_(min=0.0)
    d.fill_diagonal_(0.0)
    return d


def classical_mds_gpu(delta: torch.Tensor, p: int, iterations: int = 40, seed: int = 0) -> np.ndarray:
    """Top-p eigenvectors of -1/2 J delta^2 J by subspace iteration (on the GPU)."""
    n = delta.shape[0]
    g = torch.Generator(device=delta.device)
    g.manual_seed(seed)

    def bmul(v):
        v = v - v.mean(0)
        w = torch.empty_like(v)
        for r0 in range(0, n, 8192):
            r1 = min(n, r0 + 8192)
            w[r0:r1] = (delta[r0:r1].double() ** 2) @ v
        return -0.5 * (w - w.mean(0))

    v = torch.linalg.qr(torch.randn(n, p, generator=g, device=delta.device, dtype=torch.float64))[0]
    for _ in range(iterations):
        v = torch.linalg.qr(bmul(v))[0]
    lam = torch.clamp((v * bmul(v)).sum(0), min=0.0)
    return (v * lam.sqrt()).cpu().numpy()


def mean_squared_residual(delta: torch.Tensor, x: np.ndarray) -> float:
    """Mean of (delta_ij - |x_i - x_j|)^2 over i != j (on the GPU)."""
    n = delta.shape[0]
    xt = torch.as_tensor(x, device=delta.device)
    acc = 0.0
    for r0 in range(0, n, 4096):
        r1 = min(n, r0 + 4096)
        dist = torch.cdist(xt[r0:r1], xt, compute_mode="donot_use_mm_for_euclid_dist")
        acc += float(((delta[r0:r1].double() - dist) ** 2).sum())
    return acc / (n * (n - 1.0))


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--n", type=int, default=50_000)
    ap.add_argument("--p", type=int, default=3)
    ap.add_argument("--iterations", type=int, default=1000)
    ap.add_argument("--burn-in", type=int, default=200)
    ap.add_argument("--steps", type=int, default=30)
    ap.add_argument("--seed", type=int, default=11)
    ap.add_argument("--fixed-precision-proposal", action="store_true",
                    help="keep the reference's tau proposal half-width 0.01 throughout")
    ap.add_argument("--surrogate", action="store_true", help="also run the surrogate-gradient chain")
    ap.add_argument("--landmarks", type=int, default=512)
    ap.add_argument("--width", type=int, default=512)
    ap.add_argument("--layers", type=int, default=3)
    ap.add_argument("--harvest-rows", type=int, default=250)
    args = ap.parse_args(argv)

    dev = torch.device("cuda", 0)
    t0 = time.time()
    d = make_delta(args.n, 20, 0.05, args.seed, dev)
    x0 = classical_mds_gpu(d, args.p)
    tau0 = 1.0 / mean_squared_residual(d, x0)  # start tau at the residual precision of the start
    host = d.cpu().numpy()
    del d
    torch.cuda.empty_cache()
    e = Engine(args.p, args.n, F.FLOAT | F.LEFT_TRUNCATION)
    e.setPairwiseData(host)
    del host
    e.setParameters([tau0])
    setup = time.time() - t0

    rng = np.random.default_rng(args.seed)
    pairs = rng.integers(0, args.n, (50, 2))
    pairs = pairs[pairs[:, 0] != pairs[:, 1]]
    locs = rng.choice(args.n, 50, replace=False)
    common = dict(iterations=args.iterations, burn_in=args.burn_in, leapfrog_steps=args.steps, step_size=1e-3,
                  adapt_step_size=True, target_accept=0.8, learn_precision=True, precision_half_width=0.01,
                  adapt_precision_proposal=not args.fixed_precision_proposal, learn_trait_precision=True,
                  seed=args.seed, traced_pairs=pairs, traced_locations=locs)
    t = time.time()
    res = hmc(e, x0, **common)
    wall = time.time() - t
    sur_out = None
    if args.surrogate:
        e.setParameters([tau0])
        s = Surrogate(e, landmarks=args.landmarks, width=args.width, layers=args.layers,
                      max_training_rows=(args.burn_in - args.burn_in // 2) * args.harvest_rows, seed=args.seed)
        t = time.time()
        sres = hmc(e, x0, surrogate=s, harvest_iterations=args.burn_in, harvest_start=args.burn_in // 2,
                   harvest_rows=args.harvest_rows, train_steps=4000, train_batch=512, train_learning_rate=1e-3,
                   fallback_accept=0.6, fallback_window=50, **common)
        s_wall = time.time() - t
        s.close()
        scols = diagnostics.invariant_functionals(sres, include_precision=True)[args.burn_in:]
        s_mess, _ = diagnostics.min_ess(scols)
        sur_out = {"min_ess": s_mess, "min_ess_per_s": s_mess / sres.seconds, "seconds": sres.seconds,
                   "accept": sres.accept_rate, "fallback_iteration": sres.fallback_iteration,
                   "train_seconds": sres.train_seconds, "train_loss": sres.train_loss,
                   "surrogate_evaluations": sres.surrogate_evaluations, "wall_seconds": s_wall,
                   "tau_final": sres.precision}
    e.close()
    kept = args.iterations - args.burn_in
    cols = diagnostics.invariant_functionals(res, include_precision=True)[args.burn_in:]
    mess, k = diagnostics.min_ess(cols)
    tau_chain = res.column("precision")[args.burn_in:]
    sweeps_per_s = res.gradient_evaluations / wall
    out = {
        "metric": "HMC at scale (learned tau and trait precision)",
        "workload": {"n": args.n, "p": args.p, "iterations": args.iterations, "burn_in": args.burn_in,
                     "leapfrog_steps": args.steps, "delta_bytes": 4 * args.n * args.n},
        "seconds_per_iteration": res.seconds / kept,
        "wall_seconds": wall,
        "setup_seconds": setup,
        "sweeps": res.gradient_evaluations,
        "sweeps_per_s": sweeps_per_s,
        "sweep_gbs": sweeps_per_s * 4.0 * args.n * args.n / 1e9,
        "accept": res.accept_rate,
        "step_size": res.step_size,
        "tau_start": tau0,
        "tau_final": res.precision,
        "tau_mean": float(tau_chain.mean()),
        "tau_ess": diagnostics.ess(tau_chain),
        "min_ess": mess,
        "min_ess_functional": int(k),
        "min_ess_per_s": mess / res.seconds,
        "precision_proposal": "fixed 0.01" if args.fixed_precision_proposal else "adapted in burn-in",
        "tau_accept": float(np.mean(tau_chain[1:] != tau_chain[:-1])),
        "surrogate": sur_out,
        "ratio": (sur_out["min_ess_per_s"] / (mess / res.seconds)) if sur_out else None,
    }
    print(json.dumps(out))


if __name__ == "__main__":
    main()
