"""Batched multi-instance sweep versus one engine per instance, on one GPU.

Workload (uneven batch): 64 independent instances, N_k ~ U{500..8000} (seeded),
P_k cycling 2, 3, 6, tau_k ~ Gamma(shape 2, scale 1), delta_k = Euclidean
distances of N_k points iid N(0, I_10) (no noise), stored FP32, truncation on.
One batch evaluation = one fused likelihood + gradient sweep of every
instance. Algorithmic bytes per batch evaluation: sum_k N_k^2 * 4.

Arms, each timed with CUDA events after warm-up, inputs resident on the GPU:
  batched   mdsx_batch_evaluate_device: one graph launch (one persistent
            kernel per dimension group, schedule and shape from the tuner);
  engines   64 single-instance engines, mdsx_evaluate_device on each engine's
            own stream, all enqueued before one synchronisation (engines
            overlap on the GPU: the strongest use of separate engines);
  engines_sync  the reference's many-engines pattern as its JNI layer drives
            it: per instance, one synchronous evaluation and read-back
            (makeDirty, getSumOfIncrements, getLogLikelihoodGradient);
  e2e       the batch through its host API: every instance's locations from
            host memory, evaluation, every sum and gradient back to the host.
Prints one JSON line.
"""
from __future__ import annotations

import argparse
import json
import time

import numpy as np
import torch

from . import Engine, flags as F
from . import data as gen
from .batch import Batch


def make_instances(count: int, seed: int):
    rng = np.random.default_rng(seed)
    ns = rng.integers(500, 8001, count)
    ps = [(2, 3, 6)[k % 3] for k in range(count)]
    taus = rng.gamma(2.0, 1.0, count)
    return [(int(ns[k]), ps[k], float(taus[k]), int(rng.integers(1 << 30))) for k in range(count)]


def timed(fn, steps, stream):
    start = torch.cuda.Event(enable_timing=True)
    end = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    start.record(stream)
    for _ in range(steps):
        fn()
    end.record(stream)
    torch.cuda.synchronize()
    return start.elapsed_time(end) / 1e3 / steps


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--instances", type=int, default=64)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--seed", type=int, default=3)
    ap.add_argument("--tune", type=int, default=1, help="run the autotuner first")
    args = ap.parse_args(argv)

    spec = make_instances(args.instances, args.seed)
    t0 = time.time()
    batch = Batch(F.FLOAT | F.LEFT_TRUNCATION)
    engines = []
    locs = []
    for n, p, tau, s in spec:
        delta = gen.pairwise_distances(gen.latent_points(n, 10, s), dtype=np.float32)
        x = np.random.default_rng(s + 1).standard_normal((n, p))
        k = batch.add_instance(p, n)
        batch.setPairwiseData(k, delta)
        batch.updateLocations(k, -1, x)
        batch.setParameters(k, [tau])
        e = Engine(p, n, F.FLOAT | F.LEFT_TRUNCATION)
        e.setPairwiseData(delta)
        e.updateLocations(-1, x)
        e.setParameters([tau])
        engines.append(e)
        locs.append(x)
        del delta
    setup_s = time.time() - t0
    bytes_per_eval = sum(4.0 * n * n for n, _, _, _ in spec)
    candidates = batch.tune(repetitions=5) if args.tune else 0
    shapes = {p: batch.group_shape(p) for p in sorted({p for _, p, _, _ in spec})}

    dev = torch.device("cuda", 0)
    total_grad = sum(n * p for n, p, _, _ in spec)
    d_sums = torch.empty(4 * len(spec), dtype=torch.float64, device=dev)
    d_grads = torch.empty(total_grad, dtype=torch.float64, device=dev)
    stream = torch.cuda.Stream(device=dev)
    # the batch and the engines run on their own streams; events on the default
    # stream bracket them after device-wide synchronisation
    for _ in range(args.warmup):
        batch.evaluate_device(d_sums.data_ptr(), d_grads.data_ptr())
    torch.cuda.synchronize()
    cur = torch.cuda.current_stream(dev)

    def batched():
        batch.evaluate_device(d_sums.data_ptr(), d_grads.data_ptr())

    t_batch = timed(lambda: (batched(), torch.cuda.synchronize()), args.steps, cur)
    egrad = [torch.empty(n * p, dtype=torch.float64, device=dev) for n, p, _, _ in spec]
    esum = torch.empty(len(spec), dtype=torch.float64, device=dev)

    def many():
        for k, e in enumerate(engines):
            e.evaluate_device(esum[k:k + 1].data_ptr(), egrad[k].data_ptr())

    for _ in range(args.warmup):
        many()
    torch.cuda.synchronize()
    t_engines = timed(lambda: (many(), torch.cuda.synchronize()), args.steps, cur)

    # the reference's pattern: synchronous calls, one instance after the other
    def many_sync():
        for e in engines:
            e.makeDirty()
            e.getSumOfIncrements()
            e.getLogLikelihoodGradient()

    many_sync()
    t = time.perf_counter()
    for _ in range(args.steps):
        many_sync()
    t_sync = (time.perf_counter() - t) / args.steps

    # end to end through the host API
    for _ in range(args.warmup):
        batch.evaluate()
    t = time.perf_counter()
    for _ in range(args.steps):
        for k, x in enumerate(locs):
            batch.updateLocations(k, -1, x)
        batch.evaluate()
        for k in range(len(spec)):
            batch.getSumOfIncrements(k)
    t_e2e = (time.perf_counter() - t) / args.steps
    h2d = sum(x.nbytes for x in locs)
    d2h = 8 * (4 * len(spec) + total_grad)

    for e in engines:
        e.close()
    batch.close()
    out = {
        "metric": "batched instance-evals/s",
        "workload": {"instances": len(spec), "n_range": [500, 8000], "p_cycle": [2, 3, 6],
                     "sum_n2": int(sum(n * n for n, _, _, _ in spec)), "bytes_per_batch_eval": bytes_per_eval},
        "batched": {"seconds_per_batch_eval": t_batch, "instance_evals_per_s": len(spec) / t_batch,
                    "gbs": bytes_per_eval / t_batch / 1e9},
        "engines": {"seconds_per_batch_eval": t_engines, "instance_evals_per_s": len(spec) / t_engines,
                    "gbs": bytes_per_eval / t_engines / 1e9},
        "engines_sync": {"seconds_per_batch_eval": t_sync, "instance_evals_per_s": len(spec) / t_sync,
                         "gbs": bytes_per_eval / t_sync / 1e9},
        "e2e": {"seconds_per_batch_eval": t_e2e, "instance_evals_per_s": len(spec) / t_e2e,
                "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "speedup_vs_engines": t_engines / t_batch,
        "speedup_vs_engines_sync": t_sync / t_batch,
        "tuned_candidates": candidates,
        "shapes": {str(p): {"schedule": ("stream-K", "row-block queue", "unordered pairs")[s[0]], "rows_per_warp": s[1],
                            "ctas_per_sm": s[2], "grid": s[3]} for p, s in shapes.items()},
        "setup_seconds": setup_s,
    }
    print(json.dumps(out))


if __name__ == "__main__":
    main()
