"""Benchmark of the fused MDS likelihood+gradient sweep on GB300.

Workload (one "step"): the N=20 000, P=2 evaluation batch -- 200 fused
log-likelihood + gradient evaluations, each at fresh locations x ~ N(0,1),
over delta = distances of 20 000 points iid N(0, I_10) plus iid N(0, 0.05^2)
noise clipped at 0, stored FP32 (1.6 GB), tau = 2, truncation on, FP32 pair
arithmetic with compensated FP32 partials and FP64 reductions.

  value  evals/s with delta and the location pool resident in HBM (device API:
         mdsx_update_locations_device + mdsx_evaluate_device), CUDA events on
         the engine's stream.
  e2e    the same evaluations through the reference-facing API with host
         buffers: updateLocations(-1, x) / getSumOfIncrements() /
         getLogLikelihoodGradient(out), copies inside the timed region.
  roofline  the sweep's algorithmic bytes per evaluation (N^2 * 4 + 2 N P * 4)
         over the mean CUDA-event duration of its kernels (the unordered-pair
         sweep and its finish kernel, or the row-block sweep with --schedule
         rows), against the measured HBM peak.
  cpu_baseline  the oracle's port of the reference's per-evaluation work
         (likelihood pass + gradient pass, libm transcendentals) on all host
         cores over a bounded sample of rows, scaled to evals/s.

--impl reference times that CPU port as the reference arm.
Multi-GPU (torchrun): every rank runs the same workload on its own GPU
(independent replicas); value sums all ranks' evaluations over the slowest
rank's time.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, REPO)

N, P, TAU = 20000, 2, 2.0
EVALS_PER_STEP = 200
METRIC = "loglik+grad evals/s & HBM GB/s at N=20k; HMC minESS/s surrogate vs plain, 1 GPU"
UNIT = "evals/s"
def workload(n: int, precision: str = "f32", evals: int = EVALS_PER_STEP) -> str:
    math = "FP32 pairs + FP64 reductions" if precision == "f32" else "FP64 pairs (DELTA_F32 mode)"
    return (f"fused loglik+grad sweep, N={n}, P=2, tau=2, truncation, delta FP32-stored ({n * n * 4 / 1e9:.2f} GB), "
            f"{math}, {evals} evals per step at fresh locations")
DATA = ("synthetic: delta = ||Y_i - Y_j|| + N(0, 0.05^2) noise clipped at 0, Y ~ N(0, I_10) (seed 666); "
        "x ~ N(0,1) per evaluation")


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="mdsx", choices=["mdsx", "reference"])
    ap.add_argument("--n", type=int, default=N)
    ap.add_argument("--precision", default="f32", choices=["f32", "f64"],
                    help="pair arithmetic: f32 (the headline; FP32 pairs, FP64 reductions) or f64 (FP64 pairs over "
                         "the same FP32-stored delta; bound by the FP64 pipe, 10 evaluations per step)")
    ap.add_argument("--schedule", default="pairs", choices=["pairs", "rows"],
                    help="sweep schedule: each unordered pair once (default) or the row-block schedule")
    ap.add_argument("--cpu-seconds", type=float, default=4.0, help="wall time of one CPU baseline sample")
    ap.add_argument("--workload", default="sweep", choices=["sweep", "c1"],
                    help="sweep: the headline N=20000 FP32 sweep; c1: the reference's benchmark case "
                         "(N=1000, FP64, 100 iterations through the host API)")
    return ap.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def peaks():
    path = os.path.join(REPO, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def profiled_traffic(schedule):
    """DRAM bytes per evaluation from the committed ncu summary of that schedule, if present."""
    name = "pair_sweep_f32_n20000.txt" if schedule == "pairs" else "sweep_f32_n20000.txt"
    path = os.path.join(REPO, "profiles", name)
    try:
        with open(path) as f:
            for line in f:
                if line.startswith("traffic_bytes_per_launch:"):
                    return float(line.split(":", 1)[1])
    except OSError:
        pass
    return None


class ClockSampler:
    """nvidia-smi clocks and throttle reasons every 200 ms while running."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append((time.time(), line.strip()))

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self, t0, t1):
        rows = []
        for t, line in self.lines:
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                rows.append((t, float(parts[1]), float(parts[2]), parts[5:9]))
            except ValueError:
                continue
        inside = [r for r in rows if t0 <= r[0] <= t1] or rows
        if not inside:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no nvidia-smi samples"], "samples": 0}
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in inside for k, v in enumerate(r[3]) if v.lower() == "active"})
        return {"sm_mhz": statistics.median(r[1] for r in inside), "sm_max_mhz": max(r[2] for r in inside),
                "reasons": reasons, "samples": len(inside)}


def cpu_port_sample(delta, x_rows, tau, target_seconds):
    """Times the oracle port over a bounded row sample; returns (evals/s, cores, sample text)."""
    import oracle

    n = delta.shape[0]
    cores = os.cpu_count() or 1
    rows = max(cores, 16)
    t = time.perf_counter()
    oracle.port_eval_rows(delta, x_rows, tau, True, 0, rows, threads=cores)
    dt = time.perf_counter() - t
    rows = int(min(n, max(rows, rows * target_seconds / max(dt, 1e-6))))
    t = time.perf_counter()
    oracle.port_eval_rows(delta, x_rows, tau, True, 0, rows, threads=cores)
    dt = time.perf_counter() - t
    evals_per_s = (rows / n) / dt
    sample = (f"rows 0..{rows - 1} of the N={n} matrix (likelihood pass + gradient pass, all {n} columns), "
              f"{dt:.2f} s on {cores} threads, scaled by N/rows")
    return evals_per_s, cores, sample


def make_delta(n):
    import numpy as np

    from massivemds_gb300 import data as gen

    return gen.noisy_delta(n, dim=10, noise_sd=0.05, seed=666, dtype=np.float32)


def across_ranks_max(value: float, world: int, device) -> float:
    """The largest value over all ranks (every rank gets it); the job's time is
    its slowest replica's."""
    if world <= 1:
        return value
    import torch

    t = torch.tensor([value], dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def job_throughput(units_per_rank: int, world: int, seconds: float) -> float:
    """Whole-job throughput: the units all ranks processed over the slowest rank's time."""
    return units_per_rank * world / seconds


def run_c1(args):
    """The reference's own benchmark case: N = 1000, P = 2, FP64, truncation,
    tau = 1, delta = distances of 1000 points iid N(0, I_10), x ~ N(0, 1); one
    iteration = updateLocations(-1, x) + getLogLikelihood() +
    getLogLikelihoodGradient() through the engine's host API (the call sequence
    src/benchmark.cpp:250-309 times on its CPU engines). cpu_baseline: the same
    per-iteration work in the oracle's C port of the reference serial engine,
    on all host threads."""
    import numpy as np
    import torch

    rank, world, local = dist_env()
    if rank != 0:
        return
    import massivemds_gb300 as m
    from massivemds_gb300 import data as gen

    n, p, tau, iters = 1000, 2, 1.0, 100
    delta = gen.euclidean_delta(n, dim=10, seed=666)
    xs = np.random.default_rng(667).standard_normal((args.warmup + args.steps, iters, n, p))
    e = m.Engine(p, n, m.flags.LEFT_TRUNCATION, local)
    e.setPairwiseData(delta)
    e.setParameters([tau])
    grad = np.empty(n * p)

    def step(batch):
        for k in range(iters):
            e.updateLocations(-1, batch[k])
            e.getLogLikelihood()
            e.getLogLikelihoodGradient(grad)

    for w in range(args.warmup):
        step(xs[w])
    sampler = ClockSampler(local)
    sampler.start()
    time.sleep(0.3)
    torch.cuda.synchronize()
    t0 = time.time()
    for s_ in range(args.steps):
        step(xs[args.warmup + s_])
    t1 = time.time()
    sampler.stop()
    e.close()
    sec_per_step = (t1 - t0) / args.steps
    value = iters / sec_per_step

    import oracle  # cpu_baseline leg

    cores = os.cpu_count() or 1
    t = time.perf_counter()
    sample_iters = 10
    for k in range(sample_iters):
        oracle.sum_of_increments(delta, xs[0, k], tau, True, threads=cores)
        oracle.gradient(delta, xs[0, k], tau, True, threads=cores)
    cpu_value = sample_iters / (time.perf_counter() - t)
    line = {
        "metric": "iterations/s (updateLocations + getLogLikelihood + getLogLikelihoodGradient)",
        "value": value, "unit": "iterations/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1000.0 * sec_per_step, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64", "data": "synthetic: delta = ||Y_i - Y_j||, Y ~ N(0, I_10) (seed 666); x ~ N(0,1) per iteration",
        "config": {"workload": "reference benchmark case: N=1000, P=2, FP64, truncation, tau=1, 100 iterations "
                               "per step through the host API", "n": n, "p": p, "tau": tau,
                   "iterations_per_step": iters, "l2": "delta 8 MB stays in L2 (timed as a user would see it)"},
        "e2e": {"value": value, "unit": "iterations/s", "h2d_bytes_per_step": iters * n * p * 8,
                "d2h_bytes_per_step": iters * (n * p * 8 + 8)},
        "clocks": sampler.summary(t0, t1),
        "cpu_baseline": {"value": cpu_value, "unit": "iterations/s", "cores": cores, "kind": "port",
                         "sample": f"{sample_iters} iterations of the same workload"},
    }
    print(json.dumps(line), flush=True)


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    import numpy as np

    delta = make_delta(args.n)
    x = np.random.default_rng(667).standard_normal((args.n, P))
    vals = []
    info = None
    for _ in range(args.warmup + args.steps):
        v, cores, sample = cpu_port_sample(delta, x, TAU, args.cpu_seconds)
        vals.append(v)
        info = (cores, sample)
    vals = vals[args.warmup:]
    value = statistics.mean(vals)
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 * EVALS_PER_STEP / value,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": DATA,
        "config": {"workload": workload(args.n).replace("FP32 pairs + FP64 reductions", "reference CPU port in FP64"),
                   "n": args.n, "p": P, "tau": TAU, "evals_per_step": EVALS_PER_STEP},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": info[0], "kind": "port", "sample": info[1]},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": ("reference engine compiled from its sources is not available on this host (its sources are "
                 "not here); the oracle's port of the reference serial engine's per-evaluation work is timed"),
    }
    print(json.dumps(line), flush=True)


def run_mdsx(args):
    import numpy as np
    import torch

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    import massivemds_gb300 as m

    n = args.n
    f64 = args.precision == "f64"
    evals = 10 if f64 else EVALS_PER_STEP
    delta = make_delta(n)
    eng = m.Engine(P, n, (m.flags.DELTA_F32 if f64 else m.flags.FLOAT) | m.flags.LEFT_TRUNCATION, local)
    eng.set_sweep_schedule(m.flags.SWEEP_PAIRS if args.schedule == "pairs" else m.flags.SWEEP_ROWS)
    eng.setPairwiseData(delta)
    eng.setParameters([TAU])
    stream = torch.cuda.Stream()
    eng.set_stream(stream.cuda_stream)

    # location pool: one set per evaluation of a step
    rng = np.random.default_rng(1000 + rank)
    pool_host = torch.from_numpy(rng.standard_normal((evals, n, P))).pin_memory()
    pool_dev = pool_host.to(f"cuda:{local}")
    d_sum = torch.zeros(1, dtype=torch.float64, device=f"cuda:{local}")

    def device_step(events=None):
        for k in range(evals):
            eng.update_locations_device(pool_dev[k].data_ptr())
            if events is not None:
                events[k][0].record(stream)
            eng.evaluate_device(d_sum.data_ptr(), None)
            if events is not None:
                events[k][1].record(stream)

    torch.cuda.synchronize()
    for _ in range(args.warmup):
        device_step()
    torch.cuda.synchronize()

    sampler = ClockSampler(local)
    sampler.start()
    time.sleep(0.5)
    kev = [[(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
            for _ in range(evals)] for _ in range(args.steps)]
    start, stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    t0 = time.time()
    start.record(stream)
    for s in range(args.steps):
        device_step(kev[s])
    stop.record(stream)
    torch.cuda.synchronize()
    t1 = time.time()
    if world > 1:
        torch.distributed.barrier()
    sampler.stop()
    elapsed_ms = start.elapsed_time(stop)
    kernel_ms = statistics.mean(a.elapsed_time(b) for ev in kev for a, b in ev)
    launches = eng.last_launch_count()  # sweep launches per evaluation
    gpu_launches = args.steps * evals * (launches + 1)  # + the location conversion kernel

    elapsed_ms = across_ranks_max(elapsed_ms, world, f"cuda:{local}")
    value = job_throughput(args.steps * evals, world, elapsed_ms / 1000.0)

    # end to end through the reference-facing API with host buffers
    eng.set_stream(None)
    grad_host = torch.empty(n * P, dtype=torch.float64).pin_memory()
    g_np = grad_host.numpy()
    pool_np = pool_host.numpy()
    for k in range(min(evals, 10)):
        eng.updateLocations(-1, pool_np[k])
        eng.getSumOfIncrements()
        eng.getLogLikelihoodGradient(g_np)
    e2e_steps = max(1, args.steps)
    if world > 1:
        torch.distributed.barrier()
    t = time.perf_counter()
    for _ in range(e2e_steps):
        for k in range(evals):
            eng.updateLocations(-1, pool_np[k])
            eng.getSumOfIncrements()
            eng.getLogLikelihoodGradient(g_np)
    e2e_s = time.perf_counter() - t
    e2e_s = across_ranks_max(e2e_s, world, f"cuda:{local}")
    e2e_value = job_throughput(e2e_steps * evals, world, e2e_s)

    hbm_peak, peak_kind = peaks()
    bytes_per_launch = float(n) * n * 4 + 2.0 * n * P * 4
    achieved = bytes_per_launch / (kernel_ms / 1000.0) / 1e9
    traffic = profiled_traffic(args.schedule) if n == N else None  # the committed captures are of N = 20000
    if f64:
        kernel_name = ("pair_kernel<2,true,PairMathF64<float>> + pair_finish_kernel<2,double>"
                       if args.schedule == "pairs" else "sweep_kernel<double,float,2,true>")
        traffic = None  # FP64-pipe bound: the HBM fraction below is small by construction
    else:
        kernel_name = ("pair_kernel<2,true,PairMathF32> + pair_finish_kernel<2,float>" if args.schedule == "pairs"
                       else "sweep_kernel<float,float,2,true>")

    line = None
    if rank == 0:
        x0 = pool_np[0]
        cpu_v, cores, sample = cpu_port_sample(delta, x0, TAU, args.cpu_seconds)
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": elapsed_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": args.precision, "data": DATA,
            "config": {"workload": workload(n, args.precision, evals), "n": n, "p": P, "tau": TAU, "evals_per_step": evals,
                       "schedule": args.schedule, "precision": args.precision,
                       "delta_bytes": n * n * 4, "l2": f"inputs larger than L2 ({n * n * 4 / 1e9:.2f} GB delta vs 129 MB L2), no flush",
                       "parallelism": f"replicas x{world}" if world > 1 else "single GPU"},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
                         "frac": achieved / hbm_peak, "traffic": traffic,
                         "kernel": kernel_name, "kernel_ms": kernel_ms,
                         "peak_kind": peak_kind},
            "e2e": {"value": e2e_value, "unit": UNIT,
                    "h2d_bytes_per_step": evals * n * P * 8,
                    "d2h_bytes_per_step": evals * (n * P * 8 + 32)},
            "gpu_launches": gpu_launches,
            "clocks": sampler.summary(t0, t1),
            "cpu_baseline": {"value": cpu_v, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample},
        }
    eng.close()
    if world > 1:
        torch.distributed.destroy_process_group()
    if line is not None:
        print(json.dumps(line), flush=True)


def main():
    args = parse()
    if args.workload == "c1":
        if args.impl == "reference":
            print(json.dumps({"impl": "reference", "unavailable": "the c1 workload's CPU time is its cpu_baseline"}))
        else:
            run_c1(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_mdsx(args)


if __name__ == "__main__":
    main()
