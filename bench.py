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
  parity  after the timed region: the sums of every evaluation of the last
         timed step and the gradients of three of them, against the FP64
         oracle on the same FP32 delta.
  f64    the same workload in FP64 pair arithmetic over the FP32-stored delta
         (the precision the reference's double engine computes in), timed and
         checked against the oracle on the same states.
  c1, c3 the reference's own benchmark case (N=1000, FP64, through the host
         API) and the 64-instance batch, short runs with their own clocks.
  cpu_baseline  the oracle's port of the reference's per-evaluation work
         (likelihood pass + gradient pass, libm transcendentals) on all host
         cores over one whole evaluation, with the other CPU paths beside it
         (one core; the reference's FLOAT engine work order; SIMD/TBB notes).

--impl reference times that CPU port as the reference arm: one whole
evaluation per step.
Multi-GPU (torchrun): every rank runs the same workload on its own GPU
(independent replicas); value sums all ranks' evaluations over the slowest
rank's time.
"""
from __future__ import annotations

import argparse
import json
import os
import platform
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
PARITY_TOL = {"f32": 1e-5, "f64_sum": 1e-10, "f64_grad": 1e-9}


def workload(n: int, precision: str = "f32", evals: int = EVALS_PER_STEP) -> str:
    math = {"f32": "FP32 pairs + FP64 reductions", "f64": "FP64 pairs (DELTA_F32 mode)",
            "dd": "double-float pairs on the FP32 pipes (DOUBLE_FLOAT | DELTA_F32), FP64 bars"}[precision]
    return (f"fused loglik+grad sweep, N={n}, P=2, tau=2, truncation, delta FP32-stored ({n * n * 4 / 1e9:.2f} GB), "
            f"{math}, {evals} eval{'s' if evals != 1 else ''} per step at fresh locations")


DATA = ("synthetic: delta = ||Y_i - Y_j|| + N(0, 0.05^2) noise clipped at 0, Y ~ N(0, I_10) (seed 666); "
        "x ~ N(0,1) per evaluation")


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="mdsx", choices=["mdsx", "reference"])
    ap.add_argument("--n", type=int, default=N)
    ap.add_argument("--precision", default="f32", choices=["f32", "f64", "dd"],
                    help="pair arithmetic: f32 (the headline; FP32 pairs, FP64 reductions), f64 (FP64 pairs over "
                         "the same FP32-stored delta; bound by the FP64 pipe, 10 evaluations per step) or dd "
                         "(double-float pairs on the FP32 pipes at the FP64 bars, 50 evaluations per step)")
    ap.add_argument("--schedule", default="pairs", choices=["pairs", "rows"],
                    help="sweep schedule: each unordered pair once (default) or the row-block schedule")
    ap.add_argument("--workload", default="sweep", choices=["sweep", "c1", "c3"],
                    help="sweep: the headline N=20000 line (with f64, c1 and c3 sub-objects); c1: the reference's "
                         "benchmark case alone (N=1000, FP64, host API); c3: the 64-instance batch alone")
    ap.add_argument("--partition", default="replicas", choices=["replicas", "rows"],
                    help="multi-GPU: independent replicas of the workload (weak scaling, the default) or one "
                         "problem split by rows of delta across the ranks (strong scaling, NCCL all-reduce of "
                         "the sum and all-gather of the gradient rows every evaluation)")
    ap.add_argument("--cpu-seconds", type=float, default=3.0,
                    help="wall time of each bounded CPU row sample (one-core and FP32 paths)")
    ap.add_argument("--sections", default="parity,f64,noalloc,c1,c3",
                    help="comma list of the headline line's extra sections to run ('' for none)")
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


def host_info():
    """The CPU the baselines ran on."""
    model = None
    try:
        with open("/proc/cpuinfo") as f:
            for line in f:
                key = line.split(":", 1)[0].strip().lower()
                if key in ("model name", "cpu model", "hardware"):
                    model = line.split(":", 1)[1].strip()
                    break
    except OSError:
        pass
    if model is None:
        try:
            out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
            for line in out.splitlines():
                if line.lower().startswith("model name"):
                    model = line.split(":", 1)[1].strip()
                    break
        except (OSError, subprocess.SubprocessError):
            pass
    try:
        cc = subprocess.run(["gcc", "--version"], capture_output=True, text=True, timeout=10).stdout.splitlines()[0]
    except (OSError, subprocess.SubprocessError, IndexError):
        cc = None
    return {"uname_m": platform.machine(), "nproc": os.cpu_count(), "cpu_model": model, "compiler": cc}


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


def sampled(local, fn):
    """Runs fn() with nvidia-smi sampling around it; returns (fn's result, clocks)."""
    import torch

    sampler = ClockSampler(local)
    sampler.start()
    time.sleep(0.4)
    torch.cuda.synchronize()
    t0 = time.time()
    res = fn()
    torch.cuda.synchronize()
    t1 = time.time()
    sampler.stop()
    return res, sampler.summary(t0, t1)


# ---------------------------------------------------------------- CPU paths

AVX_NOTE = ("unavailable on this box ({}): the reference's SSE/AVX/AVX-512 engines need x86 and xsimd 7.1.3 "
            "(src/AbstractMultiDimensionalScaling.hpp:13-23)")
TBB_NOTE = ("the reference's TBB code path is timed as its work split over std::threads (no Intel TBB on this "
            "host)")


def cpu_port_full(delta, x, tau, threads):
    """One whole evaluation (every row: likelihood pass + gradient pass) of the
    oracle's FP64 port of the reference's serial per-evaluation work; seconds."""
    import oracle

    n = delta.shape[0]
    t = time.perf_counter()
    oracle.port_eval_rows(delta, x, tau, True, 0, n, threads=threads)
    return time.perf_counter() - t


def cpu_rows_rate(fn, n, target_seconds, min_rows):
    """evals/s of fn(rows) timed on a bounded row sample, scaled by N/rows; (rate, rows, seconds)."""
    rows = min(n, min_rows)
    t = time.perf_counter()
    fn(rows)
    dt = time.perf_counter() - t
    rows = int(min(n, max(rows, rows * target_seconds / max(dt, 1e-6))))
    t = time.perf_counter()
    fn(rows)
    dt = time.perf_counter() - t
    return (rows / n) / dt, rows, dt


def cpu_paths(delta, x, tau, threaded_f64_value=None, target_seconds=3.0):
    """The CPU paths beside the GPU number: the FP64 port on all threads (one
    whole evaluation), on one thread, and the reference FLOAT engine's work
    order on all threads (bounded row samples, scaled to evals/s)."""
    import numpy as np

    import oracle

    n = delta.shape[0]
    cores = os.cpu_count() or 1
    if threaded_f64_value is None:
        threaded_f64_value = 1.0 / cpu_port_full(delta, x, tau, cores)
    serial, s_rows, s_dt = cpu_rows_rate(lambda r: oracle.port_eval_rows(delta, x, tau, True, 0, r, threads=1),
                                         n, target_seconds, 16)
    d32 = delta if delta.dtype == np.float32 else delta.astype(np.float32)
    f32, f_rows, f_dt = cpu_rows_rate(lambda r: oracle.port_eval_rows_f32(d32, x, tau, True, 0, r, threads=cores),
                                      n, target_seconds, 4 * cores)
    return {
        "threaded_f64": {"value": threaded_f64_value, "unit": UNIT, "cores": cores,
                         "sample": "one whole evaluation (all rows)"},
        "serial_f64": {"value": serial, "unit": UNIT, "cores": 1,
                       "sample": f"rows 0..{s_rows - 1} ({s_dt:.2f} s), scaled by N/rows"},
        "threaded_f32": {"value": f32, "unit": UNIT, "cores": cores,
                         "sample": f"the reference FLOAT engine's work order, rows 0..{f_rows - 1} ({f_dt:.2f} s), "
                                   "scaled by N/rows"},
        "avx": AVX_NOTE.format(platform.machine()) if platform.machine() not in ("x86_64", "AMD64") else
        "unavailable: xsimd 7.1.3 is not installed",
        "tbb": TBB_NOTE,
        "host": host_info(),
    }


# ------------------------------------------------------------------ parity

def rel(a, b):
    return abs(a - b) / max(abs(b), 1e-300)


def grad_rel(g, ref):
    import numpy as np

    g = np.asarray(g).reshape(ref.shape)
    return float(np.abs(g - ref).max() / max(np.abs(ref).max(), 1e-300))


def oracle_states(delta, xs, tau):
    """(sum, gradient) of the FP64 oracle at each location set (all host threads)."""
    import oracle

    return [oracle.evaluate(delta, x, tau, True) for x in xs]


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


# --------------------------------------------------------------------- C1

def measure_c1(local, steps, warmup):
    """The reference's own benchmark case: N = 1000, P = 2, FP64, truncation,
    tau = 1, delta = distances of 1000 points iid N(0, I_10), x ~ N(0, 1); one
    iteration = updateLocations(-1, x) + getLogLikelihood() +
    getLogLikelihoodGradient() through the engine's host API (the call sequence
    src/benchmark.cpp:250-309 times on its CPU engines). Baseline: the same
    per-iteration work in the oracle's C port of the reference serial engine,
    on all host threads and on one."""
    import numpy as np

    import massivemds_gb300 as m
    from massivemds_gb300 import data as gen

    n, p, tau, iters = 1000, 2, 1.0, 100
    delta = gen.euclidean_delta(n, dim=10, seed=666)
    xs = np.random.default_rng(667).standard_normal((warmup + steps, iters, n, p))
    line = c1_run(local, m.flags.LEFT_TRUNCATION, delta, xs, n, p, tau, iters, steps, warmup)
    dd = c1_run(local, m.flags.LEFT_TRUNCATION | m.flags.DOUBLE_FLOAT, delta, xs, n, p, tau, iters, steps, warmup,
                baseline=False)
    line["double_float"] = {k: dd[k] for k in ("value", "unit", "ms_per_step", "parity", "clocks")}
    line["double_float"]["arithmetic"] = "double-float (f32 pairs) at the FP64 bars"
    return line


def c1_run(local, flags, delta, xs, n, p, tau, iters, steps, warmup, baseline=True):
    """C1 with the given engine flags (FP64 or double-float pair math); with
    `baseline`, also the oracle port's CPU timing."""
    import numpy as np

    import massivemds_gb300 as m

    e = m.Engine(p, n, flags, local)
    e.setPairwiseData(delta)
    e.setParameters([tau])
    grad = np.empty(n * p)
    lls = np.empty((warmup + steps, iters))

    def step(s):
        for k in range(iters):
            e.updateLocations(-1, xs[s, k])
            lls[s, k] = e.getLogLikelihood()
            e.getLogLikelihoodGradient(grad)

    for w in range(warmup):
        step(w)

    def timed():
        t = time.perf_counter()
        for s_ in range(steps):
            step(warmup + s_)
        return time.perf_counter() - t

    seconds, clocks = sampled(local, timed)
    e.close()
    sec_per_step = seconds / steps
    value = iters / sec_per_step

    import oracle  # the CPU baseline and the check of the last iteration

    x_last = xs[warmup + steps - 1, iters - 1]
    s_ref, g_ref = oracle.evaluate(delta, x_last, tau, True)
    ll_ref = oracle.log_likelihood(s_ref, n, tau)
    cores = os.cpu_count() or 1
    base = {}
    for label, threads in (("threaded_f64", cores), ("serial_f64", 1)) if baseline else ():
        t = time.perf_counter()
        sample_iters = 10
        for k in range(sample_iters):
            oracle.port_eval_rows(delta, xs[0, k], tau, True, 0, n, threads=threads)
        base[label] = {"value": sample_iters / (time.perf_counter() - t), "unit": "iterations/s", "cores": threads,
                       "sample": f"{sample_iters} iterations of the same workload"}
    return {
        "metric": "iterations/s (updateLocations + getLogLikelihood + getLogLikelihoodGradient)",
        "value": value, "unit": "iterations/s", "steps": steps, "warmup": warmup,
        "ms_per_step": 1000.0 * sec_per_step, "higher_is_better": True, "dtype": "f64",
        "data": "synthetic: delta = ||Y_i - Y_j||, Y ~ N(0, I_10) (seed 666); x ~ N(0,1) per iteration",
        "config": {"workload": "reference benchmark case: N=1000, P=2, FP64, truncation, tau=1, 100 iterations "
                               "per step through the host API", "n": n, "p": p, "tau": tau,
                   "iterations_per_step": iters, "l2": "delta 8 MB stays in L2 (timed as a user would see it)"},
        "e2e": {"value": value, "unit": "iterations/s", "h2d_bytes_per_step": iters * n * p * 8,
                "d2h_bytes_per_step": iters * (n * p * 8 + 8)},
        "parity": {"loglik_rel": rel(float(lls[warmup + steps - 1, iters - 1]), ll_ref),
                   "grad_rel": grad_rel(grad, g_ref), "iterations_checked": 1,
                   "tolerance": [PARITY_TOL["f64_sum"], PARITY_TOL["f64_grad"]]},
        "clocks": clocks,
        "cpu_baseline": dict(base["threaded_f64"], kind="port", paths=base) if baseline else None,
    }


# --------------------------------------------------------------------- C3

def measure_c3(local, steps, warmup, check=3):
    """The batched workload: 64 instances, N_k ~ U{500..8000}, P cycling 2, 3,
    6, tau_k ~ Gamma(2, 1), delta_k = distances of N_k points iid N(0, I_10),
    FP32 with FP64 reductions, one persistent launch per dimension group in one
    graph, shapes from the autotuner. Times the device-resident batch
    evaluation (CUDA events) and the host API; checks `check` instances of the
    last timed evaluation against the FP64 oracle."""
    import numpy as np
    import torch

    from massivemds_gb300 import data as gen, flags as F
    from massivemds_gb300.batch import Batch
    from massivemds_gb300.batch_bench import make_instances

    spec = make_instances(64, 3)
    t0 = time.time()
    batch = Batch(F.FLOAT | F.LEFT_TRUNCATION, local)
    locs, deltas = [], {}
    order = sorted(range(len(spec)), key=lambda k: spec[k][0])
    checked = sorted({order[0], order[len(order) // 2], order[-1]}) if check else []
    for k, (n, p, tau, s) in enumerate(spec):
        delta = gen.pairwise_distances(gen.latent_points(n, 10, s), dtype=np.float32)
        x = np.random.default_rng(s + 1).standard_normal((n, p))
        batch.add_instance(p, n)
        batch.setPairwiseData(k, delta)
        batch.updateLocations(k, -1, x)
        batch.setParameters(k, [tau])
        locs.append(x)
        if k in checked:
            deltas[k] = delta
        del delta
    setup_s = time.time() - t0
    candidates = batch.tune(repetitions=3)
    shapes = {p: batch.group_shape(p) for p in sorted({p for _, p, _, _ in spec})}
    dev = torch.device("cuda", local)
    total_grad = sum(n * p for n, p, _, _ in spec)
    d_sums = torch.empty(4 * len(spec), dtype=torch.float64, device=dev)
    d_grads = torch.empty(total_grad, dtype=torch.float64, device=dev)
    for _ in range(warmup):
        batch.evaluate_device(d_sums.data_ptr(), d_grads.data_ptr())
    torch.cuda.synchronize()
    cur = torch.cuda.current_stream(dev)

    def timed():
        start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        start.record(cur)
        for _ in range(steps):
            batch.evaluate_device(d_sums.data_ptr(), d_grads.data_ptr())
            torch.cuda.synchronize()
        end.record(cur)
        torch.cuda.synchronize()
        return start.elapsed_time(end) / 1e3 / steps

    t_batch, clocks = sampled(local, timed)
    sums = d_sums.cpu().numpy().reshape(len(spec), 4)
    grads = d_grads.cpu().numpy()

    for _ in range(2):
        batch.evaluate()
    t = time.perf_counter()
    for _ in range(steps):
        for k, x in enumerate(locs):
            batch.updateLocations(k, -1, x)
        batch.evaluate()
        for k in range(len(spec)):
            batch.getSumOfIncrements(k)
    t_e2e = (time.perf_counter() - t) / steps
    batch.close()

    import oracle  # the check of the last timed evaluation

    offs = np.cumsum([0] + [n * p for n, p, _, _ in spec])
    worst_s = worst_g = 0.0
    for k in checked:
        n, p, tau, _ = spec[k]
        s_ref, g_ref = oracle.evaluate(deltas[k], locs[k], tau, True)
        worst_s = max(worst_s, rel(float(sums[k, 2]), s_ref))
        worst_g = max(worst_g, grad_rel(grads[offs[k]:offs[k + 1]], g_ref))
    bytes_per_eval = sum(4.0 * n * n for n, _, _, _ in spec)
    hbm_peak, peak_kind = peaks()
    gbs = bytes_per_eval / t_batch / 1e9
    return {
        "metric": "instance-evals/s (64-instance batch, one fused sweep of every instance)",
        "value": len(spec) / t_batch, "unit": "instance-evals/s", "steps": steps, "warmup": warmup,
        "ms_per_batch_eval": 1000.0 * t_batch, "higher_is_better": True, "dtype": "f32",
        "config": {"workload": "64 instances, N ~ U{500..8000} (seed 3), P cycling 2, 3, 6, tau ~ Gamma(2, 1), "
                               "delta = ||Y_i - Y_j|| with Y ~ N(0, I_10), FP32 delta, truncation",
                   "sum_n2": int(sum(n * n for n, _, _, _ in spec)), "bytes_per_batch_eval": bytes_per_eval,
                   "shapes": {str(p): {"schedule": ("stream-K", "row-block queue", "unordered pairs")[sh[0]],
                                       "rows_per_warp": sh[1], "ctas_per_sm": sh[2], "grid": sh[3]}
                              for p, sh in shapes.items()},
                   "tuned_candidates": candidates, "setup_seconds": setup_s},
        "roofline": {"bound": "hbm", "achieved": gbs, "peak": hbm_peak, "unit": "GB/s", "frac": gbs / hbm_peak,
                     "peak_kind": peak_kind},
        "e2e": {"value": len(spec) / t_e2e, "unit": "instance-evals/s", "ms_per_batch_eval": 1000.0 * t_e2e,
                "h2d_bytes_per_step": sum(x.nbytes for x in locs), "d2h_bytes_per_step": 8 * (4 * len(spec) + total_grad)},
        "parity": {"sum_rel_max": worst_s, "grad_rel_max": worst_g, "instances_checked": len(checked),
                   "instance_sizes": [spec[k][0] for k in checked], "tolerance": PARITY_TOL["f32"]},
        "clocks": clocks,
    }


# --------------------------------------------------------------- headline

def measure_noalloc(local, delta, xs, refs, calls=20, warmup=3):
    """The allocation-free FP32 sweep (mdsx_sweep_f32_noalloc: static scratch,
    caller-owned device buffers, synchronous) against the engine's row-block
    FP32 sweep, the kernel it runs, on the same delta: GPU time per call from
    CUDA events on the call's stream (the call's own host synchronisation
    inside the window), and the results at the checked states against the
    oracle."""
    import numpy as np
    import torch

    import massivemds_gb300 as m
    from massivemds_gb300._lib import load

    lib = load()
    n = delta.shape[0]
    dev = torch.device("cuda", local)
    stream = torch.cuda.Stream(device=dev)
    ddelta = torch.from_numpy(delta).to(dev)  # row stride N (a multiple of 4 floats)
    pool = torch.from_numpy(np.ascontiguousarray(xs)).to(dev)
    out_sum = torch.zeros(1, dtype=torch.float64, device=dev)
    out_grad = torch.zeros(n * P, dtype=torch.float64, device=dev)

    def call(k):
        rc = lib.mdsx_sweep_f32_noalloc(ddelta.data_ptr(), n, pool[k % len(xs)].data_ptr(), n, P, TAU, 1,
                                        out_sum.data_ptr(), out_grad.data_ptr(), stream.cuda_stream)
        if rc != 0:
            raise RuntimeError(lib.mdsx_last_error(None).decode())

    def events_ms(fn):
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(calls)]
        for k in range(calls):
            ev[k][0].record(stream)
            fn(k)
            ev[k][1].record(stream)
        torch.cuda.synchronize()
        return statistics.mean(a.elapsed_time(b) for a, b in ev)

    for k in range(warmup):
        call(k)
    noalloc_ms = events_ms(call)
    worst_s = worst_g = 0.0
    for k, (s_ref, g_ref) in enumerate(refs):
        call(k)
        torch.cuda.synchronize()
        worst_s = max(worst_s, rel(float(out_sum.item()), s_ref))
        worst_g = max(worst_g, grad_rel(out_grad.cpu().numpy(), g_ref))
    eng = m.Engine(P, n, m.flags.FLOAT | m.flags.LEFT_TRUNCATION, local)
    eng.set_sweep_schedule(m.flags.SWEEP_ROWS)
    eng.setPairwiseData(delta)
    eng.setParameters([TAU])
    eng.set_stream(stream.cuda_stream)

    def engine_call(k):
        eng.update_locations_device(pool[k % len(xs)].data_ptr())
        eng.evaluate_device(out_sum.data_ptr(), out_grad.data_ptr())

    for k in range(warmup):
        engine_call(k)
    torch.cuda.synchronize()
    engine_ms = events_ms(engine_call)
    eng.set_stream(None)
    eng.close()
    del ddelta
    return {"ms_per_call": noalloc_ms, "engine_rows_ms": engine_ms, "ratio": noalloc_ms / engine_ms,
            "what": "one synchronous mdsx_sweep_f32_noalloc call (location conversion, padding-row marks, "
                    "row-block sweep, results to the caller's buffers) against the engine's location update + "
                    "row-block evaluation with its results copied out, CUDA events, N=20000 FP32",
            "parity": {"sum_rel_max": worst_s, "grad_rel_max": worst_g, "calls_checked": len(refs),
                       "tolerance": PARITY_TOL["f32"]}}


def measure_f64(local, delta, xs, refs, steps=10, warmup=3, double_float=False):
    """FP64-accurate pair arithmetic over the FP32-stored delta (DELTA_F32):
    evals/s and the sweep's kernel time; the results at the checked states
    against the oracle at the FP64 bars. double_float: the double-float pair
    math on the FP32 pipes (MDSX_FLAG_DOUBLE_FLOAT) instead of FP64."""
    import torch

    import massivemds_gb300 as m

    n = delta.shape[0]
    flags = m.flags.DELTA_F32 | m.flags.LEFT_TRUNCATION | (m.flags.DOUBLE_FLOAT if double_float else 0)
    eng = m.Engine(P, n, flags, local)
    eng.setPairwiseData(delta)
    eng.setParameters([TAU])
    stream = torch.cuda.Stream()
    eng.set_stream(stream.cuda_stream)
    dev = f"cuda:{local}"
    pool = torch.from_numpy(xs).to(dev)
    d_sum = torch.zeros(1, dtype=torch.float64, device=dev)
    for k in range(warmup):
        eng.update_locations_device(pool[k % len(xs)].data_ptr())
        eng.evaluate_device(d_sum.data_ptr(), None)
    torch.cuda.synchronize()

    def timed():
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
        start, stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        start.record(stream)
        for k in range(steps):
            eng.update_locations_device(pool[k % len(xs)].data_ptr())
            ev[k][0].record(stream)
            eng.evaluate_device(d_sum.data_ptr(), None)
            ev[k][1].record(stream)
        stop.record(stream)
        torch.cuda.synchronize()
        return start.elapsed_time(stop), statistics.mean(a.elapsed_time(b) for a, b in ev)

    (elapsed_ms, kernel_ms), clocks = sampled(local, timed)
    eng.set_stream(None)
    worst_s = worst_g = 0.0
    for x, (s_ref, g_ref) in zip(xs, refs):
        eng.updateLocations(-1, x)
        worst_s = max(worst_s, rel(eng.getSumOfIncrements(), s_ref))
        worst_g = max(worst_g, grad_rel(eng.getLogLikelihoodGradient(), g_ref))
    eng.close()
    hbm_peak, _ = peaks()
    gbs = (float(n) * n * 4 + 2.0 * n * P * 8) / (kernel_ms / 1e3) / 1e9
    kernel = ("pair_kernel<2,true,PairMathDD<float>> + pair_finish_kernel<2,double>" if double_float
              else "pair_kernel<2,true,PairMathF64<float>> + pair_finish_kernel<2,double>")
    return {"value": steps / (elapsed_ms / 1e3), "unit": UNIT, "steps": steps, "kernel_ms": kernel_ms,
            "kernel": kernel, "arithmetic": "double-float (f32 pairs)" if double_float else "f64",
            "hbm_gbs": gbs, "hbm_frac": gbs / hbm_peak, "bound": "FP32 pipes" if double_float else "FP64 pipe",
            "parity": {"sum_rel_max": worst_s, "grad_rel_max": worst_g, "evals_checked": len(xs),
                       "tolerance": [PARITY_TOL["f64_sum"], PARITY_TOL["f64_grad"]]},
            "clocks": clocks}


def run_reference(args):
    """The reference arm: the oracle's FP64 port of the reference serial
    engine's per-evaluation work (a likelihood pass and a gradient pass over
    every row) on all host threads; one step = one whole evaluation."""
    rank, world, _ = dist_env()
    if rank != 0:
        return
    import numpy as np

    delta = make_delta(args.n)
    rng = np.random.default_rng(667)
    cores = os.cpu_count() or 1
    for _ in range(args.warmup):
        cpu_port_full(delta, rng.standard_normal((args.n, P)), TAU, cores)
    secs = [cpu_port_full(delta, rng.standard_normal((args.n, P)), TAU, cores) for _ in range(args.steps)]
    value = len(secs) / sum(secs)
    paths = cpu_paths(delta, rng.standard_normal((args.n, P)), TAU, threaded_f64_value=value,
                      target_seconds=args.cpu_seconds)
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 * statistics.mean(secs),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": DATA,
        "config": {"workload": workload(args.n, evals=1).replace("FP32 pairs + FP64 reductions",
                                                                 "reference CPU port in FP64"),
                   "n": args.n, "p": P, "tau": TAU, "evals_per_step": 1},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": f"{args.steps} whole evaluations (every row), one per step, at fresh locations",
                         "paths": paths},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": ("the reference engine compiled from its sources is not available on this host (its sources are "
                 "not here); the oracle's port of the reference serial engine's per-evaluation work is timed"),
    }
    print(json.dumps(line), flush=True)


def run_partitioned(args):
    """One N x N problem split by rows across the ranks (massivemds_gb300.partition):
    rank r sweeps rows [r0, r1) of delta with an engine over those rows only
    (row-block schedule, FP32, truncation); every rank holds the same
    locations; per evaluation the ranks all-reduce the sum of increments and
    all-gather the gradient rows (NCCL). value = whole-problem evals/s."""
    import numpy as np
    import torch
    import torch.distributed as dist

    import massivemds_gb300 as m
    from massivemds_gb300.partition import row_ranges

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    dev = torch.device("cuda", local)
    n, evals = args.n, EVALS_PER_STEP
    ranges = row_ranges(n, world)
    r0, r1 = ranges[rank]
    width = max(b - a for a, b in ranges) * P
    delta = make_delta(n)
    eng = m.Engine(P, n, m.flags.FLOAT | m.flags.LEFT_TRUNCATION, local, rows=(r0, r1))
    eng.setPairwiseData(delta[r0:r1])
    eng.setParameters([TAU])
    stream = torch.cuda.Stream(device=dev)
    eng.set_stream(stream.cuda_stream)
    pool = torch.from_numpy(np.random.default_rng(1000).standard_normal((evals, n, P))).to(dev)  # same on all ranks
    d_sums = torch.zeros(evals, dtype=torch.float64, device=dev)
    d_rows = torch.zeros(width, dtype=torch.float64, device=dev)
    d_grad = torch.zeros(world * width, dtype=torch.float64, device=dev)

    def step():
        with torch.cuda.stream(stream):
            for k in range(evals):
                eng.update_locations_device(pool[k].data_ptr())
                eng.evaluate_device(d_sums[k:k + 1].data_ptr(), d_rows.data_ptr())
                dist.all_reduce(d_sums[k:k + 1])
                dist.all_gather_into_tensor(d_grad, d_rows)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    sampler = ClockSampler(local)
    sampler.start()
    time.sleep(0.5)
    dist.barrier()
    torch.cuda.synchronize()
    t0 = time.time()
    start, stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    start.record(stream)
    for _ in range(args.steps):
        step()
    stop.record(stream)
    torch.cuda.synchronize()
    t1 = time.time()
    dist.barrier()
    sampler.stop()
    elapsed_ms = across_ranks_max(start.elapsed_time(stop), world, dev)
    launches = eng.last_launch_count()
    sums = d_sums.cpu().numpy()
    grad = np.concatenate([d_grad[r * width:r * width + (b - a) * P].cpu().numpy() for r, (a, b) in enumerate(ranges)])
    eng.close()
    if rank == 0:
        s_ref, g_ref = oracle_states(delta, pool[evals - 1:].cpu().numpy(), TAU)[0]
        line = {
            "metric": METRIC, "value": args.steps * evals / (elapsed_ms / 1e3), "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": elapsed_ms / args.steps,
            "higher_is_better": True, "scaling": "strong", "vs_baseline": None, "dtype": "f32", "data": DATA,
            "config": {"workload": workload(n), "n": n, "p": P, "tau": TAU, "evals_per_step": evals,
                       "parallelism": f"rows x{world} (delta rows split; NCCL all-reduce of the sum and all-gather "
                                      "of the gradient per evaluation)",
                       "rows_per_rank": [b - a for a, b in ranges], "delta_bytes_per_rank": (r1 - r0) * n * 4},
            "parity": {"sum_rel": rel(float(sums[-1]), s_ref), "grad_rel": grad_rel(grad, g_ref),
                       "evals_checked": 1, "tolerance": PARITY_TOL["f32"]},
            "gpu_launches": args.steps * evals * (launches + 1),  # sweep kernels + the location conversion
            "clocks": sampler.summary(t0, t1),
        }
        print(json.dumps(line), flush=True)
    dist.destroy_process_group()


def run_mdsx(args):
    import numpy as np
    import torch

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    import massivemds_gb300 as m

    sections = {s for s in args.sections.split(",") if s}
    n = args.n
    f64 = args.precision in ("f64", "dd")  # FP64-accurate results, held to the FP64 bars
    evals = {"f64": 10, "dd": 50}.get(args.precision, EVALS_PER_STEP)
    delta = make_delta(n)
    flags = {"f32": m.flags.FLOAT, "f64": m.flags.DELTA_F32,
             "dd": m.flags.DELTA_F32 | m.flags.DOUBLE_FLOAT}[args.precision]
    eng = m.Engine(P, n, flags | m.flags.LEFT_TRUNCATION, local)
    eng.set_sweep_schedule(m.flags.SWEEP_PAIRS if args.schedule == "pairs" else m.flags.SWEEP_ROWS)
    eng.setPairwiseData(delta)
    eng.setParameters([TAU])
    stream = torch.cuda.Stream()
    eng.set_stream(stream.cuda_stream)

    # location pool: one set per evaluation of a step
    rng = np.random.default_rng(1000 + rank)
    pool_host = torch.from_numpy(rng.standard_normal((evals, n, P))).pin_memory()
    pool_dev = pool_host.to(f"cuda:{local}")
    d_sums = torch.zeros(evals, dtype=torch.float64, device=f"cuda:{local}")
    check_idx = [0, evals // 2, evals - 1]
    d_grads = torch.zeros((len(check_idx), n * P), dtype=torch.float64, device=f"cuda:{local}")

    def device_step(events=None, keep=False):
        for k in range(evals):
            eng.update_locations_device(pool_dev[k].data_ptr())
            if events is not None:
                events[k][0].record(stream)
            g = d_grads[check_idx.index(k)].data_ptr() if keep and k in check_idx else None
            eng.evaluate_device(d_sums[k:k + 1].data_ptr(), g)
            if events is not None:
                events[k][1].record(stream)

    torch.cuda.synchronize()
    for _ in range(args.warmup):
        device_step()
    torch.cuda.synchronize()
    d_sums.fill_(float("nan"))
    d_grads.fill_(float("nan"))
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
        device_step(kev[s], keep=(s == args.steps - 1))
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
    timed_sums = d_sums.cpu().numpy()
    timed_grads = d_grads.cpu().numpy()

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
    eng.close()

    hbm_peak, peak_kind = peaks()
    bytes_per_launch = float(n) * n * 4 + 2.0 * n * P * 4
    achieved = bytes_per_launch / (kernel_ms / 1000.0) / 1e9
    traffic = profiled_traffic(args.schedule) if n == N else None  # the committed captures are of N = 20000
    if args.precision == "dd":
        kernel_name = "pair_kernel<2,true,PairMathDD<float>> + pair_finish_kernel<2,double>"
        traffic = None  # FP32-pipe bound: the HBM fraction below is small by construction
    elif f64:
        kernel_name = ("pair_kernel<2,true,PairMathF64<float>> + pair_finish_kernel<2,double>"
                       if args.schedule == "pairs" else "sweep_kernel<double,float,2,true>")
        traffic = None  # FP64-pipe bound: the HBM fraction below is small by construction
    else:
        kernel_name = ("pair_kernel<2,true,PairMathF32> + pair_finish_kernel<2,float>" if args.schedule == "pairs"
                       else "sweep_kernel<float,float,2,true>")

    line = None
    if rank == 0:
        cpu_s = cpu_port_full(delta, pool_np[0], TAU, os.cpu_count() or 1)
        paths = cpu_paths(delta, pool_np[0], TAU, threaded_f64_value=1.0 / cpu_s, target_seconds=args.cpu_seconds)
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": elapsed_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": args.precision, "data": DATA,
            "config": {"workload": workload(n, args.precision, evals), "n": n, "p": P, "tau": TAU,
                       "evals_per_step": evals, "schedule": args.schedule, "precision": args.precision,
                       "delta_bytes": n * n * 4,
                       "l2": f"inputs larger than L2 ({n * n * 4 / 1e9:.2f} GB delta vs 129 MB L2), no flush",
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
            "cpu_baseline": {"value": 1.0 / cpu_s, "unit": UNIT, "cores": os.cpu_count() or 1, "kind": "port",
                             "sample": f"one whole evaluation (all {n} rows: likelihood pass + gradient pass), "
                                       f"{cpu_s:.2f} s", "paths": paths},
        }
        if "parity" in sections or "f64" in sections or "noalloc" in sections:
            xs = pool_np[check_idx]
            refs = oracle_states(delta, xs, TAU)
            if "parity" in sections:
                tol_s = PARITY_TOL["f64_sum"] if f64 else PARITY_TOL["f32"]
                tol_g = PARITY_TOL["f64_grad"] if f64 else PARITY_TOL["f32"]
                line["parity"] = {
                    "sum_rel_max": max(rel(float(timed_sums[k]), refs[m_][0]) for m_, k in enumerate(check_idx)),
                    "grad_rel_max": max(grad_rel(timed_grads[m_], refs[m_][1]) for m_ in range(len(check_idx))),
                    "evals_checked": len(check_idx), "of": "evaluations 0, 100 and 199 of the last timed step",
                    "sums_finite": int(np.isfinite(timed_sums).sum()), "tolerance": [tol_s, tol_g]}
            if "f64" in sections and not f64:
                line["f64"] = measure_f64(local, delta, xs, refs)
                # the same FP64 bars from the FP32 pipes
                line["f64"]["double_float"] = measure_f64(local, delta, xs, refs, double_float=True)
            if "noalloc" in sections and not f64 and n <= 32768:
                line["noalloc"] = measure_noalloc(local, delta, xs, refs)
        del delta
        if "c1" in sections:
            line["c1"] = measure_c1(local, steps=5, warmup=3)
        if "c3" in sections:
            line["c3"] = measure_c3(local, steps=10, warmup=3)
    if world > 1:
        torch.distributed.destroy_process_group()
    if line is not None:
        print(json.dumps(line), flush=True)


def main():
    args = parse()
    if args.workload in ("c1", "c3"):
        rank, _, local = dist_env()
        if args.impl == "reference":
            print(json.dumps({"impl": "reference",
                              "unavailable": f"the {args.workload} workload's CPU time is its cpu_baseline"}))
        elif rank == 0:
            import torch

            torch.cuda.set_device(local)
            fn = measure_c1 if args.workload == "c1" else measure_c3
            line = fn(local, steps=args.steps, warmup=args.warmup)
            line.update({"n_gpus": 1, "scaling": "weak", "vs_baseline": None})
            print(json.dumps(line), flush=True)
    elif args.impl == "reference":
        run_reference(args)
    elif args.partition == "rows":
        run_partitioned(args)
    else:
        run_mdsx(args)


if __name__ == "__main__":
    main()
