"""Benchmark: LL + gradient evaluations per second of the dense Gaussian-process likelihood at n=16384, d=8.

Workload (the single-GPU configuration of the headline metric): n = 16384 points X ~ U[0,1]^8,
y = sum_j sin(2 pi x_j) + 0.1 N(0,1), matern5_2 kernel, NuggetKriging with alpha = 1 / (1 + 1e-6)
(nugget = 1e-6 sigma2), theta ~ U[0.2, 1.5]^8, all drawn from numpy's PCG64 with seed 123.  One step = one
logLikelihoodFun(gamma = [theta, alpha], return_grad = true) -- covariance build, blocked FP64 Cholesky, solves,
GLS, R^-1 and the adjoint gradient -- on the FP64 path.

  value  device throughput: evaluations / s from the CUDA-event stage timings of each step (design resident)
  e2e    wall clock through the C ABI (lkg_kriging_log_likelihood_fun): gamma copied host -> device and
         (LL, gradient) device -> host every step
Usage: python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference] [--n 16384]
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "LL+grad evals/s at n=16k d=8 (mixed vs FP64 GPU, rel err); batched fits/s"
UNIT = "evals/s"


def make_inputs(n, d=8, seed=123):
    rng = np.random.default_rng(seed)
    X = rng.uniform(size=(n, d))
    y = np.sin(2 * np.pi * X).sum(axis=1) + 0.1 * rng.standard_normal(n)
    theta = rng.uniform(0.2, 1.5, size=d)
    alpha = 1.0 / (1.0 + 1e-6)
    return X, y, theta, alpha


class ClockSampler:
    """nvidia-smi samples of SM clocks and throttle reasons during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "200"], stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (OSError, FileNotFoundError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                smax = float(parts[1])
            except ValueError:
                continue
            for nm, v in zip(names, parts[4:8]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


def kernel_stats(lib):
    need = lib.lkg_stats_report(None, 0)
    buf = ctypes.create_string_buffer(max(need, 1))
    lib.lkg_stats_report(buf, need)
    out = {}
    for line in buf.value.decode().splitlines():
        name, launches, timed, ms, flops, byts = line.split("\t")
        out[name] = dict(launches=int(launches), timed=int(timed), ms=float(ms), flops=float(flops),
                         bytes=float(byts))
    return out


def measured_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        try:
            return json.loads(p.read_text())
        except ValueError:
            pass
    return {}


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def cpu_baseline(X, y, theta, alpha, reps=1):
    from oracle import baseline as B
    from oracle import oracle as O
    O.build()
    vals = []
    det = None
    t0 = time.time()
    for _ in range(reps):
        s, det = B.dense_eval_sample(X, y, theta, alpha, "matern5_2")
        vals.append(1.0 / s)
    wall = time.time() - t0
    sample = ("reference-restated path at full n=%d: serial pair loops on the last %.1f%% of the pairs, dpotrf+dtrcon "
              "in full, inv_sympd dtrsm on %.2f%% of the identity columns, scaled by exact work ratios; %.1f s wall"
              % (det["n"], 100 * det["pair_fraction"], 100 * det["rhs_fraction"], wall))
    return dict(value=float(np.mean(vals)), unit=UNIT, cores=int(det["blas_threads"]), kind="port", sample=sample,
                stages_s={k: round(v, 4) for k, v in det["stages_s"].items()})


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    X, y, theta, alpha = make_inputs(args.n)
    from oracle import baseline as B
    from oracle import oracle as O
    O.build()
    for _ in range(args.warmup):
        B.dense_eval_sample(X, y, theta, alpha, "matern5_2", pair_fraction=0.03, rhs_fraction=1.0 / 64)
    times = []
    det = None
    t0 = time.time()
    for _ in range(args.steps):
        s, det = B.dense_eval_sample(X, y, theta, alpha, "matern5_2", pair_fraction=0.03, rhs_fraction=1.0 / 64)
        times.append(s)
    wall = time.time() - t0
    value = args.steps / float(np.sum(times))
    sample = ("each step: reference-restated LL+grad at full n=%d timed on bounded samples (serial pair loops on "
              "%.1f%% of the pairs, dpotrf+dtrcon in full, inv_sympd on %.2f%% of the identity columns), scaled by "
              "exact work ratios; %.1f s wall for %d steps" % (args.n, 100 * det["pair_fraction"],
                                                               100 * det["rhs_fraction"], wall, args.steps))
    line = dict(metric=METRIC, value=value, unit=UNIT, n_gpus=world, steps=args.steps, warmup=args.warmup,
                ms_per_step=1000.0 * float(np.mean(times)), higher_is_better=True, scaling="weak", vs_baseline=None,
                dtype="f64", data="synthetic",
                config=dict(workload="dense LL+grad, n=%d, d=8, matern5_2, nugget 1e-6" % args.n,
                            l2="inputs larger than L2"),
                impl="reference",
                cpu_baseline=dict(value=value, unit=UNIT, cores=int(det["blas_threads"]), kind="port",
                                  sample=sample),
                e2e=dict(value=value, unit=UNIT, h2d_bytes_per_step=0, d2h_bytes_per_step=0))
    print(json.dumps(line), flush=True)


def run_gpu(args):
    rank, world, local = dist_env()
    import torch
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    import libkriging_gb300 as lk
    lib = lk.load()
    peak_fp64 = ctypes.c_double()
    if lib.lkg_probe_fp64_peak(ctypes.byref(peak_fp64)) != 0:
        raise RuntimeError("FP64 peak probe failed: " + lk._lib.last_error())
    X, y, theta, alpha = make_inputs(args.n)
    gamma = np.concatenate([theta, [alpha]])
    k = lk.Kriging("matern5_2", "nugget")
    k.fit(y, X, "constant", False, "none", "LL", {"theta": theta.reshape(1, -1), "sigma2": 1.0, "nugget": 1e-6})

    def barrier():
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    for _ in range(args.warmup):
        k.logLikelihoodFun(gamma, True, False, bench=True)
    # device-resident throughput (CUDA events on the library stream, per stage, summed per step)
    barrier()
    lib.lkg_stats_reset()
    lib.lkg_stats_enable(1)
    clocks = ClockSampler(local)
    clocks.start()
    dev_ms = []
    t0 = time.perf_counter()
    for _ in range(args.steps):
        ll, g, _ = k.logLikelihoodFun(gamma, True, False, bench=True)
        dev_ms.append(sum(k.last_bench.values()))
    barrier()
    wall_value = time.perf_counter() - t0
    clk = clocks.stop()
    lib.lkg_stats_enable(0)
    stats = kernel_stats(lib)
    launches = sum(v["launches"] for v in stats.values())
    # end to end through the C ABI: gamma from pinned host memory in, (LL, grad) out, wall clock
    gam_h = torch.tensor(gamma, dtype=torch.float64).pin_memory().numpy()
    grad_h = torch.zeros(gamma.size, dtype=torch.float64).pin_memory().numpy()
    llv = ctypes.c_double()
    barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        lk._lib.check(lib.lkg_kriging_log_likelihood_fun(k._h, lk._lib.ptr(gam_h), gam_h.size, 1, 0,
                                                          ctypes.byref(llv), lk._lib.ptr(grad_h), None))
    barrier()
    e2e_wall = time.perf_counter() - t0
    max_dev = float(np.mean(dev_ms))
    e2e_s = e2e_wall / args.steps
    if world > 1:
        t = torch.tensor([max_dev, e2e_s], dtype=torch.float64, device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        max_dev, e2e_s = float(t[0]), float(t[1])
    value = world * 1000.0 / max_dev
    e2e = world / e2e_s
    # roofline of the dominant kernel (largest total CUDA-event time in the timed region)
    dom = max(stats.items(), key=lambda kv: kv[1]["ms"])
    name, s = dom
    achieved = s["flops"] / (s["ms"] * 1e-3) / 1e12
    traffic = None
    tf = ROOT / "profiles" / "dram_traffic.json"
    if tf.exists():
        try:
            ratio = json.loads(tf.read_text()).get(name, {}).get("ratio")
            if ratio is not None and s["launches"] > 0:
                traffic = ratio * s["bytes"] / s["launches"]  # DRAM bytes per launch, scaled from the ncu capture
        except ValueError:
            traffic = None
    roofline = dict(bound="fp64", kernel=name, achieved=achieved, peak=peak_fp64.value, unit="TFLOP/s",
                    frac=achieved / peak_fp64.value, traffic=traffic,
                    peak_source="lkg_probe_fp64_peak measured on this GPU (DFMA pipe; MEASURED_PEAKS.json has no "
                                "FP64 entry); per-launch algorithmic flops / mean CUDA-event launch time",
                    launches=s["launches"], share=s["ms"] / sum(v["ms"] for v in stats.values()))
    line = dict(metric=METRIC, value=value, unit=UNIT, n_gpus=world, steps=args.steps, warmup=args.warmup,
                ms_per_step=max_dev, higher_is_better=True, scaling="weak", vs_baseline=None, dtype="f64",
                data="synthetic (seeded PCG64, seed 123)",
                config=dict(workload="dense LL+grad, n=%d, d=8, matern5_2, nugget 1e-6, FP64 path" % args.n,
                            parallelism="replicas" if world > 1 else "single GPU",
                            l2="inputs larger than L2 (R, L^-1, R^-1: 3 x %.2f GB)" % (8.0 * args.n * args.n / 1e9)),
                e2e=dict(value=e2e, unit=UNIT, h2d_bytes_per_step=8 * gamma.size,
                         d2h_bytes_per_step=8 * (1 + gamma.size)),
                gpu_launches=int(launches), roofline=roofline, clocks=clk, ll=float(ll),
                wall_s_timed_region=wall_value,
                measured_peaks={k2: v for k2, v in measured_peaks().items() if k2 in ("hbm_gbs", "bf16_tflops")},
                stage_ms={kk: round(v, 3) for kk, v in k.last_bench.items()},
                kernels={kk: dict(launches=v["launches"], ms=round(v["ms"], 3),
                                  tflops=(v["flops"] / (v["ms"] * 1e-3) / 1e12) if v["ms"] > 0 else None)
                         for kk, v in sorted(stats.items(), key=lambda kv: -kv[1]["ms"])})
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(X, y, theta, alpha)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--n", type=int, default=16384)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
