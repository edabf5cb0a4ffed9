"""Benchmark: LL + gradient evaluations per second of the dense Gaussian-process likelihood at n=16384, d=8, and
batched multistart fits per second at n=2048, d=6.

Workload (the single-GPU configuration of the headline metric): n = 16384 points X ~ U[0,1]^8,
y = sum_j sin(2 pi x_j) + 0.1 N(0,1), matern5_2 kernel, NuggetKriging with alpha = 1 / (1 + 1e-6)
(nugget = 1e-6 sigma2), theta ~ U[0.2, 1.5]^8, all drawn from numpy's PCG64 with seed 123.  One step = one
logLikelihoodFun(gamma = [theta, alpha], return_grad = true) -- covariance build, blocked Cholesky, solves, GLS,
R^-1 and the adjoint gradient.  The headline line is the mixed-precision path (O(n^3) products as error-free bf16
digit products on the tensor cores, 8 digits for the Cholesky, 5 for the inverse); the same line carries the FP64
path's figures ("fp64"), the speed-up, the relative LL / gradient difference between the two, and both paths' errors
against the oracle's full-size evaluation ("rel_err_vs_oracle").

  value         device throughput: evaluations / s from the CUDA-event stage timings of each step (design resident)
  e2e           wall clock through the C ABI (lkg_kriging_log_likelihood_fun): gamma copied host -> device and
                (LL, gradient) device -> host every step
  cpu_baseline  one full, unsampled reference-restated evaluation on the host cores (oracle/baseline.py)
  batched       the second half of the metric: BFGS64 fits of an n=2048, d=6 gauss design with sigma2 and nugget
                fixed, every optimiser round one batched GPU evaluation of the 64 starts (its own value, e2e,
                roofline and CPU baseline, all FP64); "batched.mixed" is the same fit on the mixed path with its
                speed-up and its distance from the FP64 fit
Other workloads (--workload): "multistart" (the batched record alone), "vecchia" (Vecchia LL + gradient at n = 2^20,
m = 30) and "nested" (NestedKriging, 10^6 points; --nested-nk adds NK aggregation on one 128-point chunk, --mixed
the mixed path with its difference from FP64).  --impl reference times the reference-restated CPU path alone.
Usage: python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference] [--n 16384] [--workload W]
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


def _digits_note(lib, slices):
    """Operand precision of the mixed path for `slices`: 7-bit digits, slices + 1 (6..8) for the Cholesky and
    max(5, slices - 2) for the inverse and W^T W."""
    inv = max(4, slices - 2)
    return "Cholesky %d 7-bit digits, inverse %d" % (min(8, max(6, slices + 1)), min(8, max(5, inv)))


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


def cpu_baseline(X, y, theta, alpha):
    """One full, unsampled reference-restated LL + gradient evaluation of the headline workload on the host cores.
    Returns (cpu_baseline record, oracle LL, oracle gradient): the same evaluation is the oracle's value at full
    size that the GPU paths' errors are stated against."""
    from oracle import baseline as B
    ll, g, secs, det = B.eval_full(X, y, theta, "matern5_2", alpha=alpha)
    sample = ("one full, unsampled reference-restated LL+grad evaluation at n=%d (pair loops over %d threads, "
              "OpenBLAS dpotrf/dtrcon/dtrtrs on %s threads, R^-1 as the reference codes it: two triangular solves "
              "against I): %.1f s" % (det["n"], det["threads"], det["blas_threads"], secs))
    rec = dict(value=1.0 / secs, unit=UNIT, cores=int(det["threads"]), kind="port", sample=sample,
               stages_s=det["stages_s"])
    return rec, ll, np.asarray(g)


def run_reference(args):
    """The reference arm: the reference-restated CPU path (oracle/baseline.py), full evaluations of the headline
    workload on every host core.  A full evaluation takes tens of seconds, so the arm runs at most one warm-up
    evaluation and stops timing once the next evaluation would pass --ref-budget-s; the line states both."""
    rank, world, _ = dist_env()
    if rank != 0:
        return
    X, y, theta, alpha = make_inputs(args.n)
    from oracle import baseline as B
    from oracle import oracle as O
    O.build()
    warm = min(args.warmup, 1)
    for _ in range(warm):
        B.eval_full(X, y, theta, "matern5_2", alpha=alpha)
    times = []
    det = None
    t0 = time.time()
    while len(times) < args.steps:
        _, _, s, det = B.eval_full(X, y, theta, "matern5_2", alpha=alpha)
        times.append(s)
        if time.time() - t0 + s > args.ref_budget_s:
            break
    wall = time.time() - t0
    value = len(times) / float(np.sum(times))
    sample = ("each step: one full, unsampled reference-restated LL+grad evaluation at n=%d (pair loops over %d "
              "threads, OpenBLAS on %s threads); %d of the %d requested steps timed (%.0f s budget), %d of the %d "
              "requested warm-up evaluations run; %.1f s wall" % (args.n, det["threads"], det["blas_threads"],
                                                                  len(times), args.steps, args.ref_budget_s, warm,
                                                                  args.warmup, wall))
    line = dict(metric=METRIC, value=value, unit=UNIT, n_gpus=world, steps=len(times), warmup=warm,
                steps_requested=args.steps, warmup_requested=args.warmup,
                ms_per_step=1000.0 * float(np.mean(times)), higher_is_better=True, scaling="weak", vs_baseline=None,
                dtype="f64", data="synthetic (seeded PCG64, seed 123)",
                config=dict(workload="dense LL+grad, n=%d, d=8, matern5_2, nugget 1e-6" % args.n,
                            l2="host memory (no GPU)"),
                impl="reference",
                cpu_baseline=dict(value=value, unit=UNIT, cores=int(det["threads"]), kind="port", sample=sample,
                                  stages_s=det["stages_s"]),
                e2e=dict(value=value, unit=UNIT, h2d_bytes_per_step=0, d2h_bytes_per_step=0))
    print(json.dumps(line), flush=True)


def _timed_steps(k, lib, gamma, steps, local, label, stats_steps=None):
    """K LL+grad steps; returns (mean device ms per step from the CUDA-event stage timings, last (ll, grad),
    per-kernel stats, clock record).  Each step is an NVTX range named `label` (a profiler can select one path's
    launches with it).  The timed steps run without per-launch events (which cost host time on every launch and
    would hold back the short launches of the solves); `stats_steps` (default K) further steps with per-launch
    events give the per-kernel statistics."""
    import torch
    lib.lkg_stats_enable(0)
    clocks = ClockSampler(local)
    clocks.start()
    dev_ms = []
    ll = g = None
    for _ in range(steps):
        torch.cuda.nvtx.range_push(label)
        ll, g, _ = k.logLikelihoodFun(gamma, True, False, bench=True)
        torch.cuda.nvtx.range_pop()
        dev_ms.append(sum(k.last_bench.values()))
    clk = clocks.stop()
    stage = dict(k.last_bench)
    lib.lkg_stats_reset()
    lib.lkg_stats_enable(1)
    for _ in range(steps if stats_steps is None else stats_steps):
        k.logLikelihoodFun(gamma, True, False, bench=True)
    lib.lkg_stats_enable(0)
    return float(np.mean(dev_ms)), (ll, np.asarray(g)), kernel_stats(lib), clk, stage


def _e2e(lk, lib, k, gamma, steps, barrier):
    import torch
    gam_h = torch.tensor(gamma, dtype=torch.float64).pin_memory().numpy()
    grad_h = torch.zeros(gamma.size, dtype=torch.float64).pin_memory().numpy()
    llv = ctypes.c_double()
    barrier()
    t0 = time.perf_counter()
    for _ in range(steps):
        lk._lib.check(lib.lkg_kriging_log_likelihood_fun(k._h, lk._lib.ptr(gam_h), gam_h.size, 1, 0,
                                                          ctypes.byref(llv), lk._lib.ptr(grad_h), None))
    barrier()
    return (time.perf_counter() - t0) / steps


def _roof(stats_, peak_fp64, tensor_peak):
    """Roofline entry of the kernel with the largest share of device time in `stats_` (per-launch CUDA events)."""
    name, s = max(stats_.items(), key=lambda kv: kv[1]["ms"])
    achieved = s["flops"] / (s["ms"] * 1e-3) / 1e12
    if name.startswith("k_oz_tc") or name.startswith("k_oz7"):
        pk, src, bound = tensor_peak, "MEASURED_PEAKS.json bf16_tflops (burst, cuBLAS tcgen05)", "tensor"
    elif name.startswith("k_oz"):
        pk, src, bound = tensor_peak, ("MEASURED_PEAKS.json bf16_tflops (burst, cuBLAS tcgen05); this kernel issues "
                                       "mma.sync, measured at 605 TFLOP/s on this part"), "tensor"
    else:
        pk, src, bound = peak_fp64, "lkg_probe_fp64_peak measured in this run (DFMA pipe)", "fp64"
    traffic = None
    tf = ROOT / "profiles" / "dram_traffic.json"
    if tf.exists():
        try:
            ratio = json.loads(tf.read_text()).get(name, {}).get("ratio")
            if ratio is not None and s["launches"] > 0:
                traffic = ratio * s["bytes"] / s["launches"]
        except ValueError:
            traffic = None
    return dict(bound=bound, kernel=name, achieved=achieved, peak=pk, unit="TFLOP/s",
                frac=(achieved / pk) if pk else None, traffic=traffic, peak_source=src, launches=s["launches"],
                share=s["ms"] / sum(v["ms"] for v in stats_.values()))


def _kern(stats_):
    return {kk: dict(launches=v["launches"], ms=round(v["ms"], 3),
                     tflops=(v["flops"] / (v["ms"] * 1e-3) / 1e12) if v["ms"] > 0 else None)
            for kk, v in sorted(stats_.items(), key=lambda kv: -kv[1]["ms"])}


def run_gpu(args):
    rank, world, local = dist_env()
    import torch
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    import libkriging_gb300 as lk
    lib = lk.load()
    if args.digit_tile:
        if lib.lkg_set_digit_tile(args.digit_tile) != args.digit_tile:
            raise RuntimeError(lk._lib.last_error())
    peak_fp64 = ctypes.c_double()
    if lib.lkg_probe_fp64_peak(ctypes.byref(peak_fp64)) != 0:
        raise RuntimeError("FP64 peak probe failed: " + lk._lib.last_error())
    peak_dmma = ctypes.c_double()
    if lib.lkg_probe_dmma_peak(ctypes.byref(peak_dmma)) != 0:
        raise RuntimeError("DMMA peak probe failed: " + lk._lib.last_error())
    X, y, theta, alpha = make_inputs(args.n)
    gamma = np.concatenate([theta, [alpha]])
    k = lk.Kriging("matern5_2", "nugget")
    k.fit(y, X, "constant", False, "none", "LL", {"theta": theta.reshape(1, -1), "sigma2": 1.0, "nugget": 1e-6})

    def barrier():
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    # ---- FP64 path (secondary figures: fewer steps) ----
    k.set_precision(0)
    for _ in range(min(args.warmup, 2)):
        k.logLikelihoodFun(gamma, True, False, bench=True)
    barrier()
    fp64_steps = min(args.steps, 5)
    fp64_ms, (ll64, g64), st64, clk64, stage64 = _timed_steps(k, lib, gamma, fp64_steps, local, "fp64_step",
                                                              stats_steps=2)
    barrier()
    # ---- mixed path (headline) ----
    k.set_precision(args.slices)
    # the autotuner picks the SMs kept for the Cholesky look-ahead at this size (timed evaluations, tabled)
    lookahead_tuned = k.autotune_lookahead(gamma)
    for _ in range(args.warmup):
        k.logLikelihoodFun(gamma, True, False, bench=True)
    barrier()
    t0 = time.perf_counter()
    mix_ms, (llm, gm), stats, clk, stage = _timed_steps(k, lib, gamma, args.steps, local, "mixed_step",
                                                        stats_steps=min(args.steps, 5))
    barrier()
    wall_value = time.perf_counter() - t0
    used = k.last_slices()
    e2e_s = _e2e(lk, lib, k, gamma, args.steps, barrier)
    launches = sum(v["launches"] for v in stats.values())
    stats_steps = min(args.steps, 5)
    if world > 1:
        t = torch.tensor([mix_ms, e2e_s, fp64_ms], dtype=torch.float64, device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        mix_ms, e2e_s, fp64_ms = float(t[0]), float(t[1]), float(t[2])
    value = world * 1000.0 / mix_ms
    rel_ll = abs(llm - ll64) / abs(ll64)
    rel_g = float(np.linalg.norm(gm - g64) / np.linalg.norm(g64))
    peaks = measured_peaks()
    tensor_peak = peaks.get("bf16_tflops")
    line = dict(metric=METRIC, value=value, unit=UNIT, n_gpus=world, steps=args.steps, warmup=args.warmup,
                ms_per_step=mix_ms, higher_is_better=True, scaling="weak", vs_baseline=None,
                dtype="bf16+f64 (mixed: exact bf16 digit products on tcgen05, f64 panels, folds and reductions)",
                data="synthetic (seeded PCG64, seed 123)",
                config=dict(workload="dense LL+grad, n=%d, d=8, matern5_2, nugget 1e-6" % args.n,
                            precision="mixed: O(n^3) products on bf16 tensor cores by error-free digit splitting "
                                      "(%s), FP64 panels and reductions" % _digits_note(lib, used),
                            digit_products="tcgen05, 7-bit digits, 128x%d tiles, %s" % (
                                lib.lkg_get_digit_tile(), "two TMEM accumulator sets" if lib.lkg_get_digit_tile() == 32
                                else "one TMEM accumulator set"),
                            parallelism="replicas" if world > 1 else "single GPU",
                            cholesky_lookahead_sms=dict(autotuned=lookahead_tuned,
                                                        setting=lib.lkg_get_lookahead()),
                            l2="inputs larger than L2 (R, L^-1, R^-1: 3 x %.2f GB)" % (8.0 * args.n * args.n / 1e9)),
                e2e=dict(value=world / e2e_s, unit=UNIT, h2d_bytes_per_step=8 * gamma.size,
                         d2h_bytes_per_step=8 * (1 + gamma.size)),
                fp64=dict(value=world * 1000.0 / fp64_ms, ms_per_step=fp64_ms, steps=fp64_steps, dtype="f64",
                          roofline=_roof(st64, peak_fp64.value, tensor_peak),
                          stage_ms={kk: round(v, 3) for kk, v in stage64.items()}, kernels=_kern(st64),
                          clocks=clk64),
                speedup_mixed_vs_fp64=fp64_ms / mix_ms,
                rel_err_vs_fp64=dict(ll=rel_ll, grad=rel_g, ll_fp64=float(ll64), ll_mixed=float(llm)),
                gpu_launches=int(round(launches / max(1, stats_steps) * args.steps)),
                roofline=_roof(stats, peak_fp64.value, tensor_peak), clocks=clk,
                wall_s_timed_region=wall_value,
                measured_peaks={k2: v for k2, v in peaks.items() if k2 in ("hbm_gbs", "bf16_tflops",
                                                                           "bf16_tflops_sustained")},
                fp64_peak_tflops=peak_fp64.value, fp64_dmma_tflops=peak_dmma.value,
                stage_ms={kk: round(v, 3) for kk, v in stage.items()}, kernels=_kern(stats),
                kernel_stats_steps=stats_steps)
    if rank == 0 and world == 1 and not args.no_batched:
        # the batched fits in FP64 (the record's value), and the same fits on the mixed path beside them: at this
        # design's conditioning (cond(R) up to ~1e11) the mixed gradient can steer a fit to another local optimum,
        # so the mixed fit is reported with its distance from the FP64 fit, not as the value
        b64 = batched_multistart(lk, lib, steps=args.batched_steps, warmup=1, peak_fp64=peak_fp64.value,
                                 cpu=not args.no_cpu_baseline)
        bmx = batched_multistart(lk, lib, steps=1, warmup=1, peak_fp64=peak_fp64.value, cpu=False,
                                 mixed_slices=args.slices)
        b64["mixed"] = {kk: bmx[kk] for kk in ("value", "e2e", "device_ms_per_fit", "rounds_per_fit",
                                               "evaluations_per_fit", "theta", "ll", "dtype", "roofline")}
        b64["mixed"]["speedup_vs_fp64"] = dict(device=bmx["value"] / b64["value"],
                                               e2e=bmx["e2e"]["value"] / b64["e2e"]["value"])
        b64["mixed"]["rel_err_vs_fp64_fit"] = dict(
            ll=abs(bmx["ll"] - b64["ll"]) / abs(b64["ll"]),
            theta=float(np.linalg.norm(np.subtract(bmx["theta"], b64["theta"])) / np.linalg.norm(b64["theta"])))
        line["batched"] = b64
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        rec, ll_o, g_o = cpu_baseline(X, y, theta, alpha)
        line["cpu_baseline"] = rec
        line["rel_err_vs_oracle"] = dict(
            oracle="full-size CPU restatement of the reference path (the cpu_baseline evaluation)",
            ll_oracle=float(ll_o),
            mixed=dict(ll=abs(llm - ll_o) / abs(ll_o), grad=float(np.linalg.norm(gm - g_o) / np.linalg.norm(g_o))),
            fp64=dict(ll=abs(ll64 - ll_o) / abs(ll_o),
                      grad=float(np.linalg.norm(g64 - g_o) / np.linalg.norm(g_o))),
            targets=dict(mixed_ll=1e-8, mixed_grad=1e-6, fp64_ll=1e-10, fp64_grad=1e-7))
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def make_multistart_inputs(n=2048, d=6, starts=64, seed=123):
    """Batched multistart workload: X ~ U[0,1]^6, y = sum_j cos(3 x_j) x_j + N(0, 0.01) (variance 0.01), gauss,
    64 starting points theta ~ U[0.1, 2]^6; the nugget 1e-8 is Nugget mode with sigma2 and nugget fixed."""
    rng = np.random.default_rng(seed)
    X = rng.uniform(size=(n, d))
    y = (np.cos(3 * X) * X).sum(axis=1) + 0.1 * rng.standard_normal(n)
    thetas = rng.uniform(0.1, 2.0, size=(starts, d))
    s2 = float(np.var(y))
    return X, y, thetas, dict(sigma2=s2, is_sigma2_estim=False, nugget=1e-8 * s2, is_nugget_estim=False)


def batched_multistart(lk, lib, steps=2, warmup=1, peak_fp64=None, cpu=True, mixed_slices=0):
    """The batched half of the metric: BFGS64 fits of the n = 2048, d = 6 gauss design (sigma2 and nugget fixed).

    value   fits/s on the device: 1 / (batched rounds per fit x device ms of one 64-candidate round), the round timed
            by the library's CUDA-event stage timings with the design resident
    e2e     fits/s wall clock through the C ABI (lkg_kriging_fit_params: X, y and the 64 starts copied in from host
            memory, theta and LL read back), every round of the fit one batched GPU evaluation
    cpu_baseline  64 sequential reference-restated evaluations (one optimiser round of the reference's sequential
            multistart) timed in full, scaled to a fit by the GPU fit's round count"""
    import torch
    X, y, thetas, params = make_multistart_inputs()
    P = dict(params, theta=thetas)
    starts, d = thetas.shape
    method = "BFGS%d" % starts
    k = lk.Kriging("gauss", "nugget")
    k.set_precision(mixed_slices)
    for _ in range(warmup):
        k.fit(y, X, "constant", False, method, "LL", P)
    clocks = ClockSampler(0)
    clocks.start()
    ev0, ro0 = k.eval_counts()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(steps):
        k.fit(y, X, "constant", False, method, "LL", P)
    torch.cuda.synchronize()
    fit_s = (time.perf_counter() - t0) / steps
    ev1, ro1 = k.eval_counts()
    rounds_per_fit = (ro1 - ro0) / steps
    evals_per_fit = (ev1 - ev0) / steps
    theta_hat, ll_hat = k.theta().tolist(), k.logLikelihood()
    # device time of one fit: the CUDA-event durations of every kernel the fit launches (per-launch events)
    lib.lkg_stats_reset()
    lib.lkg_stats_enable(1)
    k.fit(y, X, "constant", False, method, "LL", P)
    lib.lkg_stats_enable(0)
    st = kernel_stats(lib)
    clk = clocks.stop()
    dev_fit_ms = sum(v["ms"] for v in st.values())
    n = X.shape[0]
    rec = dict(metric="batched multistart fits/s (BFGS%d, n=%d, d=%d, gauss, nugget 1e-8 sigma2 fixed)"
                      % (starts, n, d),
               value=1000.0 / dev_fit_ms, unit="fits/s", steps=steps, warmup=warmup,
               dtype="f64" if not mixed_slices else "bf16+f64",
               config=dict(workload="multistart BFGS%d, n=%d, d=%d, gauss, Nugget mode with sigma2 and nugget fixed "
                                    "(alpha = 1/(1+1e-8)), starts ~ U[0.1, 2]^6" % (starts, n, d),
                           l2="inputs larger than L2 (64 x R, L^-1, R^-1 of %.1f MB each)" % (8.0 * n * n / 1e6)),
               rounds_per_fit=rounds_per_fit, evaluations_per_fit=evals_per_fit,
               device_ms_per_fit=dev_fit_ms,
               fit_flops=evals_per_fit * float(n) ** 3,
               e2e=dict(value=1.0 / fit_s, unit="fits/s", ms_per_fit=1000.0 * fit_s,
                        h2d_bytes_per_step=8 * (X.size + y.size + thetas.size),
                        d2h_bytes_per_step=8 * (d + 1)),
               theta=theta_hat, ll=ll_hat, clocks=clk,
               gpu_launches_per_fit=int(sum(v["launches"] for v in st.values())),
               roofline=_roof(st, peak_fp64, measured_peaks().get("bf16_tflops")), kernels=_kern(st))
    if cpu:
        from oracle import baseline as B
        s2, nu = params["sigma2"], params["nugget"]
        alpha = s2 / (s2 + nu)
        t_round = 0.0
        det = None
        for i in range(starts):
            _, _, secs, det = B.eval_full(X, y, thetas[i], "gauss", alpha=alpha, fixed_var=(s2, nu))
            t_round += secs
        t_eval = t_round / starts
        rec["cpu_baseline"] = dict(
            value=1.0 / (evals_per_fit * t_eval), unit="fits/s", cores=int(det["threads"]), kind="port",
            eval_s=t_eval,
            sample="%d reference-restated LL+grad evaluations at the %d starting points timed in full (%.1f s, %.3f s "
                   "each); the reference runs its starts one after another, so a fit costs the GPU fit's %.0f "
                   "evaluations x %.3f s" % (starts, starts, t_round, t_eval, evals_per_fit, t_eval))
    return rec


def run_gpu_multistart(args):
    import libkriging_gb300 as lk
    lib = lk.load()
    peak_fp64 = ctypes.c_double()
    if lib.lkg_probe_fp64_peak(ctypes.byref(peak_fp64)) != 0:
        raise RuntimeError("FP64 peak probe failed: " + lk._lib.last_error())
    rec = batched_multistart(lk, lib, steps=args.steps, warmup=args.warmup, peak_fp64=peak_fp64.value,
                             cpu=not args.no_cpu_baseline, mixed_slices=args.slices if args.mixed else 0)
    line = dict(rec, n_gpus=1, ms_per_step=rec["e2e"]["ms_per_fit"], higher_is_better=True, scaling="weak",
                vs_baseline=None, data="synthetic (seeded PCG64, seed 123)")
    print(json.dumps(line), flush=True)


def make_vecchia_inputs(n=1 << 20, d=3, seed=123):
    """Vecchia workload: X ~ U[0,1]^3, y = sum_j sin(2 pi x_j) + N(0, 1e-4) (variance 1e-4), gauss, m = 30; the
    nugget 1e-6 is LinearAlgebra::set_num_nugget(1e-6) (the jitter of every conditional block)."""
    rng = np.random.default_rng(seed)
    X = rng.uniform(size=(n, d))
    y = np.sin(2 * np.pi * X).sum(axis=1) + 0.01 * rng.standard_normal(n)
    return X, y


def run_gpu_vecchia(args):
    """One step = one Vecchia LL + gradient evaluation (VLL(30)) of the fitted n = 2^20 model, sets resident on the
    device.  The line also times the GPU construction of the sets (maxmin order + neighbours) and the whole fit."""
    import libkriging_gb300 as lk
    lib = lk.load()
    peak_fp64 = ctypes.c_double()
    if lib.lkg_probe_fp64_peak(ctypes.byref(peak_fp64)) != 0:
        raise RuntimeError("FP64 peak probe failed: " + lk._lib.last_error())
    n = args.n if args.n != 16384 else (1 << 20)
    X, y = make_vecchia_inputs(n)
    lk.set_num_nugget(1e-6)
    t0 = time.perf_counter()
    lk.vecchia_sets(X, 30)
    sets_s = time.perf_counter() - t0
    k = lk.Kriging("gauss")
    k.set_vecchia_exact_commit(False)
    lib.lkg_stats_reset()
    lib.lkg_stats_enable(1)
    t0 = time.perf_counter()
    k.fit(y, X, "constant", False, "BFGS", "LLVecchia(30)", {"theta": np.full((1, 3), 0.1)})
    fit_s = time.perf_counter() - t0
    lib.lkg_stats_enable(0)
    fit_stats = kernel_stats(lib)
    th = k.theta()
    for _ in range(args.warmup):
        k.logLikelihoodVecchiaFun(th, True)
    clocks = ClockSampler(0)
    clocks.start()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        vll, g = k.logLikelihoodVecchiaFun(th, True)
    wall = time.perf_counter() - t0
    clk = clocks.stop()
    # predictVecchia at scale: 10^4 new points, each kriged on its 30 nearest observations
    Xq = np.random.default_rng(124).uniform(size=(10000, 3))
    k.predictVecchia(Xq[:100], True, 30)
    t0 = time.perf_counter()
    pmean, psd = k.predictVecchia(Xq, True, 30)
    pv_s = time.perf_counter() - t0
    lib.lkg_stats_reset()
    lib.lkg_stats_enable(1)
    for _ in range(min(args.steps, 3)):
        k.logLikelihoodVecchiaFun(th, True)
    lib.lkg_stats_enable(0)
    stats = kernel_stats(lib)
    line = dict(metric="VLL(30)+grad evals/s at n=2^20, d=3 (gauss, num_nugget 1e-6)", value=args.steps / wall,
                unit="evals/s", n_gpus=1, steps=args.steps, warmup=args.warmup, ms_per_step=1000 * wall / args.steps,
                higher_is_better=True, scaling="weak", vs_baseline=None, dtype="f64",
                data="synthetic (seeded PCG64, seed 123)",
                config=dict(workload="Vecchia LLVecchia(30), n=%d, d=3, gauss, light commit" % n,
                            l2="inputs larger than L2 (n x 30 neighbour table + per-point terms)"),
                e2e=dict(value=args.steps / wall, unit="evals/s", h2d_bytes_per_step=8 * 3,
                         d2h_bytes_per_step=8 * 4,
                         note="logLikelihoodVecchiaFun through the C ABI: theta in, (VLL, gradient) out"),
                sets_s=sets_s, fit_s_including_sets=fit_s, theta=th.tolist(), vll=vll, clocks=clk,
                predict_vecchia=dict(points=int(Xq.shape[0]), m=30, seconds=pv_s),
                fit_kernels={kk: dict(launches=v["launches"], ms=round(v["ms"], 3)) for kk, v in fit_stats.items()},
                gpu_launches=int(sum(v["launches"] for v in stats.values()) / max(1, min(args.steps, 3))),
                roofline=_roof(stats, peak_fp64.value, None), kernels=_kern(stats))
    if not args.no_cpu_baseline:
        from oracle import oracle as O
        O.build()
        order, nbr = k.vecchia_sets()
        F = np.ones((n, 1), order="F")
        Xf = np.asfortranarray(X)
        th_c = np.ascontiguousarray(th)
        cnt = 4096
        t1 = time.perf_counter()
        O.lib().ora_vecchia_points_sample(O.KERNELS["gauss"], n, 3, 1, O._dp(Xf), O._dp(np.ascontiguousarray(y)),
                                          O._dp(F), O._dp(th_c), O._ip(order), O._ip(np.ascontiguousarray(nbr)),
                                          nbr.shape[1], 1e-6, 0, cnt)
        s = (time.perf_counter() - t1) * n / cnt
        line["cpu_baseline"] = dict(value=1.0 / s, unit="evals/s", cores=1, kind="port",
                                    sample="serial per-point loop of _logLikelihoodVecchia with gradient (the "
                                           "reference's loop is serial) on the first %d of %d ordered points, "
                                           "scaled by n" % (cnt, n))
        # the reference-style O(n^2) set construction on a bounded size, against the GPU grid construction
        ns = min(n, args.vecchia_sets_cpu_n)
        Xs = X[:ns]
        t1 = time.perf_counter()
        O.vecchia_sets(Xs, 30)
        cpu_sets = time.perf_counter() - t1
        t1 = time.perf_counter()
        lk.vecchia_sets(Xs, 30)
        gpu_sets = time.perf_counter() - t1
        # predictVecchia on the CPU: the reference's per-point work on a sample of the points, all host threads
        from oracle import baseline as Bv
        resid = (y - (k.beta()[0] if len(k.beta()) else 0.0))
        qs = 256
        pm_c, _, pv_cpu = Bv.predict_vecchia_sample("gauss", X, resid, th, k.sigma2(), Xq[:qs], 30,
                                                     num_nugget=lk.get_num_nugget())
        line["predict_vecchia"]["cpu_baseline"] = dict(
            seconds=pv_cpu * Xq.shape[0] / qs, cores=Bv.host_threads(), kind="port",
            mean_rel_diff=float(np.linalg.norm(pm_c - (pmean[:qs] - (k.beta()[0] if len(k.beta()) else 0.0)))
                                / np.linalg.norm(pm_c)),
            sample="%d of the %d points' predictions timed in full (distances to all %d observations, partial "
                   "selection, local kriging) on all host threads, scaled by the point count" % (qs, Xq.shape[0], n))
        line["sets_cpu_baseline"] = dict(n=ns, cpu_s=cpu_sets, gpu_s=gpu_sets, cores=1, kind="port",
                                         sample="make_vecchia_sets restated (O(n^2) maxmin + neighbour selection) "
                                                "on the first %d points" % ns)
    print(json.dumps(line), flush=True)


def make_nested_inputs(n_total=1_000_000, d=4, seed=123):
    """NestedKriging workload: X ~ U[0,1]^4, y = sum_j sin(4 x_j) + N(0, 0.01) (variance 0.01), matern3_2.
    The partition is synthesised: group sizes ~ lognormal(median 1000, sigma 0.67) truncated to [150, 2500] until
    they cover n_total, and the points cut into consecutive runs of a 4-D Z-order (Morton) ordering, so that every
    group is spatially compact."""
    rng = np.random.default_rng(seed)
    X = rng.uniform(size=(n_total, d))
    y = np.sin(4 * X).sum(axis=1) + 0.1 * rng.standard_normal(n_total)
    sizes = []
    left = n_total
    while left > 0:
        s = int(np.clip(round(np.exp(np.log(1000.0) + 0.67 * rng.standard_normal())), 150, 2500))
        if left - s < 150:
            s = left if left <= 2500 else left - 150
        sizes.append(s)
        left -= s
    q = np.minimum((X * 65536).astype(np.uint64), np.uint64(65535))
    key = np.zeros(n_total, dtype=np.uint64)
    for b in range(16):
        for j in range(d):
            key |= ((q[:, j] >> np.uint64(b)) & np.uint64(1)) << np.uint64(b * d + j)
    order = np.argsort(key, kind="stable")
    labels = np.empty(n_total, dtype=np.int32)
    start = 0
    for g, s in enumerate(sizes):
        labels[order[start:start + s]] = g
        start += s
    return X, y, labels, np.array(sizes)


def run_gpu_nested(args):
    """One step = the submodel objective (concentrated LL + theta-gradient) of every group in one batched
    evaluation; the complete NestedKriging fit (all submodel BFGS fits, common prior, refits) is timed once."""
    import libkriging_gb300 as lk
    lib = lk.load()
    n_total = args.nested_n
    X, y, labels, sizes = make_nested_inputs(n_total)
    p, d = len(sizes), X.shape[1]
    nk = lk.NestedKriging("matern3_2", aggregation="gPoE")
    if args.mixed:
        nk.set_precision(args.slices)
    clocks = ClockSampler(0)
    clocks.start()
    t0 = time.perf_counter()
    nk.fit_groups(y, X, labels, "constant", "BFGS", "LL")
    fit_s = time.perf_counter() - t0
    print("nested: %d groups fitted in %.1f s" % (len(sizes), fit_s), file=sys.stderr, flush=True)
    rng = np.random.default_rng(7)
    thetas = rng.uniform(0.1, 0.6, size=(p, d))
    for _ in range(args.warmup):
        nk.logLikelihoodGroups(thetas, True)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        ll, g = nk.logLikelihoodGroups(thetas, True)
    wall = time.perf_counter() - t0
    # per-kernel table from one more evaluation with per-launch CUDA events (kept out of the timed steps)
    lib.lkg_stats_reset()
    lib.lkg_stats_enable(1)
    nk.logLikelihoodGroups(thetas, True)
    lib.lkg_stats_enable(0)
    stats = kernel_stats(lib)
    mixed_err = None
    if args.mixed:  # the same evaluation on the FP64 path
        nk.set_precision(0)
        ll64, g64 = nk.logLikelihoodGroups(thetas, True)
        nk.set_precision(args.slices)
        mixed_err = dict(ll_max=float(np.max(np.abs(ll - ll64) / np.abs(ll64))),
                         grad_max=float(np.max(np.linalg.norm(g - g64, axis=1) / np.linalg.norm(g64, axis=1))))
    Xp = np.random.default_rng(124).uniform(size=(args.nested_q, d))
    t1 = time.perf_counter()
    mean, sd = nk.predict(Xp, True)
    pred_s = time.perf_counter() - t1
    clk = clocks.stop()
    n3 = float(np.sum(sizes.astype(np.float64) ** 3))
    dom = max(stats.items(), key=lambda kv: kv[1]["ms"]) if stats else ("", {"ms": 0.0, "flops": 0.0})
    line = dict(metric="NestedKriging submodel LL+grad evals/s (all groups batched), N=%d, d=4, matern3_2" % n_total,
                value=p * args.steps / wall, unit="evals/s", n_gpus=1, steps=args.steps, warmup=args.warmup,
                ms_per_step=1000 * wall / args.steps, higher_is_better=True, scaling="weak", vs_baseline=None,
                dtype="bf16+f64" if args.mixed else "f64",
                data="synthetic (seeded PCG64, seed 123; lognormal group sizes, Z-order partition)",
                config=dict(workload="NestedKriging N=%d d=4 matern3_2, %d groups of %d..%d points (median %d)"
                            % (n_total, p, sizes.min(), sizes.max(), int(np.median(sizes))),
                            precision="mixed %d digits" % args.slices if args.mixed else "FP64",
                            l2="inputs larger than L2 (sum n_g^2 * 8 B = %.1f GB of covariance per step)"
                               % (8.0 * np.sum(sizes.astype(np.float64) ** 2) / 1e9)),
                groups=p, sum_n_cubed=n3, fit_seconds=fit_s, submodel_fits_per_s=p / fit_s,
                rel_err_vs_fp64=mixed_err,
                predict_gpoe_points=args.nested_q, predict_seconds=pred_s, theta=nk.theta().tolist(),
                sigma2=nk.sigma2(), clocks=clk, gpu_launches=int(sum(v["launches"] for v in stats.values())),
                kernels={kk: dict(launches=v["launches"], ms=round(v["ms"], 3)) for kk, v in stats.items()},
                dominant=dict(kernel=dom[0], ms=dom[1]["ms"], share=dom[1]["ms"] / max(1e-9, sum(
                    v["ms"] for v in stats.values()))))
    if args.nested_nk:
        # NK aggregation on one 128-point chunk: a model with the fitted common theta (optim "none", so every group
        # keeps it), its NK factorisations, then one chunk of predictions; the pair cross-covariances are
        # sum_{i<j} n_i n_j kernel evaluations and 2 x 128 x that many FP64 flops per chunk
        nkm = lk.NestedKriging("matern3_2", aggregation="NK")
        if args.mixed:
            nkm.set_precision(args.slices)
        t0 = time.perf_counter()
        nkm.fit_groups(y, X, labels, "constant", "none", "LL", {"theta": np.asarray(nk.theta()).reshape(1, -1)})
        nk_setup_s = time.perf_counter() - t0
        s1 = float(np.sum(sizes.astype(np.float64)))
        pair_evals = 0.5 * (s1 * s1 - float(np.sum(sizes.astype(np.float64) ** 2)))
        lib.lkg_stats_reset()
        lib.lkg_stats_enable(1)
        t0 = time.perf_counter()
        m_nk, s_nk = nkm.predict(Xp[:128], True)
        nk_s = time.perf_counter() - t0
        lib.lkg_stats_enable(0)
        st_nk = kernel_stats(lib)
        line["nk_chunk"] = dict(points=128, seconds=nk_s, setup_seconds=nk_setup_s, group_pairs=p * (p - 1) // 2,
                                pair_kernel_evaluations=pair_evals, bilinear_flops=2.0 * 128 * pair_evals,
                                kernels={kk: dict(launches=v["launches"], ms=round(v["ms"], 3))
                                         for kk, v in st_nk.items()},
                                mean_rel_diff_vs_gpoe=float(np.linalg.norm(m_nk - mean[:128]) /
                                                            np.linalg.norm(mean[:128])))
        del nkm
    print("nested (GPU part): " + json.dumps(line), file=sys.stderr, flush=True)
    if not args.no_cpu_baseline:
        from oracle import baseline as B
        from oracle import oracle as O
        O.build()
        pick = np.random.default_rng(3).choice(p, size=min(8, p), replace=False)
        t_s, n3s = 0.0, 0.0
        det = None
        for gi in pick:
            idx = np.flatnonzero(labels == gi)
            _, _, s, det = B.eval_full(X[idx], y[idx], thetas[gi], "matern3_2")
            t_s += s
            n3s += float(len(idx)) ** 3
        per_step = t_s * n3 / n3s
        # the gPoE prediction on the CPU: the sample groups' full predictions of qs points, scaled to every group
        # and the q points by sum n_g^2 q (the triangular solves dominate)
        qs = min(2000, args.nested_q)
        t_p, n2s = 0.0, 0.0
        for gi in pick[:4]:
            idx = np.flatnonzero(labels == gi)
            _, _, s = B.predict_group_full(X[idx], y[idx], nk.theta(), "matern3_2", nk.beta0(), Xp[:qs])
            t_p += s
            n2s += float(len(idx)) ** 2 * qs
        n2q = float(np.sum(sizes.astype(np.float64) ** 2)) * args.nested_q
        line["predict_cpu_baseline"] = dict(
            seconds=t_p * n2q / n2s, points=args.nested_q, gpu_seconds=pred_s, cores=int(det["threads"]), kind="port",
            sample="4 groups' predictions of %d points timed in full (covariances, factor, triangular solves), "
                   "scaled to all %d groups and %d points by sum n_g^2 q" % (qs, p, args.nested_q))
        line["cpu_baseline"] = dict(value=p / per_step, unit="evals/s", cores=int(det["threads"]), kind="port",
                                    sample="reference-restated LL+grad of %d groups (%s points) each timed in full, "
                                           "scaled to all %d groups by sum n_g^3 (the reference fits its groups one "
                                           "after another)" % (len(pick), ",".join(
                                               str(int(np.sum(labels == gi))) for gi in pick), p))
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--n", type=int, default=16384)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--slices", type=int, default=7, help="digit slices of the mixed path (4..8)")
    ap.add_argument("--workload", default="dense", choices=["dense", "multistart", "vecchia", "nested"])
    ap.add_argument("--mixed", action="store_true", help="multistart / nested workloads on the mixed path")
    ap.add_argument("--nested-n", type=int, default=1_000_000, help="points of the nested workload")
    ap.add_argument("--nested-q", type=int, default=100_000, help="gPoE prediction points of the nested workload")
    ap.add_argument("--vecchia-sets-cpu-n", type=int, default=1 << 16,
                    help="points of the O(n^2) CPU set construction timed beside the GPU one (vecchia workload)")
    ap.add_argument("--nested-nk", action="store_true",
                    help="nested workload: also time NK aggregation on one 128-point chunk")
    ap.add_argument("--no-batched", action="store_true", help="omit the batched multistart sub-record")
    ap.add_argument("--digit-tile", type=int, default=0, choices=[0, 32, 64],
                    help="output tile width of the digit products (0: the library's default)")
    ap.add_argument("--batched-steps", type=int, default=2, help="timed BFGS64 fits of the batched sub-record")
    ap.add_argument("--ref-budget-s", type=float, default=300.0,
                    help="reference arm: stop timing full CPU evaluations once the next would pass this many s")
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == "multistart":
        run_gpu_multistart(args)
    elif args.workload == "nested":
        run_gpu_nested(args)
    elif args.workload == "vecchia":
        run_gpu_vecchia(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
