#!/usr/bin/env python
"""Benchmark of the MPSFT recovery loop on GB300.

Workload (one "step"): a batched recovery (the Demo1::Run loop of
jiaweichiu/mpsft, src/demo1.cc:36-59) of G independent synthetic signals of
the headline configuration: N = 2^22 complex64 samples, S = 1000 modes at
distinct uniform-random frequencies, |c| log-uniform in [1e-2, 1], uniform
phase, complex Gaussian noise at 60 dB SNR; reference parameters trials = 1,
window_delta = 1e-5, window_threshold = 0.1, max_stale_iter = 5,
min_bins = 51 (src/demo1_bench.cc:34-39), thresholds 3 sigma/sqrt(B) and
sigma/sqrt(B). FP32 gather/fold/FFT, FP64 pencil and coefficients.

Printed: one JSON line. ``value`` is recoveries per second with the signals
resident in HBM (G x 32 MiB > L2, so no L2 flush is needed); ``e2e`` is the
same through the public API from pinned host buffers (host-to-device copy of
every signal and device-to-host read of every result inside the timed region;
the next step's copies run on a copy stream during the current step's solve).

``--impl reference`` times the reference's algorithm on the host cores: the
oracle's FP64 restatement (oracle/liboracle.so, or liboracle_fast.so with the
reference's -O3 -ffast-math flags when that build is faster here), one
process per core, each recovering its own signal of the same configuration.

Also reported (rank 0): the plain per-signal FP64 GPU path and the same
64-signal batch on the FP64 kernels (batching and precision gains apart), the
accuracy of one recovery against an FP64 dense FFT (hits, misses, algorithm
and precision errors), dense full-N FFT rates (scipy on the host cores, cuFFT
on the device), the device test-data pipeline (generation, PostAnalyze)
against its host form, the 256-signal uneven batch (config 3), the N = 2^26
stress signal alone and four at a time (config 5), and the reference's own
binning micro-benchmark shape (N = 4194301, B = 501, bits = 15).

``roofline`` is the binning kernel's: algorithmic bytes over event-timed
launch durations of a profiled pass (every binning launch timed alone), for
all launches and per phase (``first``: the first iteration, B = 2001;
``fixed_bins``: the late iterations at B = min_bins = 51), with each phase's
DRAM bytes per gathered sample as ncu measured them on this workload
(profiles/bin_fold_phases_config2_batch64.md).

Multi-GPU: one process per GPU under torchrun; every rank recovers its own G
signals (independent replicas, no collective on the data path); the time is the
maximum over ranks.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time
from concurrent.futures import ThreadPoolExecutor

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = ("solves/s, N=2^22 S=1000: batched FP32 vs plain GPU @ coef err≤1e-5; "
          "bin GB/s")
N = 1 << 22
S = 1000
SEED_RNG = 123537
WORKLOAD = ("MPSFT recovery (Demo1::Run loop), N=2^22 complex64, S=1000, "
            "|c| log-uniform [1e-2,1], 60 dB SNR, trials=1, delta=1e-5, "
            "min_bins=51, max_stale_iter=5")


def parse_args():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=30)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--batch", type=int, default=64, help="signals per step per GPU")
    p.add_argument("--workload", choices=["config2", "config3"], default="config2",
                   help="config3: one step = the 256-signal uneven batch "
                        "(N in 2^16..2^24, S in [10, 2000]); reported on its own "
                        "line, not the headline")
    p.add_argument("--impl", choices=["gpu", "reference"], default="gpu")
    p.add_argument("--cpu-seconds", type=float, default=10.0,
                   help="bounded CPU-baseline sample length")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-extras", action="store_true",
                   help="skip the extra workloads (batched FP64, configs 3 and 5, "
                        "the reference's binning micro-benchmark shape)")
    p.add_argument("--profile-case", action="store_true",
                   help="one batched solve with the host-driven loop and "
                        "nothing else (the case the ncu summaries capture)")
    return p.parse_args()


def solve_opts(ctx, sigma, precision):
    import mpsft_gb300 as m
    return ctx.solve_options(S, sigma, trials=1, min_bins=51, window_delta=1e-5,
                             window_threshold=0.1, max_stale_iter=5,
                             precision=precision)


# ------------------------------------------------------------------ clocks
class ClockSampler:
    """Samples SM clocks and throttle reasons with nvidia-smi while running."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,"
              "clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "50"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"]}
        self.proc.terminate()
        try:
            out, _ = self.proc.communicate(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
            out, _ = self.proc.communicate()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown",
                 "sw_power_cap"]
        for line in out.splitlines():
            f = [v.strip() for v in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax),
                "samples": len(sm), "reasons": sorted(reasons)}


# ------------------------------------------------------------ CPU baseline
# The oracle port in two builds: "port" (-O2, no FP contraction: the checker's
# build) and "port_fast" (the reference's optimised flags, -O3 -ffast-math).
# The CPU baseline reports the faster of the two.
_BUILDS = {"port": "-O2 strict FP", "port_fast": "-O3 -ffast-math"}


def _oracle_lib(kind: str):
    from oracle import oracle
    if not oracle.available(kind):
        (oracle.build_port if kind == "port" else oracle.build_port_fast)()
    return oracle.Oracle(kind)


def host_cpu() -> str:
    try:
        out = subprocess.run(["lscpu"], stdout=subprocess.PIPE,
                             stderr=subprocess.DEVNULL, text=True).stdout
        for line in out.splitlines():
            if line.startswith("Model name:"):
                return line.split(":", 1)[1].strip()
    except OSError:
        pass
    import platform
    return platform.processor() or platform.machine()


def _cpu_worker_init(seed, kind="port"):
    global _W_SIG, _W_KIND
    from mpsft_gb300.signals import config2
    _W_SIG = config2(seed)
    _W_KIND = kind


def _cpu_worker_solve(rseed):
    port = _oracle_lib(_W_KIND)
    t0 = time.perf_counter()
    modes, _ = port.demo1_run(_W_SIG.x.astype(np.complex128), S, _W_SIG.sigma, rseed,
                              min_bins=51, window_delta=1e-5, max_stale_iter=5)
    return time.perf_counter() - t0, len(modes)


def _time_build(kind: str, x, sigma, seconds: float, min_runs: int = 1):
    port = _oracle_lib(kind)
    done, t_total, sets = 0, 0.0, []
    while t_total < seconds or done < min_runs:
        t0 = time.perf_counter()
        modes, _ = port.demo1_run(x, S, sigma, SEED_RNG + done, min_bins=51,
                                  window_delta=1e-5, max_stale_iter=5)
        t_total += time.perf_counter() - t0
        sets.append(sorted(modes))
        done += 1
    return done, t_total, sets


def faster_build(x, sigma) -> str:
    """The faster oracle build on this host (two solves each, after one warm-up)."""
    best, best_t = "port", None
    for kind in _BUILDS:
        _time_build(kind, x, sigma, 0.0)
        _, t, _ = _time_build(kind, x, sigma, 0.0, min_runs=2)
        if best_t is None or t < best_t:
            best, best_t = kind, t
    return best


def cpu_baseline_single(seconds: float) -> dict:
    """The oracle port on one host core, a bounded sample of whole solves in
    each build; the value is the faster build's."""
    from mpsft_gb300.signals import config2
    sg = config2(1001)
    x = sg.x.astype(np.complex128)
    res = {}
    for kind in _BUILDS:
        _time_build(kind, x, sg.sigma, 0.0)  # warm-up
        res[kind] = _time_build(kind, x, sg.sigma, seconds / 2)
    rates = {kind: d / t for kind, (d, t, _) in res.items()}
    best = max(rates, key=rates.get)
    d, t, _ = res[best]
    n_same = min(len(v[2]) for v in res.values())
    same = all(res["port"][2][i] == res["port_fast"][2][i] for i in range(n_same))
    return {"value": rates[best], "unit": "solves/s", "cores": 1,
            "kind": "port",
            "sample": f"{d} full config-2 recoveries on 1 core ({t:.1f} s, "
                      f"oracle/mpsft_oracle.cc, {_BUILDS[best]}, FP64)",
            "host": host_cpu(),
            "builds": {_BUILDS[k]: v for k, v in rates.items()},
            "builds_same_frequency_sets": same}


def run_reference(args) -> None:
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    import multiprocessing as mp
    from mpsft_gb300.signals import config2
    cores = len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") \
        else (os.cpu_count() or 1)
    sg = config2(2024)
    kind = faster_build(sg.x.astype(np.complex128), sg.sigma)
    ctxm = mp.get_context("spawn")
    step_times = []
    with ctxm.Pool(cores, initializer=_cpu_worker_init, initargs=(2024, kind)) as pool:
        # warm-up: every worker builds its signal and runs once
        for w in range(args.warmup):
            pool.map(_cpu_worker_solve, [SEED_RNG + 1000 * w + i for i in range(cores)])
        for s in range(args.steps):
            t0 = time.perf_counter()
            pool.map(_cpu_worker_solve, [SEED_RNG + 77 * s + i for i in range(cores)])
            step_times.append(time.perf_counter() - t0)
    total = sum(step_times)
    value = cores * args.steps / total
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "solves/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * total / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic",
        "config": {"workload": WORKLOAD, "batch": cores,
                   "implementation": "oracle port of the reference algorithm "
                                     f"({_BUILDS[kind]}, the faster build here), "
                                     "one process per host core"},
        "cpu_baseline": {"value": value, "unit": "solves/s", "cores": cores,
                         "kind": "port",
                         "sample": f"{args.steps} steps x {cores} recoveries, one "
                                   f"per core",
                         "host": host_cpu()},
        "e2e": {"value": value, "unit": "solves/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# ------------------------------------------------------- multi-rank helpers
def rank_seeds(rank: int, batch: int) -> list[int]:
    """Signal seeds of one rank: every rank recovers its own batch (replicas)."""
    return [10_000 + rank * batch + i for i in range(batch)]


def max_over_ranks(ms: float, dist, device) -> float:
    """The slowest rank's time (the job's time); ms itself on one rank."""
    import torch
    t = torch.tensor([ms], dtype=torch.float64, device=device)
    if dist:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_rate(world: int, batch: int, steps: int, ms: float) -> float:
    """Recoveries per second of the whole job: every rank's signals over the
    slowest rank's time."""
    return world * batch * steps / (ms / 1e3)


# ----------------------------------------------------------------- GPU arm
def dense_fft(torch, sigs_host, device, reps: int = 5) -> dict:
    """Dense full-N FFTs of the same signals, the comparators of a sparse
    recovery: scipy's FP64 FFT (pocketfft) on the host cores, one worker and
    all of them, and cuFFT (through torch.fft) over the resident batch in
    complex64 and complex128. Rates are transforms per second."""
    import scipy.fft
    cores = len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") \
        else (os.cpu_count() or 1)
    out = {"unit": "full-N transforms/s", "n": N}
    x = sigs_host[0].x.astype(np.complex128)
    for w in (1, cores):
        scipy.fft.fft(x, workers=w)
        t0 = time.perf_counter()
        for _ in range(reps):
            scipy.fft.fft(x, workers=w)
        out[f"scipy_fft_f64_{w}_cores"] = reps / (time.perf_counter() - t0)
    G = len(sigs_host)
    xb = torch.empty((G, N), dtype=torch.complex64, device=device)
    for i, sg in enumerate(sigs_host):
        xb[i].copy_(torch.from_numpy(sg.x))
    for name, dt in (("cufft_c64", torch.complex64), ("cufft_c128", torch.complex128)):
        xt = xb if dt == torch.complex64 else xb.to(dt)
        y = torch.fft.fft(xt)
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(reps):
            y = torch.fft.fft(xt)
        e1.record()
        torch.cuda.synchronize()
        out[name] = G * reps / (e0.elapsed_time(e1) / 1e3)
        del y, xt
    out["cufft_batch"] = G
    del xb
    torch.cuda.empty_cache()
    return out


def test_data_pipeline(ctx, m, sg, k32, c32, reps: int = 5) -> dict:
    """Demo1's constructor and PostAnalyze for one config-2 signal, on the
    device (mpsft_signal_generate, mpsft_post_analyze) and on the host
    (numpy's FFT and normal draws; the oracle's PostAnalyze over a numpy
    spectrum). Times in ms per signal, each call synchronous."""
    from mpsft_gb300.signals import make_signal
    out = {}
    sig = ctx.generate(sg.n, sg.k, sg.c, sg.sigma, 1, m.C64)
    sig.free()
    t0 = time.perf_counter()
    for r in range(reps):
        sig = ctx.generate(sg.n, sg.k, sg.c, sg.sigma, 1 + r, m.C64)
        sig.free()
    out["generate_device_ms"] = 1e3 * (time.perf_counter() - t0) / reps
    t0 = time.perf_counter()
    make_signal(sg.n, S, 99, magnitude="loguniform", mag_range=(1e-2, 1.0),
                snr_db=60.0)
    out["generate_host_ms"] = 1e3 * (time.perf_counter() - t0)
    sig = ctx.upload(sg.x)
    ctx.post_analyze(sig, sg.k, k32, c32)
    t0 = time.perf_counter()
    for _ in range(reps):
        dev = ctx.post_analyze(sig, sg.k, k32, c32)
    out["post_analyze_device_ms"] = 1e3 * (time.perf_counter() - t0) / reps
    sig.free()
    port = _oracle_lib("port")
    t0 = time.perf_counter()
    host = port.post_analyze(np.fft.fft(sg.x.astype(np.complex128)) / sg.n, sg.k,
                             k32, c32)
    out["post_analyze_host_ms"] = 1e3 * (time.perf_counter() - t0)
    out["post_analyze_same"] = all(
        (np.isnan(host[key]) and np.isnan(dev[key])) or
        abs(host[key] - dev[key]) <= 1e-9 * abs(host[key]) for key in host)
    out["analysis"] = dev
    return out


def accuracy(sg, k32, c32, k64, c64) -> dict:
    """Errors of one recovery against an FP64 dense FFT x^ = fft(x)/N, as
    Demo1::PostAnalyze (src/demo1.cc:61-112) reports them: found modes that
    are true modes (hits) and the others (misses), the coefficient error of
    the hits, and the precision error of the FP32 path against the FP64 path."""
    x = sg.x.astype(np.complex128)
    xf = np.fft.fft(x) / sg.n
    true = set(int(v) for v in sg.k)

    def errs(kk, cc):
        hit = np.array([int(v) in true for v in kk], bool)
        kh = np.asarray(kk)[hit].astype(np.int64)
        d = np.asarray(cc)[hit] - xf[kh]
        return {"hits": int(hit.sum()), "misses": int((~hit).sum()),
                "algorithm_err": float(np.linalg.norm(d) / np.linalg.norm(xf[kh])),
                "hit_l1_err": float(np.abs(d).mean())}

    out = {"fp32_path": errs(k32, c32), "fp64_path": errs(k64, c64),
           "true_modes": len(true)}
    if np.array_equal(k32, k64):
        out["precision_err"] = float(np.linalg.norm(c32 - c64) / np.linalg.norm(c64))
    return out


def load_peaks() -> dict:
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return {"hbm_gbs": d.get("hbm_gbs"), "source": "measured"}
    return {"hbm_gbs": 6800.0, "source": "fallback"}


PHASE_PROFILE = os.path.join(ROOT, "profiles", "bin_fold_phases_config2_batch64.md")


def random_gather_ceiling(torch, device, gathers: int = 1 << 25,
                          span_bytes: int = 2 << 30, reps: int = 5) -> dict:
    """The GPU's rate of 8-byte reads at uniformly random addresses of a
    2 GiB buffer (a library gather kernel, torch.take): the ceiling of a
    binning launch whose samples are too sparse to share DRAM lines (the
    late iterations). Reported beside the roofline, which stays against the
    copy bandwidth."""
    x = torch.empty(span_bytes // 8, dtype=torch.float64, device=device)
    idx = torch.randint(0, x.numel(), (gathers,), device=device)
    y = torch.take(x, idx)
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(reps):
        y = torch.take(x, idx)
    e1.record()
    torch.cuda.synchronize()
    rate = gathers * reps / (e0.elapsed_time(e1) / 1e3)
    del x, idx, y
    torch.cuda.empty_cache()
    return {"gathers_per_s": rate, "sector_gb_per_s": 32 * rate / 1e9,
            "how": f"torch.take of {gathers} float64 at uniform random indices "
                   f"of a {span_bytes >> 30} GiB buffer"}


def profile_traffic() -> dict:
    """Measured DRAM traffic of the binning launches per phase, from the ncu
    summary committed under profiles/: {phase: {"dram_bytes_per_launch",
    "gathers_per_launch", "dram_bytes_per_gather"}} ({} when absent). Lines
    read: ``traffic <phase>: key=value ...``."""
    out = {}
    if not os.path.exists(PHASE_PROFILE):
        return out
    for line in open(PHASE_PROFILE):
        if not line.startswith("traffic "):
            continue
        head, _, rest = line.partition(":")
        phase = head.split()[1]
        vals = {}
        for tok in rest.split():
            k, _, v = tok.partition("=")
            try:
                vals[k] = float(v)
            except ValueError:
                pass
        out[phase] = vals
    return out


def phase_of(rec: dict, min_bins: int) -> list[str]:
    """Phases a binning launch belongs to: "first" (the first iteration, the
    largest bins), "fixed_bins" (every signal at min_bins: the late
    iterations), and "all"."""
    ph = ["all"]
    if rec["iteration"] == 0:
        ph.append("first")
    if rec["max_bins"] == min_bins:
        ph.append("fixed_bins")
    return ph


def binning_roofline(records: list[dict], min_bins: int, peak: float,
                     traffic: dict) -> dict:
    """Achieved GB/s (algorithmic bytes / event-timed duration) per phase over
    the profiled launches, with the measured DRAM bytes of that phase's
    launches (ncu) where the summary has them."""
    acc = {}
    for r in records:
        for ph in phase_of(r, min_bins):
            a = acc.setdefault(ph, {"launches": 0, "bytes": 0, "gathers": 0, "ms": 0.0})
            a["launches"] += 1
            a["bytes"] += r["bytes"]
            a["gathers"] += r["gathers"]
            a["ms"] += r["ms"]
    out = {}
    for ph, a in acc.items():
        if a["ms"] <= 0:
            continue
        achieved = a["bytes"] / (a["ms"] / 1e3) / 1e9
        d = {"achieved": achieved, "frac": achieved / peak,
             "launches": a["launches"], "kernel_ms": a["ms"],
             "bytes_per_launch": a["bytes"] / a["launches"],
             "gathers_per_launch": a["gathers"] / a["launches"],
             "traffic": None}
        t = traffic.get(ph)
        if t and "dram_bytes_per_gather" in t:
            # the measured launches are this workload's own (same signals and
            # draws); per gathered sample so that a different step count or
            # phase mix reads the same figure
            d["dram_bytes_per_gather"] = t["dram_bytes_per_gather"]
            d["traffic"] = t["dram_bytes_per_gather"] * d["gathers_per_launch"]
            d["algorithmic_bytes_per_gather"] = a["bytes"] / a["gathers"]
        out[ph] = d
    return out


def _event_ms(torch, stream, fn, steps: int, warmup: int) -> float:
    """Mean ms per call of fn over steps calls after warmup calls, from CUDA
    events on stream (the context's stream), synchronised on both sides."""
    for _ in range(warmup):
        fn()
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(steps):
        fn()
    e1.record(stream)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / steps


def _profiled_roofline(ctx, fn, peak: float, min_bins: int = 51) -> dict:
    """One call of fn with every binning launch timed: all-launch and
    per-phase achieved GB/s (no measured traffic)."""
    ctx.set_profiling(True)
    try:
        fn()
        recs = ctx.bin_launches()
    finally:
        ctx.set_profiling(False)
    ph = binning_roofline(recs, min_bins, peak, {})
    return {k: {kk: v[kk] for kk in ("achieved", "frac", "launches", "kernel_ms")}
            for k, v in ph.items()}


def extra_batched_fp64(torch, ctx, m, stream, sigs, sigs_host) -> dict:
    """The same 64-signal batch through the FP64 kernels (the plain path's
    arithmetic, batched): separates the batching gain from the precision
    gain."""
    opts = [solve_opts(ctx, sg.sigma, m.FP64) for sg in sigs_host]
    rngs = [m.Rng(SEED_RNG + i) for i in range(len(sigs))]

    def step():
        for i, r in enumerate(rngs):
            r.seed(SEED_RNG + i)
        return ctx.solve_batched(sigs, rngs, opts)

    ms = _event_ms(torch, stream, step, 2, 1)
    return {"value": len(sigs) / (ms / 1e3), "unit": "solves/s",
            "ms_per_step": ms, "batch": len(sigs)}


def extra_config3(torch, ctx, m, stream, peak: float) -> dict:
    """Config 3: 256 signals, N = 2^e with e uniform in 16..24, S uniform in
    [10, 2000], unit modes, sigma = 1e-6, made on the device; one batched
    solve per step. Reports the share of iterations the precision policy ran
    on the FP64 kernels."""
    from mpsft_gb300.signals import config3_spec
    specs = [config3_spec(i) for i in range(256)]
    sigs = [ctx.generate(sp.n, sp.k, sp.c, sp.sigma, sp.seed, m.C64) for sp in specs]
    opts = [ctx.solve_options(sp.k.size, sp.sigma, trials=1, min_bins=51,
                              window_delta=1e-5, window_threshold=0.1,
                              max_stale_iter=5, precision=m.FP32) for sp in specs]
    rngs = [m.Rng(SEED_RNG + i) for i in range(256)]
    last = {}

    def step():
        for i, r in enumerate(rngs):
            r.seed(SEED_RNG + i)
        last["stats"] = ctx.solve_batched(sigs, rngs, opts)[1]

    try:
        ms = _event_ms(torch, stream, step, 3, 1)
        st = last["stats"]
        iters = sum(x["iterations"] for x in st)
        fp64 = sum(x["fp64_iterations"] for x in st)
        roof = _profiled_roofline(ctx, step, peak)
    finally:
        for sg in sigs:
            sg.free()
    return {"value": 256 / (ms / 1e3), "unit": "solves/s", "ms_per_step": ms,
            "signals": 256, "samples": int(sum(sp.n for sp in specs)),
            "iterations_per_step": iters, "fp64_iterations_per_step": fp64,
            "fp64_iteration_share": fp64 / iters,
            "binning_roofline": roof.get("all")}


def extra_config5(torch, ctx, m, stream, peak: float) -> dict:
    """Config 5: N = 2^26 complex64 (512 MiB, x far beyond L2), S = 4000 with
    25% close pairs, |c| log-uniform [1e-3, 1], 40 dB, made on the device;
    one signal and a batch of four. The binning gathers from HBM: its
    achieved GB/s against the measured HBM copy rate."""
    from mpsft_gb300.signals import config5_spec
    specs = [config5_spec(5 + i) for i in range(4)]
    sigs = [ctx.generate(sp.n, sp.k, sp.c, sp.sigma, sp.seed, m.C64) for sp in specs]
    opts = [ctx.solve_options(4000, sp.sigma, trials=1, min_bins=51,
                              window_delta=1e-5, window_threshold=0.1,
                              max_stale_iter=5, precision=m.FP32) for sp in specs]
    out = {}
    try:
        for g in (1, 4):
            rngs = [m.Rng(SEED_RNG + i) for i in range(g)]

            def step(g=g, rngs=rngs):
                for i, r in enumerate(rngs):
                    r.seed(SEED_RNG + i)
                ctx.solve_batched(sigs[:g], rngs, opts[:g])

            ms = _event_ms(torch, stream, step, 2, 1)
            roof = _profiled_roofline(ctx, step, peak)
            out[f"batch{g}"] = {"value": g / (ms / 1e3), "unit": "solves/s",
                                "ms_per_step": ms, "binning_roofline": roof}
    finally:
        for sg in sigs:
            sg.free()
    return out


def extra_bm_bin_in_time(ctx, m) -> dict:
    """The reference's own binning micro-benchmark shape (BM_BinInTime,
    src/binner_bench.cc:28-53): N = 4194301, B = 501, bits = 15 (31 rows),
    delta = 1e-6; each call draws a transform and q from the RNG and bins one
    signal resident on the device, the bins returned to host memory (the
    reference's Run writes a host matrix). Published reference time: 13.18 ms
    per call (BinInTimeV4, one i7-6700K core, README.md:82)."""
    n, bins, bits, delta = 4194301, 501, 15, 1e-6
    rng = np.random.default_rng(28)
    x = (rng.standard_normal(n) + 1j * rng.standard_normal(n)).astype(np.complex128)
    out = {"config": "N=4194301 B=501 bits=15 delta=1e-6", "published_ref_ms": 13.18}
    for name, dt, prec in (("fp32_c64", np.complex64, m.FP32),
                           ("fp64_c128", np.complex128, m.FP64)):
        sig = ctx.upload(x.astype(dt))
        r = m.Rng(123534)

        def call():
            a = (r.int32() % (n - 1)) + 1
            b = r.int32() % n
            c = r.int32() % n
            q = r.int32() % n
            return ctx.bin_in_time(sig, bins, bits, delta, a, b, c, q, precision=prec)

        for _ in range(3):
            call()
        reps = 30
        t0 = time.perf_counter()
        for _ in range(reps):
            call()
        call_ms = 1e3 * (time.perf_counter() - t0) / reps
        ctx.set_profiling(True)
        kms, kbytes = [], []
        for _ in range(5):
            call()
            rec = ctx.bin_launches()[0]
            kms.append(rec["ms"])
            kbytes.append(rec["bytes"])
        ctx.set_profiling(False)
        sig.free()
        kern = statistics.median(kms)
        out[name] = {"call_ms": call_ms, "kernel_ms": kern,
                     "kernel_gb_per_s": statistics.median(kbytes) / (kern / 1e3) / 1e9,
                     "speedup_vs_published": 13.18 / call_ms}
    return out


def run_config3(args) -> None:
    """The uneven batch of config 3 as one batched solve per step (device-
    resident signals; a parity workload measured for information)."""
    import torch
    import mpsft_gb300 as m
    from mpsft_gb300.signals import config3

    torch.cuda.set_device(0)
    sigs_host = [config3(i) for i in range(256)]
    ctx = m.Context(0)
    stream = torch.cuda.Stream(device=0)
    ctx.set_stream(stream.cuda_stream)
    sigs = [ctx.upload(sg.x) for sg in sigs_host]
    opts = [ctx.solve_options(sg.k.size, sg.sigma, trials=1, min_bins=51,
                              window_delta=1e-5, window_threshold=0.1,
                              max_stale_iter=5, precision=m.FP32)
            for sg in sigs_host]
    total_n = sum(sg.n for sg in sigs_host)
    del sigs_host

    rngs = [m.Rng(SEED_RNG + i) for i in range(len(sigs))]

    def step():
        for i, r in enumerate(rngs):  # every step draws the same transforms
            r.seed(SEED_RNG + i)
        return ctx.solve_batched(sigs, rngs, opts)

    for _ in range(max(args.warmup, 3)):
        step()
    torch.cuda.synchronize()
    clocks = ClockSampler(0)
    clocks.start()
    time.sleep(0.3)
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    steps = max(1, min(args.steps, 10))
    ev0.record(stream)
    iters, fp64_its = [], 0
    for _ in range(steps):
        out, stats = step()
        iters += [s["iterations"] for s in stats]
        fp64_its += sum(s["fp64_iterations"] for s in stats)
    ev1.record(stream)
    torch.cuda.synchronize()
    clk = clocks.stop()
    ms = ev0.elapsed_time(ev1) / steps
    print(json.dumps({
        "metric": "solves/s, config 3 uneven batch (256 signals, N 2^16..2^24, "
                  "S 10..2000)",
        "value": 256 / (ms / 1e3), "unit": "solves/s", "n_gpus": 1,
        "steps": steps, "warmup": max(args.warmup, 3), "ms_per_step": ms,
        "higher_is_better": True, "dtype": "f32", "data": "synthetic",
        "config": {"workload": "config3", "signals": 256, "samples": total_n,
                   "iterations_mean": float(np.mean(iters)),
                   "fp64_iterations_per_step": fp64_its / steps},
        "clocks": clk}), flush=True)


def run_gpu(args) -> None:
    import torch
    import mpsft_gb300 as m
    from mpsft_gb300.signals import config2

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    torch.cuda.set_device(local)
    if not os.path.exists(m.LIB_PATH):
        raise SystemExit("library not built: run __graft_entry__.build() first")

    G = args.batch
    sigs_host = [config2(s) for s in rank_seeds(rank, G)]
    ctx = m.Context(local)
    stream = torch.cuda.Stream(device=local)
    ctx.set_stream(stream.cuda_stream)
    # pinned host copies for the end-to-end leg
    pinned = []
    for sg in sigs_host:
        t = torch.empty(N, dtype=torch.complex64, pin_memory=True)
        t.numpy()[:] = sg.x
        pinned.append(t)
    sigs = [ctx.upload(sg.x) for sg in sigs_host]
    opts = [solve_opts(ctx, sg.sigma, m.FP32) for sg in sigs_host]

    rngs = [m.Rng(SEED_RNG + i) for i in range(G)]

    seeds = np.arange(SEED_RNG, SEED_RNG + G, dtype=np.int32)

    def step(profile=False):
        m.Rng.seed_many(rngs, seeds)  # every step draws the same transforms
        return ctx.solve_batched(sigs, rngs, opts)

    if args.profile_case:
        ctx.set_profiling(True)
        step()
        torch.cuda.synchronize()
        # the timed binning launches of this case, for the ncu summaries
        print(json.dumps({"bin_launches": ctx.bin_launches()}), flush=True)
        return

    for _ in range(max(args.warmup, 3)):
        step()
    torch.cuda.synchronize()
    if dist:
        dist.barrier()

    # ---- device-resident timed region: solves exactly as a user runs them
    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.3)  # first nvidia-smi sample before the region starts
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    iters = []
    launches = 0
    near = 0
    loop_ms = 0.0
    for _ in range(args.steps):
        out, stats = step()
        near += sum(s["escalated"] for s in stats)
        iters += [s["iterations"] for s in stats]
        launches += stats[0]["kernel_launches"]
        loop_ms += stats[0]["loop_ms"]
    ev1.record(stream)
    torch.cuda.synchronize()
    clk = clocks.stop()
    ms_max = max_over_ranks(ev0.elapsed_time(ev1), dist, "cuda")
    value = job_rate(world, G, args.steps, ms_max)

    # ---- the same steps again with an event pair around every binning
    # launch (the host drives the iterations here); gives the binning roofline
    ctx.set_profiling(True)
    bin_records = []
    for _ in range(args.steps):
        out, stats = step()
        bin_records += ctx.bin_launches()
    torch.cuda.synchronize()
    ctx.set_profiling(False)

    # ---- end to end through the public API from pinned host buffers: every
    # step copies its G signals host -> device and reads its results back. Two
    # sets of device signals alternate so that step k+1's copies (on a copy
    # stream, issued by a second host thread) overlap step k's solve, as a
    # serving loop would run them.
    h2d = G * N * 8
    sigs_b = [ctx.upload(sg.x) for sg in sigs_host]
    sets = [sigs, sigs_b]
    copy_stream = torch.cuda.Stream(device=local)
    ready = [torch.cuda.Event(), torch.cuda.Event()]
    pinned_np = [pin.numpy() for pin in pinned]
    writer = ThreadPoolExecutor(max_workers=1)

    def write_set(j):
        ctx.write_many(sets[j], pinned_np, copy_stream.cuda_stream)
        ready[j].record(copy_stream)

    def solve_set(j):
        m.Rng.seed_many(rngs, seeds)
        return ctx.solve_batched(sets[j], rngs, opts)

    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    d2h = 0
    write_set(0)
    for s_i in range(args.steps):
        cur = s_i % 2
        stream.wait_event(ready[cur])
        pending = writer.submit(write_set, 1 - cur) if s_i + 1 < args.steps else None
        out, stats = solve_set(cur)
        d2h += sum(k.nbytes + c.nbytes for k, c in out)
        if pending is not None:
            pending.result()
    e1.record(stream)
    writer.shutdown()
    torch.cuda.synchronize()
    e2e_ms = max_over_ranks(e0.elapsed_time(e1), dist, "cuda")
    e2e_value = job_rate(world, G, args.steps, e2e_ms)
    # the link alone: one set's copies with nothing else running
    link_ms = []
    for _ in range(3):
        c0 = torch.cuda.Event(enable_timing=True)
        c1 = torch.cuda.Event(enable_timing=True)
        c0.record(copy_stream)
        ctx.write_many(sets[0], pinned_np, copy_stream.cuda_stream)
        c1.record(copy_stream)
        torch.cuda.synchronize()
        link_ms.append(c0.elapsed_time(c1))
    link_gbs = h2d / min(link_ms) / 1e6
    for sg in sigs_b:
        sg.free()

    # ---- plain per-signal FP64 path and precision error (rank 0, one signal)
    extra = {}
    if rank == 0:
        sg0 = sigs_host[0]
        o64 = solve_opts(ctx, sg0.sigma, m.FP64)
        k64, c64, _ = ctx.solve_arrays(sigs[0], m.Rng(SEED_RNG), o64)  # warm
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        reps = 3
        for _ in range(reps):
            k64, c64, st64 = ctx.solve_arrays(sigs[0], m.Rng(SEED_RNG), o64)
        torch.cuda.synchronize()
        t64 = (time.perf_counter() - t0) / reps
        k32, c32, _ = ctx.solve_arrays(sigs[0], m.Rng(SEED_RNG), opts[0])
        same = bool(np.array_equal(k32, k64))
        perr = float(np.linalg.norm(c32 - c64) / np.linalg.norm(c64)) if same else None
        extra = {"plain_fp64_gpu": {"value": 1.0 / t64, "unit": "solves/s",
                                    "ms_per_solve": 1e3 * t64,
                                    "iterations": st64.iterations},
                 "fp32_vs_fp64": {"same_frequency_set": same,
                                  "coef_precision_err": perr},
                 "accuracy": accuracy(sg0, k32, c32, k64, c64),
                 "test_data_pipeline": test_data_pipeline(ctx, m, sg0, k32, c32),
                 "dense_fft": dense_fft(torch, sigs_host, torch.device("cuda", local))}
        extra["random_gather_ceiling"] = random_gather_ceiling(
            torch, torch.device("cuda", local))
        if not args.no_extras:
            peak = load_peaks()["hbm_gbs"]
            extra["batched_fp64"] = extra_batched_fp64(torch, ctx, m, stream, sigs,
                                                       sigs_host)
            extra["batched_fp64"]["batching_gain"] = (
                extra["batched_fp64"]["value"] / extra["plain_fp64_gpu"]["value"])
            extra["config3"] = extra_config3(torch, ctx, m, stream, peak)
            extra["config5"] = extra_config5(torch, ctx, m, stream, peak)
            extra["bm_bin_in_time"] = extra_bm_bin_in_time(ctx, m)

    if rank == 0:
        peaks = load_peaks()
        phases = binning_roofline(bin_records, 51, peaks["hbm_gbs"], profile_traffic())
        ceil = extra.get("random_gather_ceiling")
        if ceil:
            # each phase's distinct gathered samples per second against the
            # measured rate of random reads
            for ph in phases.values():
                ph["gathers_per_s"] = ph["gathers_per_launch"] / (
                    ph["kernel_ms"] / ph["launches"] / 1e3)
                ph["frac_of_random_gather_ceiling"] = (ph["gathers_per_s"] /
                                                        ceil["gathers_per_s"])
        allp = phases.get("all", {})
        achieved = allp.get("achieved")
        line = {
            "metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": world,
            "steps": args.steps, "warmup": max(args.warmup, 3),
            "ms_per_step": ms_max / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": WORKLOAD, "batch_per_gpu": G,
                       "precision": "f32 gather/fold/FFT, f64 pencil+coefficients",
                       "l2": f"inputs larger than L2: {G} x 32 MiB signals resident",
                       "parallelism": f"replicas x{world}",
                       "iterations_mean": float(np.mean(iters)),
                       "near_tie_bins_per_solve": near / (G * args.steps),
                       "loop_ms_per_step": loop_ms / args.steps},
            "e2e": {"value": e2e_value, "unit": "solves/s",
                    "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": int(d2h // max(args.steps, 1)),
                    # the copies' share of the link: e2e is copy-bound when
                    # this is the host->device rate a plain copy reaches
                    "h2d_gb_per_s": h2d * args.steps / e2e_ms / 1e6,
                    "h2d_copy_alone_gb_per_s": link_gbs},
            "roofline": {"bound": "hbm", "achieved": achieved,
                         "peak": peaks["hbm_gbs"], "unit": "GB/s",
                         "frac": (achieved / peaks["hbm_gbs"]) if achieved else None,
                         "traffic": allp.get("traffic"),
                         "achieved_bytes_per_launch": allp.get("bytes_per_launch"),
                         "kernel": "k_bin_fold32 (gather/window/modulate/fold)",
                         "bytes_model": "32 B sector per gathered sample + window "
                                        "table + fold output",
                         "launches": allp.get("launches"),
                         "kernel_ms": allp.get("kernel_ms"),
                         "peak_source": peaks["source"],
                         "traffic_source": os.path.relpath(PHASE_PROFILE, ROOT),
                         "phases": {k: v for k, v in phases.items() if k != "all"}},
            "clocks": clk,
            "gpu_launches": int(launches),
        }
        line.update(extra)
        if world == 1 and not args.no_cpu_baseline:
            line["cpu_baseline"] = cpu_baseline_single(args.cpu_seconds)
        print(json.dumps(line), flush=True)
    if dist:
        dist.barrier()
        dist.destroy_process_group()


def main():
    args = parse_args()
    if args.impl == "gpu" and args.workload == "config3":
        run_config3(args)
        return
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
