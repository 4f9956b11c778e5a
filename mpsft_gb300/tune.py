"""Autotunes the FP32 binning's launch shape on this GPU for the benchmark
workloads and writes the table that contexts load (mpsft_gb300/tuning/):

    python -m mpsft_gb300.tune [--out PATH]

Workloads (seeded synthetic signals, made on the device): the headline batch
of 64 signals N = 2^22, S = 1000, 60 dB (and 16 and 1 of them); the uneven
batch of 256 signals (N 2^16..2^24, S 10..2000; unit modes, sigma = 1e-6);
the N = 2^26 stress signal alone and four at a time. Each is solved once per
shape and repeat with every binning launch timed (mpsft_autotune).
"""
from __future__ import annotations

import argparse
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))

import mpsft_gb300 as m  # noqa: E402
from mpsft_gb300.signals import (config3_spec, config5_spec,  # noqa: E402
                                 distinct_positions)


def _opts(ctx, k, sigma):
    return ctx.solve_options(k, sigma, trials=1, min_bins=51, window_delta=1e-5,
                             window_threshold=0.1, max_stale_iter=5,
                             precision=m.FP32)


def _config2_sigs(ctx, count):
    """Config-2-shaped signals generated on the device."""
    sigs, opts = [], []
    for i in range(count):
        rng = np.random.default_rng(5000 + i)
        n, s = 1 << 22, 1000
        k = distinct_positions(rng, n, s)
        mag = np.exp(rng.uniform(np.log(1e-2), 0.0, s))
        c = mag * np.exp(2j * np.pi * rng.uniform(size=s))
        sigma = float(1e-3 * np.sqrt(np.sum(mag ** 2)))
        sigs.append(ctx.generate(n, k, c, sigma, 5000 + i, m.C64))
        opts.append(_opts(ctx, s, sigma))
    return sigs, opts


def main() -> None:
    p = argparse.ArgumentParser()
    p.add_argument("--out", default=m.TUNING_PATH)
    p.add_argument("--repeats", type=int, default=2)
    args = p.parse_args()
    os.environ["MPSFT_TUNING_FILE"] = "none"  # start from an empty table
    ctx = m.Context(0)
    for count in (64, 16, 1):
        sigs, opts = _config2_sigs(ctx, count)
        ctx.autotune(sigs, opts, repeats=args.repeats)
        for sg in sigs:
            sg.free()
    specs = [config3_spec(i) for i in range(256)]
    sigs = [ctx.generate(sp.n, sp.k, sp.c, sp.sigma, sp.seed, m.C64) for sp in specs]
    ctx.autotune(sigs, [_opts(ctx, sp.k.size, sp.sigma) for sp in specs],
                 repeats=args.repeats)
    for sg in sigs:
        sg.free()
    for count in (1, 4):
        specs = [config5_spec(5 + i) for i in range(count)]
        sigs = [ctx.generate(sp.n, sp.k, sp.c, sp.sigma, sp.seed, m.C64) for sp in specs]
        ctx.autotune(sigs, [_opts(ctx, 4000, sp.sigma) for sp in specs],
                     repeats=args.repeats)
        for sg in sigs:
            sg.free()
    os.makedirs(os.path.dirname(os.path.abspath(args.out)), exist_ok=True)
    ctx.tuning_save(args.out)
    print(open(args.out).read())
    ctx.close()


if __name__ == "__main__":
    main()
