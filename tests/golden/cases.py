"""Inputs of the golden cases, regenerated deterministically on any host.

The outputs for these inputs were produced by the reference itself
(jiaweichiu/mpsft sources compiled against the oracle's stand-in headers, see
oracle/Makefile) and stored in ref_golden.npz by make_golden.py. Signals are
not stored: they are rebuilt here from closed-form modes or numpy PCG64 seeds.
"""
from __future__ import annotations

import numpy as np

from mpsft_gb300.signals import make_signal


def as_i32(v: int) -> int:
    """C++ int32_t conversion of an integer literal (wraps like the reference's
    Transform(n, 0x3FFFFFFF, 0xEEEEEEEE, 0xDDDDDD), src/binner_test.cc:124)."""
    return int(np.array(v & 0xFFFFFFFF, np.uint32).astype(np.int32))


def evaluate_modes(n: int, modes: dict) -> np.ndarray:
    """EvaluateModes (src/gen.cc:41-53): x_t = sum c e^{2 pi i (k t mod n)/n}."""
    t = np.arange(n, dtype=np.int64)
    x = np.zeros(n, np.complex128)
    for k, c in modes.items():
        ang = 2.0 * np.pi * (((k * t) % n).astype(np.float64) / n)
        x += c * (np.cos(ang) + 1j * np.sin(ang))
    return x


# Known-answer binning case of src/binner_test.cc:54-103.
KNOWN = dict(n=1109, bins=5, bits=2, q=106, a=3, b=847, c=45, delta=1e-6,
             modes={550: 2.0 + 0.0j})
# Large-n overflow case of src/binner_test.cc:112-143 (q = 0xFFFFFF).
BIGGER = dict(n=1048573, bins=5, bits=2, q=0xFFFFFF, a=0x3FFFFFFF,
              b=as_i32(0xEEEEEEEE), c=0xDDDDDD, delta=1e-6,
              modes={565336: 2.0 + 1.0j})

# Random-signal binning cases: (name, n, bins, delta, a, b, c, q, seed).
RANDOM_BINS = [
    ("pow2_b101", 1 << 16, 101, 1e-5, 12345, 678, 910, 4444, 11),
    ("prime_b101", 65537, 101, 1e-5, 12345, 678, 910, 4444, 12),
    ("pow2_b2001", 1 << 20, 2001, 1e-5, 987653, 31337, 271828, 99991, 13),
    ("prime_b51", 1048573, 51, 1e-6, 76543, 5, 123456, 1000003, 14),
]

# Solve cases: (name, n, S, sigma, trials, min_bins, delta, seed_signal,
# seed_rng, magnitude).
SOLVES = [
    ("pow2_s50", 1 << 16, 50, 1e-6, 1, 51, 1e-5, 21, 123537, "unit"),
    ("prime_s50", 65537, 50, 1e-6, 1, 51, 1e-5, 22, 123537, "unit"),
    ("pow2_s200_t3", 1 << 18, 200, 1e-3, 3, 51, 1e-5, 23, 123537, "unit"),
    ("config1", 1 << 20, 50, 1e-6, 1, 51, 1e-5, 1, 123537, "unit"),
    ("pow2_s300_logu", 1 << 20, 300, None, 1, 51, 1e-5, 24, 123537, "loguniform"),
    ("prime_s120_t5", 65537, 120, 1e-4, 5, 51, 1e-5, 25, 123537, "unit"),
]


def random_signal(n: int, seed: int) -> np.ndarray:
    rng = np.random.default_rng(seed)
    v = rng.standard_normal((2, n))
    return v[0] + 1j * v[1]


def solve_signal(case) -> tuple[np.ndarray, float]:
    name, n, s, sigma, trials, min_bins, delta, sseed, rseed, mag = case
    if mag == "unit":
        sig = make_signal(n, s, sseed, sigma=sigma, dtype=np.complex128)
    else:
        sig = make_signal(n, s, sseed, magnitude="loguniform", snr_db=60.0,
                          dtype=np.complex64)
    return sig.x, sig.sigma


# GenerateModeMap cases (src/gen.cc:27-39): (n, k, seed of RandomSeed).
MODE_MAPS = [(1 << 20, 50, 123534), (65537, 300, 5), (1009, 1000, 77)]

# PostAnalyze cases (src/demo1.cc:61-112): (name, n, seed, true count,
# found true count, found false count, error scale of the found coefficients).
POST_ANALYZE = [
    ("mixed", 4099, 3, 60, 50, 7, 0.01),
    ("no_miss", 1 << 12, 4, 40, 40, 0, 1e-3),
    ("far_off", 1 << 13, 5, 30, 10, 20, 10.0),
]


def post_analyze_inputs(case):
    """(xh, true positions, found positions, found coefficients) of a case."""
    _, n, seed, nt, nhit, nmiss, scale = case
    rng = np.random.default_rng(seed)
    xh = (rng.standard_normal(n) + 1j * rng.standard_normal(n)) / np.sqrt(2 * n)
    tk = rng.choice(n, nt, replace=False)
    xh[tk] += np.exp(2j * np.pi * rng.uniform(size=nt))
    others = np.setdiff1d(np.arange(n), tk)
    fk = np.concatenate([tk[:nhit], rng.choice(others, nmiss, replace=False)])
    fc = xh[fk] + scale * (rng.standard_normal(fk.size)
                           + 1j * rng.standard_normal(fk.size))
    return xh, tk.astype(np.int32), fk.astype(np.int32), fc


# The reference's statistical Iterate tests (src/iterate_test.cc:84-175): n =
# kPrimes[20], 1000 unit modes, GenerateXhat noise, RandomSeed(123537) before
# the signal is built, trials = 3, window_delta = 1e-6, window_threshold = 0.1.
# IterateMore: sigma = 1e-2, bin_threshold = 0.01, bins 2001 then 1401.
# IterateFull: sigma = 1e-7, thresholds 3 sigma / sqrt(bins) and
# sigma / sqrt(bins), bins 2001 four times. Each step's REQUIREs: at least
# `good` true modes found, at most `bad` others.
ITERATE_STATS_N = 1048573
ITERATE_MORE = dict(sigma=1e-2, bins=[2001, 1401], good=[300, 600], bad=[100, 100])
ITERATE_FULL = dict(sigma=1e-7, bins=[2001] * 4, good=[250, 450, 600, 700], bad=[30] * 4)


def iterate_stats(oracle, spec):
    """Runs one of the reference's statistical scenarios on an oracle:
    [(good, bad)] after each Iterate call, and the final mode map."""
    x, k, _ = oracle.demo_signal(ITERATE_STATS_N, 1000, spec["sigma"], 123537)
    truth = set(k.tolist())
    sigma = spec["sigma"]
    mm, out = {}, []
    for bins in spec["bins"]:
        if spec is ITERATE_FULL:
            kw = dict(bin_threshold=3 * sigma / np.sqrt(bins),
                      sv_threshold=sigma / np.sqrt(bins))
        else:
            kw = dict(bin_threshold=0.01)
        _, mm = oracle.iterate(x, bins, window_delta=1e-6, trials=3,
                               window_threshold=0.1, mm=mm, **kw)
        good = sum(1 for kk in mm if kk in truth)
        out.append((good, len(mm) - good))
    return out, mm

