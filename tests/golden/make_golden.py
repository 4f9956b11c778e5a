"""Generates tests/golden/ref_golden.npz from the reference itself.

Run in the container that holds the reference tree (the GPU machine does not):

    make -C oracle ref            # compiles the reference into oracle/_ref
    python tests/golden/make_golden.py

Every array in the archive is an output of the reference's own code
(oracle/_ref/libref*.so: jiaweichiu/mpsft src/*.cc compiled unmodified against
stand-in headers; libref_pow2.so replaces only src/integer.cc so that a is odd
for power-of-two n). Inputs are rebuilt by tests/golden/cases.py.
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)

from oracle.oracle import Oracle  # noqa: E402
import cases  # noqa: E402


PA_KEYS = ["hit", "hit_l1", "hit_l2", "miss", "miss_l1", "miss_l2", "l1", "l2",
           "max_err"]


def main() -> None:
    ref = Oracle("ref")
    ref2 = Oracle("ref_pow2")
    out: dict[str, np.ndarray] = {}

    # RNG: the first draws after MainInit's seed and after the tests' seed.
    ref.seed(123534)
    out["rng_123534"] = np.array([ref.random_int32() for _ in range(16)], np.int32)
    ref2.seed(123537)
    out["transform_pow2_123537"] = np.array(
        [ref2.transform(1 << 20) for _ in range(4)], np.int32)
    ref.seed(123537)
    out["transform_prime_123537"] = np.array(
        [ref.transform(1048573) for _ in range(4)], np.int32)

    # Window.
    out["window_1109_5_1e-6"] = ref.window(1109, 5, 1e-6)
    out["window_p"] = np.array([
        len(ref.window(1 << 22, 2001, 1e-5)), len(ref.window(1 << 20, 101, 1e-6)),
        len(ref.window(4099, 11, 1e-6))], np.int32)
    xis = np.linspace(-0.02, 0.02, 41)
    out["window_freq_xi"] = xis
    out["window_freq_2001_1e-5"] = np.array(
        [ref.sample_in_freq(1 << 22, 2001, 1e-5, float(v)) for v in xis])

    # Known-answer binning (src/binner_test.cc:54-103).
    kc = cases.KNOWN
    x = cases.evaluate_modes(kc["n"], kc["modes"])
    args = (kc["bins"], kc["bits"], kc["delta"], kc["a"], kc["b"], kc["c"], kc["q"])
    out["known_v4"] = ref.bin_in_time(x, *args, btype=4)
    out["known_v0"] = ref.bin_in_time(x, *args, btype=0)
    zeros = np.zeros_like(out["known_v4"])
    ks = np.array(list(kc["modes"].keys()), np.int32)
    cs = np.array(list(kc["modes"].values()), np.complex128)
    out["known_freq"] = ref.bin_in_freq(zeros, kc["n"], kc["bins"], kc["bits"],
                                        kc["delta"], kc["a"], kc["b"], kc["c"],
                                        kc["q"], ks, cs)

    # Large-n overflow case (src/binner_test.cc:112-143).
    bc = cases.BIGGER
    x = cases.evaluate_modes(bc["n"], bc["modes"])
    args = (bc["bins"], bc["bits"], bc["delta"], bc["a"], bc["b"], bc["c"], bc["q"])
    out["bigger_v4"] = ref.bin_in_time(x, *args, btype=4)
    ks = np.array(list(bc["modes"].keys()), np.int32)
    cs = np.array(list(bc["modes"].values()), np.complex128)
    out["bigger_freq"] = ref.bin_in_freq(np.zeros_like(out["bigger_v4"]), bc["n"],
                                         bc["bins"], bc["bits"], bc["delta"],
                                         bc["a"], bc["b"], bc["c"], bc["q"], ks, cs)

    # Random signals: bins, then BinInFreq of 12 modes on top.
    for name, n, bins, delta, a, b, c, q, seed in cases.RANDOM_BINS:
        lib = ref2 if (n & (n - 1)) == 0 else ref
        x = cases.random_signal(n, seed)
        bits = lib.num_bits(n, bins)
        u = lib.bin_in_time(x, bins, bits, delta, a, b, c, q, btype=4)
        out[f"rb_{name}"] = u
        rng = np.random.default_rng(seed + 1000)
        mk = np.unique(rng.integers(0, n, 12)).astype(np.int32)
        mc = rng.standard_normal(mk.size) + 1j * rng.standard_normal(mk.size)
        out[f"rf_{name}_k"] = mk
        out[f"rf_{name}_c"] = mc
        out[f"rf_{name}"] = lib.bin_in_freq(u, n, bins, bits, delta, a, b, c, q,
                                            mk, mc)

    # Iterate twice on a solve signal (trials 3, thresholds as Demo1 sets them).
    case = cases.SOLVES[2]
    x, sigma = cases.solve_signal(case)
    n = case[1]
    ref2.seed(4242)
    mm: dict = {}
    for i, bins in enumerate((401, 201)):
        found, mm = ref2.iterate(x, bins, window_delta=1e-5, trials=3,
                                 bin_threshold=3 * sigma / np.sqrt(bins),
                                 window_threshold=0.1,
                                 sv_threshold=sigma / np.sqrt(bins), mm=mm)
        kk = np.array(sorted(mm), np.int32)
        out[f"iter{i}_k"] = kk
        out[f"iter{i}_c"] = np.array([mm[k] for k in kk], np.complex128)
        out[f"iter{i}_found"] = np.array([found], np.int32)

    # Full Demo1::Run solves.
    for case in cases.SOLVES:
        name, n, s, _, trials, min_bins, delta, _, rseed, _ = case
        x, sigma = cases.solve_signal(case)
        lib = ref2 if (n & (n - 1)) == 0 else ref
        modes, _ = lib.demo1_run(np.asarray(x, np.complex128), s, sigma, rseed,
                                 trials=trials, min_bins=min_bins,
                                 window_delta=delta, window_threshold=0.1,
                                 max_stale_iter=5)
        kk = np.array(sorted(modes), np.int32)
        out[f"solve_{name}_k"] = kk
        out[f"solve_{name}_c"] = np.array([modes[k] for k in kk], np.complex128)
        out[f"solve_{name}_sigma"] = np.array([sigma])

    # GenerateModeMap and Demo1::PostAnalyze.
    for i, (n, k, seed) in enumerate(cases.MODE_MAPS):
        kk, cc = ref.generate_mode_map(n, k, seed)
        out[f"mm{i}_k"] = kk
        out[f"mm{i}_c"] = cc
    for case in cases.POST_ANALYZE:
        xh, tk, fk, fc = cases.post_analyze_inputs(case)
        r = ref.post_analyze(xh, tk, fk, fc)
        out[f"pa_{case[0]}"] = np.array([r[k] for k in PA_KEYS], np.float64)

    # The reference's statistical Iterate scenarios: (good, bad) per call.
    # (n = kPrimes[20] is prime: the reference's own Transform)
    for name, spec in (("more", cases.ITERATE_MORE), ("full", cases.ITERATE_FULL)):
        counts, _ = cases.iterate_stats(ref, spec)
        out[f"iterstats_{name}"] = np.array(counts, np.int32)

    path = os.path.join(HERE, "ref_golden.npz")
    np.savez_compressed(path, **out)
    print(f"wrote {path}: {len(out)} arrays, {os.path.getsize(path)} bytes")


if __name__ == "__main__":
    main()
