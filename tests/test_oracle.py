"""Pins the CPU oracle (oracle/mpsft_oracle.cc) before it is trusted.

1. Against the known-answer values written in the reference's own tests
   (src/binner_test.cc, src/freqid_test.cc, src/window_test.cc).
2. Against outputs of the reference itself (tests/golden/ref_golden.npz,
   made by tests/golden/make_golden.py from oracle/_ref).
3. Where oracle/_ref is built on this host, bit for bit against it on extra
   cases.
"""
from __future__ import annotations

import numpy as np
import pytest

import cases
from oracle import oracle as orc

# Catch's Approx: |a - b| < eps * (1 + max(|a|, |b|)), eps = 100 * FLT_EPSILON
# (src/catch.hpp:2842-2875).
CATCH_EPS = 100 * np.finfo(np.float32).eps


def approx(a, b):
    return abs(a - b) < CATCH_EPS * (1.0 + max(abs(a), abs(b)))


def close(a, b, rel=1e-12):
    a = np.asarray(a)
    b = np.asarray(b)
    scale = max(np.abs(b).max(), 1e-300)
    return np.abs(a - b).max() <= rel * scale


# ---------------------------------------------------------------- literals
PENCIL_CASES = [  # src/freqid_test.cc:26-59
    ((-2.3 + 5.2j, -5.5 - 3.1j, 4.0 + 3.0j), 11.34419934, 0.91057194, False),
    ((2.3 + 5.2j, 5.5 - 3.1j, 4.0 + 3.0j), 9.80673965, 5.77476038, True),
    ((-15.3 - 5.2j, 8.0 + 3.0j, -1.5 + 3.5j), 21.27794592, 12.53032391, False),
]


@pytest.mark.parametrize("u,s0,s1,vote", PENCIL_CASES)
def test_pencil_known_answers(port, u, s0, s1, vote):
    g0, g1, gv = port.mat_pencil(*u)
    assert approx(g0, s0) and approx(g1, s1) and gv == vote


@pytest.mark.parametrize("btype", [0, 4])
def test_binner_known_answer(port, btype):
    """src/binner_test.cc:54-103: U0[1] = 1.12652 - 0.108838i, other bins of
    row 0 ~ 0, and BinInFreq gives exactly the negative, every row."""
    kc = cases.KNOWN
    x = cases.evaluate_modes(kc["n"], kc["modes"])
    args = (kc["bins"], kc["bits"], kc["delta"], kc["a"], kc["b"], kc["c"], kc["q"])
    u = port.bin_in_time(x, *args, btype=btype)
    assert approx(u[0, 1].real, 1.12652) and approx(u[0, 1].imag, -0.108838)
    for i in range(kc["bins"]):
        if i != 1:
            assert approx(abs(u[0, i]), 0.0)
    ks = np.array(list(kc["modes"]), np.int32)
    cs = np.array(list(kc["modes"].values()))
    f = port.bin_in_freq(np.zeros_like(u), kc["n"], kc["bins"], kc["bits"],
                         kc["delta"], kc["a"], kc["b"], kc["c"], kc["q"], ks, cs)
    assert approx(f[0, 1].real, -1.12652) and approx(f[0, 1].imag, 0.108838)
    assert all(approx(abs(v), 0.0) for v in (u + f).ravel())


def test_binner_versions_match(port):
    """src/binner_test.cc:28-51: V0 == V4 on bins = 1, bits = 2."""
    n = 1109
    x = cases.evaluate_modes(n, {500: 1.0})
    u0 = port.bin_in_time(x, 1, 2, 1e-6, 1, 0, 0, 100, btype=0)
    u4 = port.bin_in_time(x, 1, 2, 1e-6, 1, 0, 0, 100, btype=4)
    assert all(approx(abs(v), 0.0) for v in (u0 - u4).ravel())


def test_time_freq_duality_bigger(port):
    """src/binner_test.cc:112-143 with the int32-wrapped transform."""
    bc = cases.BIGGER
    x = cases.evaluate_modes(bc["n"], bc["modes"])
    args = (bc["bins"], bc["bits"], bc["delta"], bc["a"], bc["b"], bc["c"], bc["q"])
    u = port.bin_in_time(x, *args)
    ks = np.array(list(bc["modes"]), np.int32)
    cs = np.array(list(bc["modes"].values()))
    f = port.bin_in_freq(np.zeros_like(u), bc["n"], bc["bins"], bc["bits"],
                         bc["delta"], bc["a"], bc["b"], bc["c"], bc["q"], ks, cs)
    assert all(approx(abs(v), 0.0) for v in (u[0] + f[0]))


def test_window_properties(port):
    """src/window_test.cc:29-78: symmetric, FFT ~ 1 near 0, < delta beyond
    n/(2 bins), and equal to SampleInFreq."""
    n, bins, delta = 1109, 5, 1e-6
    wt = port.window(n, bins, delta)
    p = wt.size
    p2 = (p - 1) // 2
    for i in range(1, p2 + 1):
        assert approx(wt[i], wt[p - i])
    a = np.zeros(n)
    a[0] = wt[0]
    a[1:p2 + 1] = wt[1:p2 + 1]
    a[n - p2:] = wt[1:p2 + 1][::-1]
    ah = np.fft.fft(a)
    assert np.all(np.abs(ah.imag) < CATCH_EPS)
    for i in (0, 1, n - 1, 2, n - 2):
        assert approx(ah[i].real, 1.0)
    w = n // (2 * bins)
    assert np.all(np.abs(ah[w:n - w].real) < delta)
    for i in range(0, (n - 1) // 2 + 1, 7):
        xi = i / n
        assert approx(port.sample_in_freq(n, bins, delta, xi), ah[i].real)
        assert approx(port.sample_in_freq(n, bins, delta, -xi), ah[(n - i) % n].real)


def test_transform_inverse(port):
    """src/integer_test.cc:33-50: a * a_inv = 1 mod a prime (and 2^k)."""
    n = 536870909
    assert (10000000 * port.transform_inverse(n, 10000000)) % n == 1
    port.seed(5)
    for _ in range(2000):
        a, b, c, ainv = port.transform(n)
        assert 1 <= a < n and (a * ainv) % n == 1
    for _ in range(2000):
        a, b, c, ainv = port.transform(1 << 22)
        assert a % 2 == 1 and (a * ainv) % (1 << 22) == 1


# ------------------------------------------------------- vs the reference
def test_rng_matches_reference(port, golden):
    port.seed(123534)
    assert [port.random_int32() for _ in range(16)] == golden["rng_123534"].tolist()
    port.seed(123537)
    got = [port.transform(1 << 20) for _ in range(4)]
    assert np.array_equal(np.array(got), golden["transform_pow2_123537"])
    port.seed(123537)
    got = [port.transform(1048573) for _ in range(4)]
    assert np.array_equal(np.array(got), golden["transform_prime_123537"])


def test_window_matches_reference(port, golden):
    assert close(port.window(1109, 5, 1e-6), golden["window_1109_5_1e-6"], 1e-15)
    ps = [len(port.window(1 << 22, 2001, 1e-5)), len(port.window(1 << 20, 101, 1e-6)),
          len(port.window(4099, 11, 1e-6))]
    assert ps == golden["window_p"].tolist()
    got = [port.sample_in_freq(1 << 22, 2001, 1e-5, float(v))
           for v in golden["window_freq_xi"]]
    assert close(got, golden["window_freq_2001_1e-5"], 1e-14)


def test_known_and_bigger_match_reference(port, golden):
    kc = cases.KNOWN
    x = cases.evaluate_modes(kc["n"], kc["modes"])
    args = (kc["bins"], kc["bits"], kc["delta"], kc["a"], kc["b"], kc["c"], kc["q"])
    assert close(port.bin_in_time(x, *args, btype=4), golden["known_v4"])
    assert close(port.bin_in_time(x, *args, btype=0), golden["known_v0"])
    bc = cases.BIGGER
    x = cases.evaluate_modes(bc["n"], bc["modes"])
    args = (bc["bins"], bc["bits"], bc["delta"], bc["a"], bc["b"], bc["c"], bc["q"])
    assert close(port.bin_in_time(x, *args), golden["bigger_v4"], 1e-11)


@pytest.mark.parametrize("case", cases.RANDOM_BINS, ids=[c[0] for c in cases.RANDOM_BINS])
def test_random_bins_match_reference(port, golden, case):
    name, n, bins, delta, a, b, c, q, seed = case
    x = cases.random_signal(n, seed)
    bits = port.num_bits(n, bins)
    u = port.bin_in_time(x, bins, bits, delta, a, b, c, q)
    assert close(u, golden[f"rb_{name}"])
    f = port.bin_in_freq(golden[f"rb_{name}"], n, bins, bits, delta, a, b, c, q,
                         golden[f"rf_{name}_k"], golden[f"rf_{name}_c"])
    assert close(f, golden[f"rf_{name}"])


def test_iterate_matches_reference(port, golden):
    case = cases.SOLVES[2]
    x, sigma = cases.solve_signal(case)
    port.seed(4242)
    mm: dict = {}
    for i, bins in enumerate((401, 201)):
        found, mm = port.iterate(x, bins, window_delta=1e-5, trials=3,
                                 bin_threshold=3 * sigma / np.sqrt(bins),
                                 window_threshold=0.1,
                                 sv_threshold=sigma / np.sqrt(bins), mm=mm)
        kk = np.array(sorted(mm), np.int32)
        assert np.array_equal(kk, golden[f"iter{i}_k"])
        assert close([mm[k] for k in kk], golden[f"iter{i}_c"], 1e-11)
        assert int(found) == int(golden[f"iter{i}_found"][0])


@pytest.mark.parametrize("case", cases.SOLVES, ids=[c[0] for c in cases.SOLVES])
def test_solve_matches_reference(port, golden, case):
    name, n, s, _, trials, min_bins, delta, _, rseed, _ = case
    x, sigma = cases.solve_signal(case)
    modes, iters = port.demo1_run(np.asarray(x, np.complex128), s, sigma, rseed,
                                  trials=trials, min_bins=min_bins,
                                  window_delta=delta, window_threshold=0.1,
                                  max_stale_iter=5)
    kk = np.array(sorted(modes), np.int32)
    assert np.array_equal(kk, golden[f"solve_{name}_k"])
    assert close([modes[k] for k in kk], golden[f"solve_{name}_c"], 1e-10)
    assert iters > 0


@pytest.mark.skipif(not orc.available("ref_pow2"),
                    reason="oracle/_ref is built only where the reference tree is")
@pytest.mark.parametrize("seed", [1, 2, 3])
def test_port_bit_exact_vs_reference_here(port, seed):
    ref = orc.Oracle("ref_pow2")
    rng = np.random.default_rng(seed)
    n = int(rng.choice([1 << 14, 1 << 17, 32771]))
    bins = int(rng.choice([51, 101, 301, 1001]))
    x = cases.random_signal(n, seed + 50)
    bits = port.num_bits(n, bins)
    a, b, c, q = (int(v) for v in rng.integers(1, n, 4))
    a |= 1
    assert np.array_equal(port.bin_in_time(x, bins, bits, 1e-5, a, b, c, q),
                          ref.bin_in_time(x, bins, bits, 1e-5, a, b, c, q))


# ------------------------------------------- test data and analysis (gen, demo1)
@pytest.mark.parametrize("i", range(len(cases.MODE_MAPS)))
def test_mode_map_matches_reference(port, golden, i):
    """GenerateModeMap (src/gen.cc:27-39): same positions and coefficients."""
    n, k, seed = cases.MODE_MAPS[i]
    kk, cc = port.generate_mode_map(n, k, seed)
    assert np.array_equal(kk, golden[f"mm{i}_k"])
    assert np.array_equal(cc, golden[f"mm{i}_c"])
    assert np.allclose(np.abs(cc), 1.0, rtol=0, atol=1e-15)


PA_KEYS = ["hit", "hit_l1", "hit_l2", "miss", "miss_l1", "miss_l2", "l1", "l2",
           "max_err"]


@pytest.mark.parametrize("case", cases.POST_ANALYZE, ids=[c[0] for c in cases.POST_ANALYZE])
def test_post_analyze_matches_reference(port, golden, case):
    """Demo1::PostAnalyze (src/demo1.cc:61-112): counts equal, errors within
    1e-12 relative (summation order differs); no misses gives NaN as the
    reference's 0/0 does."""
    xh, tk, fk, fc = cases.post_analyze_inputs(case)
    got = port.post_analyze(xh, tk, fk, fc)
    want = golden[f"pa_{case[0]}"]
    for j, key in enumerate(PA_KEYS):
        if np.isnan(want[j]):
            assert np.isnan(got[key]), key
        else:
            assert abs(got[key] - want[j]) <= 1e-12 * abs(want[j]), key


# ------------------------------- the reference's statistical Iterate tests
@pytest.mark.parametrize("name", ["more", "full"])
def test_iterate_statistics_match_reference(port, golden, name):
    """IterateMore / IterateFull (src/iterate_test.cc:84-175): Demo1's signal
    construction (GenerateModeMap, GenerateXhat, backward FFT) from
    RandomSeed(123537), then Iterate calls continuing the same draw stream.
    The port finds exactly the reference's counts after every call, and they
    meet the reference test's own bounds."""
    spec = cases.ITERATE_MORE if name == "more" else cases.ITERATE_FULL
    counts, mm = cases.iterate_stats(port, spec)
    assert np.array_equal(np.array(counts, np.int32), golden[f"iterstats_{name}"])
    for (good, bad), lo, hi in zip(counts, spec["good"], spec["bad"]):
        assert good >= lo and bad <= hi
    if orc.available("ref"):
        _, ref_mm = cases.iterate_stats(orc.Oracle("ref"), spec)
        assert sorted(mm) == sorted(ref_mm)


def test_demo_signal_matches_reference_here():
    """Demo1's signal construction in the port equals the reference's bit for
    bit (both noise forms), where the reference is built on this host."""
    if not orc.available("ref"):
        pytest.skip("oracle/_ref is built only where the reference tree is")
    ref, port = orc.Oracle("ref"), orc.Oracle("port")
    for alt in (False, True):
        a = ref.demo_signal(65537, 50, 1e-3, 11, alt)
        b = port.demo_signal(65537, 50, 1e-3, 11, alt)
        for u, v in zip(a, b):
            assert np.array_equal(u, v)
