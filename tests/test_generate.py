"""Device test data and result analysis: mpsft_signal_generate,
mpsft_signal_spectrum and mpsft_post_analyze (Demo1's constructor and
PostAnalyze, src/demo1.cc:27-34 and 61-112; GenerateXhatAlt, src/gen.cc:77-89).

Checkers: oracle/gen.py (numpy restatement of the generator), numpy's FP64
FFT, and the reference's own PostAnalyze through the golden vectors.
Tolerances: samples and spectra within 1e-12 of the largest magnitude (FP64,
different FFT summation orders); complex64 samples within 2^-24 relative;
PostAnalyze figures within 1e-9 relative (the device takes the spectrum of
x = n ifft(xh) instead of xh itself).
"""
from __future__ import annotations

import numpy as np
import pytest

import cases
import mpsft_gb300 as m
from oracle import gen

PA_KEYS = ["hit", "hit_l1", "hit_l2", "miss", "miss_l1", "miss_l2", "l1", "l2",
           "max_err"]


# ------------------------------------------------------------- CPU: the checker
def test_counter_form_equals_sequential_splitmix64():
    """Output i computed directly equals the i-th step of the sequential
    generator (state += gamma, then the mix)."""
    mask = 2**64 - 1
    seed = 0x1234_5678_9ABC_DEF0
    state, seq = seed, []
    for _ in range(40):
        state = (state + 0x9E3779B97F4A7C15) & mask
        z = state
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & mask
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & mask
        seq.append(z ^ (z >> 31))
    got = gen.splitmix64(seed, np.arange(40, dtype=np.uint64))
    assert [int(v) for v in got] == seq


def test_restated_noise_has_the_reference_distribution():
    """GenerateXhatAlt's noise (src/gen.cc:77-89) has per-sample time-domain
    variance sigma^2 split evenly between real and imaginary parts
    (src/gen_test.cc:54-70 checks the same energy in the frequency domain)."""
    n, sigma = 1 << 20, 8.0
    z = gen.noise(n, sigma, 42)
    assert abs(np.mean(np.abs(z) ** 2) / sigma**2 - 1) < 0.01
    assert abs(np.var(z.real) / (sigma**2 / 2) - 1) < 0.01
    assert abs(np.var(z.imag) / (sigma**2 / 2) - 1) < 0.01
    assert abs(np.mean(z.real * z.imag)) < 0.01 * sigma**2
    assert abs(np.mean(z)) < 5 * sigma / np.sqrt(n)


# ------------------------------------------------------------- GPU
@pytest.mark.gpu
@pytest.mark.parametrize("dtype", [m.C128, m.C64], ids=["c128", "c64"])
@pytest.mark.parametrize("n", [1 << 16, 65537])
def test_generate_matches_restatement(ctx, n, dtype):
    k, c = m.Rng(123534).mode_map(n, 40)
    c = c * np.exp(np.linspace(0.0, -3.0, c.size))
    sigma, seed = 1e-3, 0xDEADBEEF
    sig = ctx.generate(n, k, c, sigma, seed, dtype)
    got = sig.read().astype(np.complex128)
    want = gen.generate(n, k, c, sigma, seed)
    scale = np.abs(want).max()
    tol = 1e-12 if dtype == m.C128 else 2.0**-24
    assert np.abs(got - want).max() <= tol * scale * (1 if dtype == m.C128 else 2)
    # noiseless: exactly the modes' backward transform
    sig0 = ctx.generate(n, k, c, 0.0, seed, dtype)
    got0 = sig0.read().astype(np.complex128)
    want0 = gen.modes(n, k, c)
    assert np.abs(got0 - want0).max() <= tol * np.abs(want0).max() * \
        (1 if dtype == m.C128 else 2)
    sig.free()
    sig0.free()


@pytest.mark.gpu
def test_generate_statistics_and_seeds(ctx):
    """GenerateXhatBasic / GenerateXhatAltBasic (src/gen_test.cc:40-70):
    noise energy sigma^2 per sample in time, sigma^2 in total over the
    spectrum; the seed alone selects the noise."""
    n, sigma = 1 << 20, 5.5
    a = ctx.generate(n, [], [], sigma, 1, m.C128)
    xa = a.read()
    assert abs(np.sqrt(np.mean(np.abs(xa) ** 2)) / sigma - 1) < 0.005
    xh = ctx.spectrum(a)
    assert abs(np.sum(np.abs(xh) ** 2) / sigma**2 - 1) < 0.01
    assert np.array_equal(ctx.generate(n, [], [], sigma, 1, m.C128).read(), xa)
    xb = ctx.generate(n, [], [], sigma, 2, m.C128).read()
    assert np.abs(np.corrcoef(xa.real, xb.real)[0, 1]) < 0.01


@pytest.mark.gpu
@pytest.mark.parametrize("dtype", [m.C128, m.C64], ids=["c128", "c64"])
@pytest.mark.parametrize("n", [1 << 18, 65537, 1048573])
def test_spectrum_matches_numpy(ctx, n, dtype):
    x = cases.random_signal(n, 11)
    if dtype == m.C64:
        x = x.astype(np.complex64)
    sig = ctx.upload(x)
    got = ctx.spectrum(sig)
    want = np.fft.fft(x.astype(np.complex128)) / n
    assert np.abs(got - want).max() <= 1e-12 * np.abs(want).max()
    sig.free()


@pytest.mark.gpu
@pytest.mark.parametrize("case", cases.POST_ANALYZE, ids=[c[0] for c in cases.POST_ANALYZE])
def test_post_analyze_matches_reference(ctx, golden, case):
    xh, tk, fk, fc = cases.post_analyze_inputs(case)
    n = xh.size
    sig = ctx.upload(np.fft.ifft(xh) * n)
    got = ctx.post_analyze(sig, tk, fk, fc)
    want = golden[f"pa_{case[0]}"]
    for j, key in enumerate(PA_KEYS):
        if np.isnan(want[j]):
            assert np.isnan(got[key]), key
        else:
            assert abs(got[key] - want[j]) <= 1e-9 * abs(want[j]), (key, got[key], want[j])
    sig.free()


@pytest.mark.gpu
def test_generate_solve_analyze_on_device(ctx, port):
    """The test-data pipeline end to end on the device: a config-2-shaped
    signal generated there, recovered by the FP32 solve, analysed there; the
    analysis equals the oracle's PostAnalyze on the host spectrum."""
    n, s = 1 << 22, 1000
    rng = np.random.default_rng(5)
    k, c = m.Rng(123534).mode_map(n, s)
    c = c * np.exp(rng.uniform(np.log(1e-2), 0.0, s))
    sigma = 1e-3 * np.sqrt(np.sum(np.abs(c) ** 2))
    sig = ctx.generate(n, k, c, sigma, 77, m.C64)
    opt = ctx.solve_options(s, sigma, min_bins=51, window_delta=1e-5,
                            max_stale_iter=5, precision=m.FP32)
    kk, cc, st = ctx.solve_arrays(sig, m.Rng(123537), opt)
    got = ctx.post_analyze(sig, k, kk, cc)
    assert got["hit"] >= 0.99 * s and got["hit"] + got["miss"] == kk.size
    assert got["hit_l1"] < 1e-3
    x = sig.read().astype(np.complex128)
    want = port.post_analyze(np.fft.fft(x) / n, k, kk, cc)
    for key in PA_KEYS:
        if np.isnan(want[key]):
            assert np.isnan(got[key])
        else:
            assert abs(got[key] - want[key]) <= 1e-9 * abs(want[key]), key
    sig.free()


@pytest.mark.gpu
def test_generate_and_analyze_reject_bad_input(ctx):
    with pytest.raises(m.MpsftError) as e:
        ctx.generate(1 << 16, [3, 3], [1.0, 1.0], 0.0, 1)
    assert e.value.status == m.ERR_INVALID
    with pytest.raises(m.MpsftError) as e:
        ctx.generate(1 << 16, [1 << 16], [1.0], 0.0, 1)
    assert e.value.status == m.ERR_INVALID
    with pytest.raises(m.MpsftError) as e:
        ctx.generate(1000, [1], [1.0], 0.0, 1)
    assert e.value.status == m.ERR_UNSUPPORTED_N
    with pytest.raises(m.MpsftError) as e:
        ctx.generate(1 << 16, [1], [1.0], -1.0, 1)
    assert e.value.status == m.ERR_INVALID
    sig = ctx.generate(1 << 16, [1], [1.0], 0.0, 1)
    with pytest.raises(m.MpsftError) as e:
        ctx.post_analyze(sig, [1], [2, 2], [1.0, 1.0])
    assert e.value.status == m.ERR_INVALID
    sig.free()
