"""Seeded synthetic sparse signals with the shapes of the benchmark workloads.

x_t = sum_k xhat_k e^{2 pi i k t / n} (the reference's unnormalised backward
FFT, src/demo1.cc:27-34) for S modes at distinct uniform-random k, plus i.i.d.
complex Gaussian noise of per-sample variance sigma^2 (the distribution of
GenerateXhatAlt, src/gen.cc:77-89: frequency-domain noise of variance
sigma^2/n per bin, which is time-domain variance sigma^2 per sample).

All draws come from numpy's PCG64 generator, so the same seed gives the same
signal on every host.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np


@dataclass
class SparseSignal:
    x: np.ndarray          # time-domain samples
    k: np.ndarray          # int64 mode positions
    c: np.ndarray          # complex128 mode coefficients
    sigma: float           # per-sample noise standard deviation
    n: int


def distinct_positions(rng: np.random.Generator, n: int, s: int) -> np.ndarray:
    out: list[int] = []
    seen: set[int] = set()
    while len(out) < s:
        for v in rng.integers(0, n, size=2 * (s - len(out)) + 8).tolist():
            if v not in seen:
                seen.add(v)
                out.append(v)
                if len(out) == s:
                    break
    return np.array(out, np.int64)


def paired_positions(rng: np.random.Generator, n: int, s: int,
                     pair_frac: float) -> np.ndarray:
    """Positions where pair_frac of the modes sit in close pairs 1-3 apart."""
    npair = int(round(s * pair_frac)) // 2
    out: list[int] = []
    seen: set[int] = set()
    while len(out) < 2 * npair:
        a = int(rng.integers(0, n))
        d = int(rng.integers(1, 4))
        b = (a + d) % n
        if a in seen or b in seen:
            continue
        seen.update((a, b))
        out += [a, b]
    while len(out) < s:
        v = int(rng.integers(0, n))
        if v not in seen:
            seen.add(v)
            out.append(v)
    return np.array(out, np.int64)


def make_signal(n: int, s: int, seed: int, *, magnitude: str = "unit",
                mag_range: tuple[float, float] = (1e-2, 1.0),
                sigma: float | None = None, snr_db: float | None = None,
                pair_frac: float = 0.0,
                dtype=np.complex64) -> SparseSignal:
    rng = np.random.default_rng(seed)
    if pair_frac > 0:
        k = paired_positions(rng, n, s, pair_frac)
    else:
        k = distinct_positions(rng, n, s)
    if magnitude == "unit":
        mag = np.ones(s)
    elif magnitude == "loguniform":
        lo, hi = mag_range
        mag = np.exp(rng.uniform(np.log(lo), np.log(hi), s))
    else:
        raise ValueError(magnitude)
    c = mag * np.exp(2j * np.pi * rng.uniform(size=s))
    if sigma is None:
        if snr_db is None:
            raise ValueError("give sigma or snr_db")
        sigma = float(10.0 ** (-snr_db / 20.0) * np.sqrt(np.sum(mag ** 2)))
    xh = np.zeros(n, np.complex128)
    xh[k] = c
    x = np.fft.ifft(xh) * n
    del xh
    noise = rng.standard_normal((2, n))
    x += (sigma / np.sqrt(2.0)) * (noise[0] + 1j * noise[1])
    return SparseSignal(x=x.astype(dtype), k=k, c=c, sigma=float(sigma), n=n)


def config1(seed: int = 1, dtype=np.complex128) -> SparseSignal:
    """N = 2^20, S = 50 unit-magnitude modes, sigma = 1e-6 (complex128)."""
    return make_signal(1 << 20, 50, seed, sigma=1e-6, dtype=dtype)


def config2(seed: int = 7) -> SparseSignal:
    """N = 2^22 complex64, S = 1000, |c| log-uniform in [1e-2, 1], 60 dB SNR."""
    return make_signal(1 << 22, 1000, seed, magnitude="loguniform",
                       mag_range=(1e-2, 1.0), snr_db=60.0)


def config3(index: int, base_seed: int = 300) -> SparseSignal:
    """Signal `index` of the uneven batch: N = 2^e with e uniform in
    {16, ..., 24}, S uniform in [10, 2000], config-1 modes and noise
    (unit magnitudes, sigma = 1e-6), complex64; seed-indexed."""
    rng = np.random.default_rng(base_seed + index)
    e = int(rng.integers(16, 25))
    s = int(rng.integers(10, 2001))
    return make_signal(1 << e, s, base_seed * 1000 + index, sigma=1e-6)


@dataclass
class SignalSpec:
    """The modes and noise level of a signal whose samples are made on the
    device (mpsft_signal_generate): no host-side synthesis."""
    n: int
    k: np.ndarray          # int64 distinct positions
    c: np.ndarray          # complex128 coefficients
    sigma: float
    seed: int              # key of the device noise generator


def config3_spec(index: int, base_seed: int = 300) -> SignalSpec:
    """config3(index)'s length, modes and noise level (the same draws), for
    generation on the device."""
    rng = np.random.default_rng(base_seed + index)
    e = int(rng.integers(16, 25))
    s = int(rng.integers(10, 2001))
    seed = base_seed * 1000 + index
    r2 = np.random.default_rng(seed)
    k = distinct_positions(r2, 1 << e, s)
    c = np.exp(2j * np.pi * r2.uniform(size=s))
    return SignalSpec(n=1 << e, k=k, c=c, sigma=1e-6, seed=seed)


def config5(seed: int = 5) -> SparseSignal:
    """N = 2^26 complex64 (512 MiB), S = 4000 with 25% of the modes in close
    pairs 1-3 apart, |c| log-uniform in [1e-3, 1], 40 dB SNR."""
    return make_signal(1 << 26, 4000, seed, magnitude="loguniform",
                       mag_range=(1e-3, 1.0), snr_db=40.0, pair_frac=0.25)


def config5_spec(seed: int = 5) -> SignalSpec:
    """config5(seed)'s modes and noise level (the same draws), for generation
    on the device (512 MiB per signal)."""
    rng = np.random.default_rng(seed)
    n, s = 1 << 26, 4000
    k = paired_positions(rng, n, s, 0.25)
    mag = np.exp(rng.uniform(np.log(1e-3), np.log(1.0), s))
    c = mag * np.exp(2j * np.pi * rng.uniform(size=s))
    sigma = float(10.0 ** (-40.0 / 20.0) * np.sqrt(np.sum(mag ** 2)))
    return SignalSpec(n=n, k=k, c=c, sigma=sigma, seed=seed)
