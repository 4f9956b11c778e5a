"""numpy restatement of the device signal generator (test infrastructure only:
tests import it as the checker of mpsft_signal_generate).

x_t = sum_j c_j e^{2 pi i k_j t / n} + noise_t: the unnormalised backward FFT
of the spectrum GenerateXhatAlt builds (src/gen.cc:77-89; Demo1's constructor,
src/demo1.cc:27-34), with the noise drawn in the time domain at per-sample
variance sigma^2 (the same distribution as GenerateXhatAlt's per-frequency
variance sigma^2 / n). The noise comes from a counter-based generator instead
of the reference's sequential mt19937: output i of SplitMix64 (Steele, Lea and
Flood, OOPSLA 2014) started at seed is mix(seed + (i + 1) * gamma); sample t
takes outputs 2t and 2t + 1 as u1, u2 = ((z >> 11) + 1) * 2^-53 in (0, 1] and
the Box-Muller transform r = sqrt(-2 ln u1), (r cos 2 pi u2, r sin 2 pi u2),
scaled by sigma / sqrt(2).
"""
from __future__ import annotations

import numpy as np

_GAMMA = np.uint64(0x9E3779B97F4A7C15)
_M1 = np.uint64(0xBF58476D1CE4E5B9)
_M2 = np.uint64(0x94D049BB133111EB)


def splitmix64(seed: int, idx: np.ndarray) -> np.ndarray:
    """Outputs idx (uint64 array) of the SplitMix64 sequence started at seed."""
    with np.errstate(over="ignore"):
        z = np.uint64(seed & (2**64 - 1)) + (idx.astype(np.uint64) + np.uint64(1)) * _GAMMA
        z = (z ^ (z >> np.uint64(30))) * _M1
        z = (z ^ (z >> np.uint64(27))) * _M2
        return z ^ (z >> np.uint64(31))


def uniform_open0(seed: int, idx: np.ndarray) -> np.ndarray:
    z = splitmix64(seed, idx)
    return ((z >> np.uint64(11)) + np.uint64(1)).astype(np.float64) * 2.0**-53


def noise(n: int, sigma: float, seed: int) -> np.ndarray:
    """The generator's noise samples 0..n-1 (complex128)."""
    t = np.arange(n, dtype=np.uint64)
    u1 = uniform_open0(seed, 2 * t)
    u2 = uniform_open0(seed, 2 * t + np.uint64(1))
    r = np.sqrt(-2.0 * np.log(u1))
    h = sigma * 0.70710678118654752440
    return h * (r * np.cos(2 * np.pi * u2)) + 1j * (h * (r * np.sin(2 * np.pi * u2)))


def modes(n: int, k, c) -> np.ndarray:
    """sum_j c_j e^{2 pi i k_j t / n}, t < n, by numpy's FFT (complex128)."""
    xh = np.zeros(n, np.complex128)
    xh[np.asarray(k, np.int64)] = np.asarray(c, np.complex128)
    return np.fft.ifft(xh) * n


def generate(n: int, k, c, sigma: float, seed: int) -> np.ndarray:
    x = modes(n, k, c)
    if sigma > 0:
        x = x + noise(n, sigma, seed)
    return x
