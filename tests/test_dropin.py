"""The entry points the drop-in adapter (mpsft_gb300/adapter) binds, called as
the adapter calls them: binning windowed by the reference Window's own table
(Window::wt(), no window delta), BinInFreq with Window::SampleInFreq's
responses given per mode, and Iterate on draws made outside the library.

The window tables and responses come from the oracle restatement of Window,
which equals the reference's bit for bit (tests/test_oracle.py); the bins and
modes are compared with the reference's own outputs
(tests/golden/ref_golden.npz) at window delta 1e-5 and 1e-6. Tolerances as in
tests/test_gpu_parity.py: bins within 1e-11 (FP64) / 1e-5 (FP32) of max|U|,
BinInFreq within 1e-12, coefficients within 1e-9 (FP64) / 1e-5 (FP32).
"""
from __future__ import annotations

import numpy as np
import pytest

import cases
import mpsft_gb300 as m

pytestmark = pytest.mark.gpu

TOL_BINS = {m.FP64: 1e-11, m.FP32: 1e-5}
TOL_COEF = {m.FP64: 1e-9, m.FP32: 1e-5}
PRECS = [m.FP64, m.FP32]
PREC_IDS = ["fp64", "fp32"]


def rel_err(a, b):
    return float(np.abs(np.asarray(a) - np.asarray(b)).max() / np.abs(b).max())


@pytest.mark.parametrize("prec", PRECS, ids=PREC_IDS)
@pytest.mark.parametrize("case", cases.RANDOM_BINS, ids=[c[0] for c in cases.RANDOM_BINS])
def test_bins_with_the_window_table(ctx, port, golden, case, prec):
    """delta 1e-5 (pow2_b101, prime_b101, pow2_b2001) and 1e-6 (prime_b51)."""
    name, n, bins, delta, a, b, c, q, seed = case
    sig = ctx.upload(cases.random_signal(n, seed))
    bits = m.load_library().mpsft_num_bits(n, bins)
    wt = port.window(n, bins, delta)
    u = ctx.bin_in_time_wt(sig, bins, bits, wt, a, b, c, q, precision=prec)
    assert rel_err(u, golden[f"rb_{name}"]) < TOL_BINS[prec]
    if prec == m.FP64:
        # the same bins as the entry point that builds the window from delta
        u2 = ctx.bin_in_time(sig, bins, bits, delta, a, b, c, q, precision=prec)
        assert rel_err(u, u2) < 1e-13
    sig.free()


@pytest.mark.parametrize("prec", PRECS, ids=PREC_IDS)
def test_known_answer_with_the_window_table(ctx, port, golden, prec):
    kc = cases.KNOWN
    sig = ctx.upload(cases.evaluate_modes(kc["n"], kc["modes"]))
    wt = port.window(kc["n"], kc["bins"], kc["delta"])
    u = ctx.bin_in_time_wt(sig, kc["bins"], kc["bits"], wt, kc["a"], kc["b"],
                           kc["c"], kc["q"], precision=prec)
    assert abs(u[0, 1] - (1.12652 - 0.108838j)) < 2e-5  # src/binner_test.cc:74-75
    assert rel_err(u, golden["known_v4"]) < TOL_BINS[prec]
    sig.free()


def _responses(port, n, bins, delta, a, b, k0):
    """Window::SampleInFreq at each mode's offset in its bin, formed as
    BinInFreqV1 forms it (src/binner.cc:571-575) and as the adapter does."""
    out = []
    for k in np.asarray(k0, np.int64):
        k1 = (a * int(k) + b) % n
        bin_ = k1 * bins // n
        xi = (bin_ + 0.5) / bins - k1 / n
        out.append(port.sample_in_freq(n, bins, delta, xi))
    return np.array(out)


@pytest.mark.parametrize("case", cases.RANDOM_BINS, ids=[c[0] for c in cases.RANDOM_BINS])
def test_bin_in_freq_with_responses(ctx, port, golden, case):
    name, n, bins, delta, a, b, c, q, seed = case
    bits = m.load_library().mpsft_num_bits(n, bins)
    k0 = golden[f"rf_{name}_k"]
    wf = _responses(port, n, bins, delta, a, b, k0)
    f = ctx.bin_in_freq_wf(golden[f"rb_{name}"], n, bins, bits, a, b, c, q, k0,
                           golden[f"rf_{name}_c"], wf)
    assert rel_err(f, golden[f"rf_{name}"]) < 1e-12


def test_time_plus_freq_is_zero(ctx, port):
    """src/binner_test.cc:77-103: BinInFreq gives the exact negative of
    BinInTime for a one-mode signal, both through the table entry points."""
    kc = cases.KNOWN
    n, bins, bits = kc["n"], kc["bins"], kc["bits"]
    sig = ctx.upload(cases.evaluate_modes(n, kc["modes"]))
    wt = port.window(n, bins, kc["delta"])
    u = ctx.bin_in_time_wt(sig, bins, bits, wt, kc["a"], kc["b"], kc["c"], kc["q"],
                           precision=m.FP64)
    k0 = np.array(list(kc["modes"]), np.int32)
    cf = np.array(list(kc["modes"].values()))
    wf = _responses(port, n, bins, kc["delta"], kc["a"], kc["b"], k0)
    f = ctx.bin_in_freq_wf(u, n, bins, bits, kc["a"], kc["b"], kc["c"], kc["q"],
                           k0, cf, wf)
    assert np.abs(f).max() < 1e-5
    sig.free()


def test_window_table_checks(ctx, port):
    sig = ctx.upload(cases.random_signal(1 << 16, 1))
    wt = port.window(1 << 16, 101, 1e-5)
    bad = wt.copy()
    bad[-1] *= 1.0 + 1e-12  # not even
    with pytest.raises(m.MpsftError) as e:
        ctx.bin_in_time_wt(sig, 101, 2, bad, 3, 1, 1, 1)
    assert e.value.status == m.ERR_INVALID
    with pytest.raises(m.MpsftError) as e:
        ctx.bin_in_time_wt(sig, 101, 2, wt[:-2], 3, 1, 1, 1)  # p not a multiple
    assert e.value.status == m.ERR_INVALID
    sig.free()


@pytest.mark.parametrize("prec", PRECS, ids=PREC_IDS)
def test_iterate_on_outside_draws(ctx, golden, prec):
    """Iterate driven by draws made outside the library (as IterateGPU draws
    them from the reference's global RNG): the reference's Iterate outputs of
    test_iterate_matches_reference, whose draws came from Rng(4242)."""
    case = cases.SOLVES[2]
    x, sigma = cases.solve_signal(case)
    n = x.size
    sig = ctx.upload(np.asarray(x, np.complex128))
    rng = m.Rng(4242)
    mm: dict = {}
    for i, bins in enumerate((401, 201)):
        a = (rng.int32() % (n - 1)) + 1
        b = rng.int32() % n
        c = rng.int32() % n
        a |= 1  # power-of-two n: the odd a of the library's Transform
        q = [rng.int32() % n for _ in range(3)]
        found, mm = ctx.iterate_draws(sig, a, b, c, pow(a, -1, n), q, bins,
                                      window_delta=1e-5,
                                      bin_threshold=3 * sigma / np.sqrt(bins),
                                      window_threshold=0.1,
                                      sv_threshold=sigma / np.sqrt(bins), mm=mm,
                                      precision=prec)
        want_k = golden[f"iter{i}_k"]
        assert sorted(mm) == want_k.tolist()
        d = np.array([mm[int(k)] for k in want_k]) - golden[f"iter{i}_c"]
        assert np.linalg.norm(d) / np.linalg.norm(golden[f"iter{i}_c"]) < TOL_COEF[prec]
        assert int(found) == int(golden[f"iter{i}_found"][0])
    sig.free()
