"""The uneven batch (config 3), the large stress case (config 5) and the
headline configuration at the reference's own prime length.

Config 3: many signals of uneven N and S solved as one batch must give each
signal exactly what its own single solve gives, and the oracle's frequency
set. The full batch (256 signals, N in 2^16..2^24, S in [10, 2000]) is made on
the device (mpsft_signal_generate); a 40-signal batch of host-made signals
checks more signals against the oracle.

Prime N: the reference's benchmarks and tests run at primes near powers of two
(kPrimes, src/base.h:50-55; published solve times at N = 4194301). At prime N
the reference's own Transform applies (no power-of-two override) and the
binning reduces indices by Barrett reduction instead of a mask.

Config 5: N = 2^26 (512 MiB, far beyond L2), S = 4000 with 25% close pairs,
40 dB: the FP32 batched path returns the oracle's exact frequency set (same
draws), coefficients within the FP32 tolerance of the oracle's FP64 ones.
"""
from __future__ import annotations

import numpy as np
import pytest

import mpsft_gb300 as m

pytestmark = pytest.mark.gpu


def _opts(ctx, s, sigma, prec=m.FP32):
    return ctx.solve_options(s, sigma, trials=1, min_bins=51, window_delta=1e-5,
                             window_threshold=0.1, max_stale_iter=5,
                             precision=prec)


def test_config3_uneven_batch(ctx, port):
    from mpsft_gb300.signals import make_signal

    rng = np.random.default_rng(33)
    specs = [(1 << int(rng.integers(16, 21)), int(rng.integers(10, 401)))
             for _ in range(40)]
    sigs_host = [make_signal(n, s, 3300 + i, sigma=1e-6)
                 for i, (n, s) in enumerate(specs)]
    sigs = [ctx.upload(sg.x) for sg in sigs_host]
    opts = [_opts(ctx, sg.k.size, sg.sigma) for sg in sigs_host]
    out, stats = ctx.solve_batched(sigs, [m.Rng(500 + i) for i in range(len(sigs))],
                                   opts)
    for i, ((k, c), st) in enumerate(zip(out, stats)):
        assert st["status"] == 0
        k1, c1, _ = ctx.solve_arrays(sigs[i], m.Rng(500 + i), opts[i])
        assert np.array_equal(k, k1)
        assert np.array_equal(c.view(np.uint64), c1.view(np.uint64))
    # the oracle's frequency sets for a few of them (FP64, same draws)
    for i in (0, 7, 19, 33):
        sg = sigs_host[i]
        want, _ = port.demo1_run(sg.x.astype(np.complex128), sg.k.size, sg.sigma,
                                 500 + i, min_bins=51, window_delta=1e-5,
                                 max_stale_iter=5)
        assert out[i][0].tolist() == sorted(want), i


def test_config3_full_batch(ctx, port):
    """The 256-signal uneven batch at its stated sizes: every signal equals its
    own single solve bit for bit, and for eight of them (the largest N and S
    among them) the oracle's frequency set, coefficients within the FP32
    tolerance."""
    from mpsft_gb300.signals import config3_spec

    specs = [config3_spec(i) for i in range(256)]
    sigs = [ctx.generate(sp.n, sp.k, sp.c, sp.sigma, sp.seed, m.C64) for sp in specs]
    opts = [_opts(ctx, sp.k.size, sp.sigma) for sp in specs]
    out, stats = ctx.solve_batched(sigs, [m.Rng(900 + i) for i in range(256)], opts)
    iters = sum(st["iterations"] for st in stats)
    fp64_iters = sum(st["fp64_iterations"] for st in stats)
    print(f"config3: {iters} iterations, {fp64_iters} on the FP64 kernels "
          f"({fp64_iters / iters:.1%}) by the precision policy")
    for i, ((k, c), st) in enumerate(zip(out, stats)):
        assert st["status"] == 0, i
        k1, c1, _ = ctx.solve_arrays(sigs[i], m.Rng(900 + i), opts[i])
        assert np.array_equal(k, k1), i
        assert np.array_equal(c.view(np.uint64), c1.view(np.uint64)), i
    big_n = [i for i, sp in enumerate(specs) if sp.n == 1 << 24][:2]
    big_s = sorted(range(256), key=lambda i: -specs[i].k.size)[:2]
    picks = sorted(set(big_n + big_s + [0, 64, 128, 192]))
    assert len(picks) >= 8
    for i in picks:
        sp = specs[i]
        x = sigs[i].read().astype(np.complex128)
        want, _ = port.demo1_run(x, sp.k.size, sp.sigma, 900 + i, min_bins=51,
                                 window_delta=1e-5, max_stale_iter=5)
        k, c = out[i]
        assert k.tolist() == sorted(want), i
        wk = np.array(sorted(want))
        wc = np.array([want[v] for v in wk])
        assert np.linalg.norm(c - wc) / np.linalg.norm(wc) < 1e-5, i
    for sg in sigs:
        sg.free()


@pytest.mark.parametrize("prec", [m.FP64, m.FP32], ids=["fp64", "fp32"])
def test_prime_n_headline_config(ctx, port, prec):
    """The headline configuration (S = 1000, |c| log-uniform [1e-2, 1], 60 dB)
    at N = kPrimes[22] = 4194301, the reference's own benchmark length: the
    oracle's frequency set (FP64, the reference's Transform, same draws);
    coefficients within 1e-9 (FP64) / 1e-5 (FP32) of the oracle's."""
    from mpsft_gb300.signals import make_signal

    n = 4194301
    sg = make_signal(n, 1000, 22, magnitude="loguniform", mag_range=(1e-2, 1.0),
                     snr_db=60.0)
    want, _ = port.demo1_run(sg.x.astype(np.complex128), 1000, sg.sigma, 123537,
                             min_bins=51, window_delta=1e-5, max_stale_iter=5)
    sig = ctx.upload(sg.x)
    k, c, st = ctx.solve_arrays(sig, m.Rng(123537), _opts(ctx, 1000, sg.sigma, prec))
    sig.free()
    assert st.status == 0
    assert k.tolist() == sorted(want)
    wk = np.array(sorted(want))
    wc = np.array([want[v] for v in wk])
    err = float(np.linalg.norm(c - wc) / np.linalg.norm(wc))
    print(f"prime n: prec={prec} iterations={st.iterations} found={k.size} "
          f"true={int(np.isin(k, sg.k).sum())} precision_err={err:.2e}")
    assert err < (1e-9 if prec == m.FP64 else 1e-5), err


def test_config5_stress(ctx, port):
    from mpsft_gb300.signals import config5

    sg = config5()
    x128 = sg.x.astype(np.complex128)
    want, _ = port.demo1_run(x128, 4000, sg.sigma, 123537, min_bins=51,
                             window_delta=1e-5, max_stale_iter=5)
    del x128
    sig = ctx.upload(sg.x)
    k, c, st = ctx.solve_arrays(sig, m.Rng(123537), _opts(ctx, 4000, sg.sigma))
    assert st.status == 0
    assert k.tolist() == sorted(want)
    wk = np.array(sorted(want))
    wc = np.array([want[v] for v in wk])
    err = float(np.linalg.norm(c - wc) / np.linalg.norm(wc))
    hits = np.isin(k, sg.k)
    print(f"config5: iterations={st.iterations} found={k.size} "
          f"true={int(hits.sum())}/{sg.k.size} precision_err={err:.2e} "
          f"near_ties={st.escalated}")
    assert err < 1e-5
