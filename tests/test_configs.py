"""The uneven batch (config 3) and the large stress case (config 5).

Config 3: many signals of uneven N and S solved as one batch must give each
signal exactly what its own single solve gives, and the oracle's frequency
set. The test batch keeps config 3's distribution but draws N from
{2^16, ..., 2^20} and S from [10, 400] so that host signal generation and the
oracle stay within seconds (the full 256-signal batch with N up to 2^24 runs
in bench.py's --workload config3 mode).

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
