"""The autotuner of the FP32 binning's launch shape (mpsft_autotune): every
shape gives the same frequency sets as the default shape (coefficients within
the FP32 tolerance, 1e-5 relative), in the solve graph and in the host-driven
loop; the tuner fills the context's table, the table survives a save and
load, and the table shipped with the package (mpsft_gb300/tuning/) loads."""
from __future__ import annotations

import os

import numpy as np
import pytest

import mpsft_gb300 as m

pytestmark = pytest.mark.gpu


def _batch(ctx):
    from mpsft_gb300.signals import make_signal

    sigs, opts = [], []
    for i, (n, s) in enumerate([(1 << 20, 300), (1 << 18, 120), (65537, 60),
                                (1 << 20, 50)]):
        sg = make_signal(n, s, 7100 + i, magnitude="loguniform", snr_db=60.0)
        sigs.append(ctx.upload(sg.x))
        opts.append(ctx.solve_options(s, sg.sigma, min_bins=51, window_delta=1e-5,
                                      max_stale_iter=5, precision=m.FP32))
    return sigs, opts


def _solve(ctx, sigs, opts):
    out, stats = ctx.solve_batched(sigs, [m.Rng(800 + i) for i in range(len(sigs))],
                                   opts)
    assert all(st["status"] == 0 for st in stats)
    return out


def test_every_shape_gives_the_same_modes(ctx):
    sigs, opts = _batch(ctx)
    try:
        ctx.set_fold_shape(0)
        want = _solve(ctx, sigs, opts)
        for shape in range(1, m.load_library().mpsft_fold_shape_count()):
            ctx.set_fold_shape(shape)
            got = _solve(ctx, sigs, opts)
            for (k, c), (wk, wc) in zip(got, want):
                assert np.array_equal(k, wk), shape
                assert np.linalg.norm(c - wc) / np.linalg.norm(wc) < 1e-5, shape
            # the host-driven loop launches the same shape
            ctx.set_profiling(True)
            got = _solve(ctx, sigs, opts)
            ctx.set_profiling(False)
            for (k, _), (wk, _) in zip(got, want):
                assert np.array_equal(k, wk), shape
    finally:
        ctx.set_fold_shape(-1)
        ctx.set_profiling(False)
        for sg in sigs:
            sg.free()


def test_autotune_fills_saves_and_loads(ctx, tmp_path):
    sigs, opts = _batch(ctx)
    try:
        ctx.set_fold_shape(0)
        want = _solve(ctx, sigs, opts)
        ctx.set_fold_shape(-1)
        ctx.autotune(sigs, opts, repeats=1)
        assert ctx.tuning_size() > 0
        path = str(tmp_path / "shapes.tsv")
        ctx.tuning_save(path)
        lines = [ln for ln in open(path) if not ln.startswith("#")]
        assert len(lines) == ctx.tuning_size()
        for ln in lines:
            _, _, _, _, shape, us = ln.split()
            assert 0 <= int(shape) < m.load_library().mpsft_fold_shape_count()
            assert float(us) > 0
        ctx.tuning_load(path)
        got = _solve(ctx, sigs, opts)
        for (k, c), (wk, wc) in zip(got, want):
            assert np.array_equal(k, wk)
            assert np.linalg.norm(c - wc) / np.linalg.norm(wc) < 1e-5
    finally:
        if os.path.exists(m.TUNING_PATH):
            ctx.tuning_load(m.TUNING_PATH)
        for sg in sigs:
            sg.free()


def test_shipped_table_loads(ctx):
    if not os.path.exists(m.TUNING_PATH):
        pytest.skip("no tuning table shipped")
    ctx.tuning_load(m.TUNING_PATH)
    assert ctx.tuning_size() > 0
