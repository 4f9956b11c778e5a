"""Parity of the CUDA path (called through the C ABI) with the reference.

Bins and operators are compared with the reference's own outputs
(tests/golden/ref_golden.npz) and with the oracle; whole solves must return
the reference's exact frequency set.

Tolerances (stated per result):
  * FP64 path: bins within 1e-11 of max|U|; coefficients within 1e-9
    (relative, norm over the common set).
  * FP32 path: bins within 1e-5 of max|U| (FP32 gather/fold/FFT, FP64 after);
    coefficients within 1e-5 relative (the precision-error target).
  * frequency sets: identical (bit-exact k0 values) for both paths.
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
    a = np.asarray(a)
    b = np.asarray(b)
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


def coef_err(got: dict, want_k, want_c):
    d = np.array([got[int(k)] for k in want_k]) - np.asarray(want_c)
    return float(np.linalg.norm(d) / np.linalg.norm(want_c))


@pytest.mark.parametrize("prec", PRECS, ids=PREC_IDS)
def test_known_answer_bins(ctx, golden, prec):
    kc = cases.KNOWN
    x = cases.evaluate_modes(kc["n"], kc["modes"])
    sig = ctx.upload(x)
    u = ctx.bin_in_time(sig, kc["bins"], kc["bits"], kc["delta"], kc["a"], kc["b"],
                        kc["c"], kc["q"], precision=prec)
    # src/binner_test.cc:74-75
    assert abs(u[0, 1] - (1.12652 - 0.108838j)) < 1e-5 * 2
    assert rel_err(u, golden["known_v4"]) < TOL_BINS[prec]


@pytest.mark.parametrize("prec", PRECS, ids=PREC_IDS)
def test_bigger_bins(ctx, golden, prec):
    bc = cases.BIGGER
    x = cases.evaluate_modes(bc["n"], bc["modes"])
    sig = ctx.upload(x)
    u = ctx.bin_in_time(sig, bc["bins"], bc["bits"], bc["delta"], bc["a"], bc["b"],
                        bc["c"], bc["q"], precision=prec)
    assert rel_err(u, golden["bigger_v4"]) < 10 * TOL_BINS[prec]
    # time + freq = 0 (src/binner_test.cc:140-142)
    ks = np.array(list(bc["modes"]), np.int32)
    cs = np.array(list(bc["modes"].values()))
    f = ctx.bin_in_freq(np.zeros_like(u), bc["n"], bc["bins"], bc["bits"],
                        bc["delta"], bc["a"], bc["b"], bc["c"], bc["q"], ks, cs)
    assert rel_err(f, golden["bigger_freq"]) < 1e-12
    assert np.abs(u[0] + f[0]).max() < 1e-5


@pytest.mark.parametrize("prec", PRECS, ids=PREC_IDS)
@pytest.mark.parametrize("case", cases.RANDOM_BINS, ids=[c[0] for c in cases.RANDOM_BINS])
def test_random_bins(ctx, golden, case, prec):
    name, n, bins, delta, a, b, c, q, seed = case
    x = cases.random_signal(n, seed)
    sig = ctx.upload(x)
    bits = m.load_library().mpsft_num_bits(n, bins)
    u = ctx.bin_in_time(sig, bins, bits, delta, a, b, c, q, precision=prec)
    assert rel_err(u, golden[f"rb_{name}"]) < TOL_BINS[prec]


SMALL_BINS = [c for c in cases.RANDOM_BINS if c[2] <= 101]


@pytest.mark.parametrize("case", SMALL_BINS, ids=[c[0] for c in SMALL_BINS])
def test_direct_bins(ctx, golden, case):
    """The FP64 direct summation used for the FP32 path's near-tie bins gives
    the reference's bins (no fold, no size-B FFT)."""
    name, n, bins, delta, a, b, c, q, seed = case
    x = cases.random_signal(n, seed)
    sig = ctx.upload(x)
    bits = m.load_library().mpsft_num_bits(n, bins)
    u = ctx.bin_in_time(sig, bins, bits, delta, a, b, c, q, precision=m.FP64_DIRECT)
    assert rel_err(u, golden[f"rb_{name}"]) < TOL_BINS[m.FP64]


@pytest.mark.parametrize("case", cases.RANDOM_BINS, ids=[c[0] for c in cases.RANDOM_BINS])
def test_bin_in_freq(ctx, golden, case):
    name, n, bins, delta, a, b, c, q, seed = case
    bits = m.load_library().mpsft_num_bits(n, bins)
    f = ctx.bin_in_freq(golden[f"rb_{name}"], n, bins, bits, delta, a, b, c, q,
                        golden[f"rf_{name}_k"], golden[f"rf_{name}_c"])
    assert rel_err(f, golden[f"rf_{name}"]) < 1e-12


def test_pencil_known_answers(ctx):
    u = np.array([[-2.3 + 5.2j, -5.5 - 3.1j, 4.0 + 3.0j],
                  [2.3 + 5.2j, 5.5 - 3.1j, 4.0 + 3.0j],
                  [-15.3 - 5.2j, 8.0 + 3.0j, -1.5 + 3.5j]])
    sig, vote = ctx.mat_pencil(u)
    want = np.array([[11.34419934, 0.91057194], [9.80673965, 5.77476038],
                     [21.27794592, 12.53032391]])
    assert np.allclose(sig, want, rtol=1.2e-5, atol=0)
    assert vote.tolist() == [False, True, False]


def test_pencil_matches_oracle(ctx, port):
    rng = np.random.default_rng(3)
    u = rng.standard_normal((500, 3)) + 1j * rng.standard_normal((500, 3))
    sig, vote = ctx.mat_pencil(u)
    for i in range(500):
        s0, s1, v = port.mat_pencil(*u[i])
        assert abs(sig[i, 0] - s0) <= 1e-13 * s0 and abs(sig[i, 1] - s1) <= 1e-12 * s0
        assert vote[i] == v


def test_window_table(ctx, golden):
    wt = ctx.window_table(1109, 5, 1e-6)
    assert rel_err(wt, golden["window_1109_5_1e-6"]) < 1e-14


@pytest.mark.parametrize("prec", PRECS, ids=PREC_IDS)
def test_iterate_matches_reference(ctx, golden, prec):
    case = cases.SOLVES[2]
    x, sigma = cases.solve_signal(case)
    sig = ctx.upload(np.asarray(x, np.complex128))
    rng = m.Rng(4242)
    mm: dict = {}
    for i, bins in enumerate((401, 201)):
        found, mm = ctx.iterate(sig, rng, bins, window_delta=1e-5, trials=3,
                                bin_threshold=3 * sigma / np.sqrt(bins),
                                window_threshold=0.1,
                                sv_threshold=sigma / np.sqrt(bins), mm=mm,
                                precision=prec)
        assert sorted(mm) == golden[f"iter{i}_k"].tolist()
        assert coef_err(mm, golden[f"iter{i}_k"], golden[f"iter{i}_c"]) < TOL_COEF[prec]
        assert int(found) == int(golden[f"iter{i}_found"][0])


def _solve(ctx, x, s, sigma, rseed, trials, min_bins, delta, prec, **kw):
    sig = ctx.upload(x)
    opt = ctx.solve_options(s, sigma, trials=trials, min_bins=min_bins,
                            window_delta=delta, window_threshold=0.1,
                            max_stale_iter=5, precision=prec, **kw)
    return ctx.solve(sig, m.Rng(rseed), opt)


@pytest.mark.parametrize("prec", PRECS, ids=PREC_IDS)
@pytest.mark.parametrize("case", cases.SOLVES, ids=[c[0] for c in cases.SOLVES])
def test_solve_matches_reference(ctx, golden, case, prec):
    name, n, s, _, trials, min_bins, delta, _, rseed, _ = case
    x, sigma = cases.solve_signal(case)
    modes, st = _solve(ctx, x, s, sigma, rseed, trials, min_bins, delta, prec)
    want_k = golden[f"solve_{name}_k"]
    assert sorted(modes) == want_k.tolist()
    assert coef_err(modes, want_k, golden[f"solve_{name}_c"]) < TOL_COEF[prec]
    assert st.iterations > 0 and st.found == len(modes)


@pytest.mark.parametrize("prec", PRECS, ids=PREC_IDS)
def test_config2_full_size_matches_oracle(ctx, port, prec):
    """N = 2^22, S = 1000, |c| log-uniform [1e-2, 1], 60 dB: same frequency set
    as the oracle (FP64, same draws); coefficient precision error within the
    stated tolerance; algorithm error vs an FP64 dense FFT reported."""
    from mpsft_gb300.signals import config2

    sgl = config2(seed=7)
    want, _ = port.demo1_run(sgl.x.astype(np.complex128), 1000, sgl.sigma, 123537,
                             min_bins=51, window_delta=1e-5, max_stale_iter=5)
    got, st = _solve(ctx, sgl.x, 1000, sgl.sigma, 123537, 1, 51, 1e-5, prec)
    assert sorted(got) == sorted(want)
    wk = np.array(sorted(want))
    err = coef_err(got, wk, [want[k] for k in wk])
    assert err < TOL_COEF[prec], err
    xf = np.fft.fft(sgl.x.astype(np.complex128)) / sgl.n
    hits = np.array(sorted(set(got) & set(sgl.k.tolist())))
    alg = np.linalg.norm([got[k] - xf[k] for k in hits]) / np.linalg.norm(xf[hits])
    print(f"prec={prec} iterations={st.iterations} found={len(got)} "
          f"precision_err={err:.2e} algorithm_err={alg:.2e}")
    assert alg < 1e-2


@pytest.mark.parametrize("shape", [6, 8])
def test_stashed_rebinning_matches_oracle(ctx, port, shape):
    """The pairwise fold shapes (6: split 4, 8: split 8) stash the samples
    they gather (row 0 while the fold reads much of the signal, every row
    once it gathers from few sectors) and the near-tie re-binning reads them
    instead of gathering them again: the oracle's frequency sets (same
    draws), coefficients within the FP32 tolerance, and the host-driven loop
    with the same frequency sets and coefficients within that tolerance."""
    from mpsft_gb300.signals import make_signal

    sigs, opts, wants, seeds = [], [], [], []
    for i, (n, s) in enumerate([(1 << 20, 300), (1 << 20, 150)]):
        sg = make_signal(n, s, 4100 + i, magnitude="loguniform", snr_db=60.0)
        seeds.append(910 + i)
        want, _ = port.demo1_run(sg.x.astype(np.complex128), s, sg.sigma, seeds[-1],
                                 min_bins=51, window_delta=1e-5, max_stale_iter=5)
        wants.append(want)
        sigs.append(ctx.upload(sg.x))
        opts.append(ctx.solve_options(s, sg.sigma, min_bins=51, window_delta=1e-5,
                                      window_threshold=0.1, max_stale_iter=5,
                                      precision=m.FP32))
    try:
        ctx.set_fold_shape(shape)
        out, stats = ctx.solve_batched(sigs, [m.Rng(sd) for sd in seeds], opts)
        assert sum(st["escalated"] for st in stats) > 0  # bins were re-binned
        for (k, c), want, st in zip(out, wants, stats):
            assert st["status"] == 0
            wk = np.array(sorted(want))
            assert k.tolist() == wk.tolist()
            got = {int(a): b for a, b in zip(k, c)}
            assert coef_err(got, wk, [want[kk] for kk in wk]) < TOL_COEF[m.FP32]
        ctx.set_profiling(True)
        out2, _ = ctx.solve_batched(sigs, [m.Rng(sd) for sd in seeds], opts)
        ctx.set_profiling(False)
        for (k, c), (k2, c2) in zip(out, out2):
            assert np.array_equal(k, k2)
            assert np.linalg.norm(c - c2) / np.linalg.norm(c) < TOL_COEF[m.FP32]
    finally:
        ctx.set_fold_shape(-1)
        ctx.set_profiling(False)
        for sg in sigs:
            sg.free()


def test_batched_equals_single(ctx):
    from mpsft_gb300.signals import make_signal

    sigs, opts, rngs, singles = [], [], [], []
    # different trials per signal share one batch (one draw table stride)
    for i, (n, s, tr) in enumerate([(1 << 16, 40, 3), (1 << 18, 120, 7),
                                    (65537, 60, 5)]):
        sg = make_signal(n, s, 100 + i, sigma=1e-5)
        sigs.append(ctx.upload(sg.x))
        opts.append(ctx.solve_options(s, sg.sigma, min_bins=51, window_delta=1e-5,
                                      max_stale_iter=5, trials=tr))
        rngs.append(m.Rng(777 + i))
        singles.append(ctx.solve(sigs[-1], m.Rng(777 + i), opts[-1])[0])
    out, stats = ctx.solve_batched(sigs, rngs, opts)
    for (k, c), single, st in zip(out, singles, stats):
        assert k.tolist() == sorted(single)
        assert np.array_equal(c, np.array([single[kk] for kk in sorted(single)]))
        assert st["status"] == 0


def test_write_many_pipelined(ctx):
    """Two signal sets alternating as a serving loop runs them: a second host
    thread refills one set from pinned memory on a copy stream (one
    mpsft_signal_write_many call) while the context solves the other; every
    step returns exactly what a solve of freshly uploaded signals returns."""
    import threading

    import torch
    from mpsft_gb300.signals import make_signal

    n, S = 1 << 16, 40
    steps = [[make_signal(n, S, 900 + 4 * s + i, sigma=1e-5) for i in range(4)]
             for s in range(4)]
    opts = [ctx.solve_options(S, sg.sigma, min_bins=51, window_delta=1e-5,
                              max_stale_iter=5) for sg in steps[0]]
    want = []
    for batch in steps:
        up = [ctx.upload(sg.x) for sg in batch]
        want.append(ctx.solve_batched(up, [m.Rng(60 + i) for i in range(4)], opts)[0])
        for sg in up:
            sg.free()
    pinned = []
    for batch in steps:
        row = []
        for sg in batch:
            t = torch.empty(n, dtype=torch.complex64, pin_memory=True)
            t.numpy()[:] = sg.x
            row.append(t.numpy())
        pinned.append(row)
    sets = [[ctx.upload(np.zeros(n, np.complex64)) for _ in range(4)] for _ in range(2)]
    copy_stream = torch.cuda.Stream()
    ready = [torch.cuda.Event(), torch.cuda.Event()]

    def write_set(j, s):
        ctx.write_many(sets[j], pinned[s], copy_stream.cuda_stream)
        ready[j].record(copy_stream)

    solve_stream = torch.cuda.Stream()
    ctx.set_stream(solve_stream.cuda_stream)
    try:
        write_set(0, 0)
        for s in range(len(steps)):
            cur = s % 2
            solve_stream.wait_event(ready[cur])
            th = None
            if s + 1 < len(steps):
                th = threading.Thread(target=write_set, args=(1 - cur, s + 1))
                th.start()
            got, stats = ctx.solve_batched(sets[cur], [m.Rng(60 + i) for i in range(4)],
                                           opts)
            if th is not None:
                th.join()
            for (k, c), (k0, c0), st in zip(got, want[s], stats):
                assert st["status"] == 0
                assert np.array_equal(k, k0)
                assert np.array_equal(c.view(np.uint64), c0.view(np.uint64))
    finally:
        ctx.set_stream(None)
    with pytest.raises(ValueError):
        ctx.write_many(sets[0][:1], [np.zeros(n, np.complex128)])


@pytest.mark.parametrize("n", [65537, 1 << 16])
def test_write_many_copies(ctx, n):
    """mpsft_signal_write_many from pinned memory (copied by a kernel through
    the buffer's device mapping; an odd n leaves an 8-byte tail) and from
    pageable memory (DMA copy) leaves the same samples as an upload: the bins
    agree bit for bit."""
    import torch

    rng = np.random.default_rng(n)
    xs = [(rng.standard_normal(n) + 1j * rng.standard_normal(n)).astype(np.complex64)
          for _ in range(3)]
    pinned = []
    for x in xs[:2]:
        t = torch.empty(n, dtype=torch.complex64, pin_memory=True)
        t.numpy()[:] = x
        pinned.append(t.numpy())
    hosts = pinned + [xs[2].copy()]          # two pinned, one pageable
    sigs = [ctx.upload(np.zeros(n, np.complex64)) for _ in range(3)]
    ctx.write_many(sigs, hosts)
    ref = [ctx.upload(x) for x in xs]
    bins, delta = 51, 1e-5
    bits = m.num_bits(n, bins)
    for got, want in zip(sigs, ref):
        ug = ctx.bin_in_time(got, bins, bits, delta, 3, 5, 7, 11, precision=m.FP32)
        uw = ctx.bin_in_time(want, bins, bits, delta, 3, 5, 7, 11, precision=m.FP32)
        assert np.array_equal(ug.view(np.uint64), uw.view(np.uint64))
    for sg in sigs + ref:
        sg.free()


@pytest.mark.parametrize("prec", PRECS, ids=PREC_IDS)
def test_deterministic(ctx, prec):
    from mpsft_gb300.signals import make_signal

    sg = make_signal(1 << 18, 200, 5, magnitude="loguniform", snr_db=50.0)
    sig = ctx.upload(sg.x)
    opt = ctx.solve_options(200, sg.sigma, min_bins=51, window_delta=1e-5,
                            max_stale_iter=5, precision=prec)
    k1, c1, _ = ctx.solve_arrays(sig, m.Rng(9), opt)
    k2, c2, _ = ctx.solve_arrays(sig, m.Rng(9), opt)
    assert np.array_equal(k1, k2) and np.array_equal(c1.view(np.uint64),
                                                     c2.view(np.uint64))


@pytest.mark.parametrize("prec", PRECS, ids=PREC_IDS)
def test_graph_loop_equals_host_loop(ctx, prec):
    """The solve as one CUDA graph (device-side stop rule, draw tables refilled
    between launches) against the host-driven loop that profiling selects:
    same modes bit for bit, same iteration count, RNG left at the same draw.
    max_stale_iter=40 runs past one table of 32 draws."""
    from mpsft_gb300.signals import make_signal

    sg = make_signal(1 << 16, 30, 21, sigma=1e-5)
    sig = ctx.upload(sg.x)
    opt = ctx.solve_options(30, sg.sigma, min_bins=51, window_delta=1e-5,
                            max_stale_iter=40, precision=prec)
    r1, r2 = m.Rng(31), m.Rng(31)
    k1, c1, s1 = ctx.solve_arrays(sig, r1, opt)
    ctx.set_profiling(True)
    try:
        k2, c2, s2 = ctx.solve_arrays(sig, r2, opt)
    finally:
        ctx.set_profiling(False)
    assert s1.iterations == s2.iterations > 40
    assert np.array_equal(k1, k2)
    assert np.array_equal(c1.view(np.uint64), c2.view(np.uint64))
    assert [r1.int32() for _ in range(4)] == [r2.int32() for _ in range(4)]
    assert s1.gathers == s2.gathers and s1.bin_bytes == s2.bin_bytes
    assert s1.escalated == s2.escalated and s1.status == s2.status == 0


def test_batched_graph_equals_host_loop(ctx):
    """An uneven FP32 batch through the solve graph (its phases: large bins,
    small bins, then fixed bins with the next iteration planned and folded
    ahead) against the host-driven loop: signals that reach fixed bins at
    different iterations (k from 10 to 400, min_bins 31 to 101), one long
    enough to refill its draw table; same modes bit for bit, same iteration
    counts and statistics."""
    from mpsft_gb300.signals import make_signal

    spec = [(1 << 16, 10, 51, 5), (1 << 17, 400, 51, 5), (65537, 60, 31, 5),
            (1 << 16, 120, 101, 5), (1 << 18, 30, 51, 40)]
    sigs, opts = [], []
    for i, (n, S, mb, stale) in enumerate(spec):
        sg = make_signal(n, S, 500 + i, sigma=1e-5)
        sigs.append(ctx.upload(sg.x))
        opts.append(ctx.solve_options(S, sg.sigma, min_bins=mb, window_delta=1e-5,
                                      max_stale_iter=stale))
    out1, st1 = ctx.solve_batched(sigs, [m.Rng(80 + i) for i in range(len(spec))], opts)
    ctx.set_profiling(True)
    try:
        out2, st2 = ctx.solve_batched(sigs, [m.Rng(80 + i) for i in range(len(spec))],
                                      opts)
    finally:
        ctx.set_profiling(False)
    assert st1[4]["iterations"] > 32
    for (k1, c1), (k2, c2), a, b in zip(out1, out2, st1, st2):
        assert a["status"] == b["status"] == 0
        assert a["iterations"] == b["iterations"]
        assert a["gathers"] == b["gathers"] and a["escalated"] == b["escalated"]
        assert np.array_equal(k1, k2)
        assert np.array_equal(c1.view(np.uint64), c2.view(np.uint64))
    for sg in sigs:
        sg.free()


def test_table_cache_across_solves(ctx):
    """The solve graph takes its window and Bluestein tables from the
    context's cache (built on first use per number of bins and window delta):
    solves that switch delta and bin range, and then repeat, give what the
    host-driven loop (per-signal tables) gives, bit for bit."""
    from mpsft_gb300.signals import make_signal

    cases = [(1 << 16, 40, 1e-5, 51), (1 << 17, 90, 1e-6, 31), (1 << 16, 40, 1e-5, 51),
             (1 << 16, 300, 1e-5, 51)]
    for n, S, delta, mb in cases:
        sg = make_signal(n, S, 40 + S, sigma=1e-5)
        sig = ctx.upload(sg.x)
        opt = ctx.solve_options(S, sg.sigma, min_bins=mb, window_delta=delta,
                                max_stale_iter=5)
        k1, c1, s1 = ctx.solve_arrays(sig, m.Rng(7), opt)
        ctx.set_profiling(True)
        try:
            k2, c2, s2 = ctx.solve_arrays(sig, m.Rng(7), opt)
        finally:
            ctx.set_profiling(False)
        assert s1.status == s2.status == 0
        assert np.array_equal(k1, k2)
        assert np.array_equal(c1.view(np.uint64), c2.view(np.uint64))


def test_close_frees_live_signals():
    """Closing a context frees its live signals first; the signals' own free
    (explicit or at collection) is then a no-op."""
    c2 = m.Context(0)
    sigs = [c2.upload(np.ones(1 << 12, np.complex64)) for _ in range(3)]
    c2.close()
    assert all(sg._freed for sg in sigs)
    sigs[0].free()
    del sigs


# ------------------------------------------------------------ error paths
def test_errors_are_statuses(ctx):
    from mpsft_gb300.signals import make_signal

    with pytest.raises(m.MpsftError) as e:
        ctx.upload(np.zeros(1000, np.complex64))  # composite, not a power of 2
    assert e.value.status == m.ERR_UNSUPPORTED_N
    sg = make_signal(1 << 14, 30, 1, sigma=1e-6)
    sig = ctx.upload(sg.x)
    with pytest.raises(m.MpsftError) as e:
        ctx.bin_in_time(sig, 100, 3, 1e-5, 3, 1, 1, 1)  # even bins
    assert e.value.status == m.ERR_INVALID
    with pytest.raises(m.MpsftError) as e:
        ctx.solve(sig, m.Rng(1), ctx.solve_options(30, 1e-6, trials=2))
    assert e.value.status == m.ERR_INVALID
    # iteration cap: stop with a status, never spin
    with pytest.raises(m.MpsftError) as e:
        ctx.solve(sig, m.Rng(1), ctx.solve_options(30, 1e-6, min_bins=51,
                                                  max_stale_iter=5, max_iter=1))
    assert e.value.status == m.ERR_ITER_CAP
    # mode table too small for what is found
    with pytest.raises(m.MpsftError) as e:
        ctx.solve(sig, m.Rng(1), ctx.solve_options(30, 1e-6, min_bins=51,
                                                  max_stale_iter=5,
                                                  mode_capacity=16))
    assert e.value.status == m.ERR_CAPACITY
    # a NaN in the signal is reported, not looped on
    bad = sg.x.copy()
    bad[::16] = np.nan
    sig2 = ctx.upload(bad)
    with pytest.raises(m.MpsftError) as e:
        ctx.solve(sig2, m.Rng(1), ctx.solve_options(30, 1e-6, min_bins=51,
                                                   max_stale_iter=5))
    assert e.value.status == m.ERR_NONFINITE
    # the context stays usable afterwards
    modes, _ = ctx.solve(sig, m.Rng(1), ctx.solve_options(30, 1e-6, min_bins=51,
                                                         max_stale_iter=5))
    assert len(modes) >= 30


@pytest.mark.parametrize("prec", PRECS, ids=PREC_IDS)
@pytest.mark.parametrize("name", ["more", "full"])
def test_iterate_statistics_match_reference(ctx, port, golden, name, prec):
    """The reference's statistical Iterate tests (src/iterate_test.cc:84-175)
    through mpsft_iterate: the signal is Demo1's construction from
    RandomSeed(123537) (built by the oracle; the library's RNG is advanced by
    the same draws, GenerateModeMap then 2n normals), then Iterate calls that
    continue the stream. Every call finds the reference's counts and the
    oracle's exact mode set. Coefficients: relative error (norm over the set)
    within 1e-6 (FP64) / 1e-2 (FP32); the largest per-mode deviations, 2.4e-7
    and 4.5e-3, are on modes the noisy scenario re-finds, whose sums are far
    below the unit modes."""
    spec = cases.ITERATE_MORE if name == "more" else cases.ITERATE_FULL
    counts, mm_o = cases.iterate_stats(port, spec)
    n = cases.ITERATE_STATS_N
    x, k, _ = port.demo_signal(n, 1000, spec["sigma"], 123537)
    truth = set(k.tolist())
    sig = ctx.upload(x)
    rng = m.Rng(123537)
    rng.mode_map(n, 1000)
    rng.normals(2 * n, keep=False)
    sigma = spec["sigma"]
    mm, got = {}, []
    for bins in spec["bins"]:
        if spec is cases.ITERATE_FULL:
            kw = dict(bin_threshold=3 * sigma / np.sqrt(bins),
                      sv_threshold=sigma / np.sqrt(bins))
        else:
            kw = dict(bin_threshold=0.01)
        _, mm = ctx.iterate(sig, rng, bins, window_delta=1e-6, trials=3,
                            window_threshold=0.1, mm=mm, precision=prec, **kw)
        good = sum(1 for kk in mm if kk in truth)
        got.append((good, len(mm) - good))
    sig.free()
    assert np.array_equal(np.array(got, np.int32), golden[f"iterstats_{name}"])
    assert sorted(mm) == sorted(mm_o)
    kk = sorted(mm_o)
    assert coef_err(mm, kk, [mm_o[q] for q in kk]) < (1e-6 if prec == m.FP64 else 1e-2)


def test_batched_result_layouts(ctx):
    """mpsft_solve_batched (one output pair per signal) and
    mpsft_solve_batched_packed (all signals in one pair, at offsets) give the
    same modes; a packed output too small for the last signal reports
    MPSFT_ERR_CAPACITY for it with its full count and a stored prefix, and
    the signals before it intact."""
    import ctypes
    from mpsft_gb300 import SolveOptions, Stats, _ptr
    from mpsft_gb300.signals import make_signal

    spec = [(1 << 16, 20, 3), (1 << 16, 35, 4), (65537, 15, 5)]
    sigs, opts = [], []
    for n, S, seed in spec:
        sg = make_signal(n, S, 900 + seed, sigma=1e-5)
        sigs.append(ctx.upload(sg.x))
        opts.append(ctx.solve_options(S, sg.sigma, min_bins=51, window_delta=1e-5))
    nsig = len(spec)
    lib = ctx._lib
    opt_arr = (SolveOptions * nsig)(*opts)
    sig_arr = (ctypes.c_void_p * nsig)(*[s._h.value for s in sigs])

    def rng_arr():
        rngs = [m.Rng(40 + i) for i in range(nsig)]
        return rngs, (ctypes.c_void_p * nsig)(*[r._h.value for r in rngs])

    cap = 4096
    ks = [np.zeros(cap, np.int32) for _ in range(nsig)]
    cs = [np.zeros(cap, np.complex128) for _ in range(nsig)]
    count = np.zeros(nsig, np.int32)
    rngs, ra = rng_arr()
    rc = lib.mpsft_solve_batched(
        ctx._h, sig_arr, opt_arr, nsig, ra,
        (ctypes.c_void_p * nsig)(*[k.ctypes.data for k in ks]),
        (ctypes.c_void_p * nsig)(*[c.ctypes.data for c in cs]),
        _ptr(np.full(nsig, cap, np.int32)), _ptr(count), (Stats * nsig)())
    assert rc == m.OK
    # packed, with room for all
    total = 3 * cap
    pk, pc = np.zeros(total, np.int32), np.zeros(total, np.complex128)
    offs, count2 = np.zeros(nsig + 1, np.int64), np.zeros(nsig, np.int32)
    rngs, ra = rng_arr()
    rc = lib.mpsft_solve_batched_packed(ctx._h, sig_arr, opt_arr, nsig, ra, _ptr(pk),
                                        _ptr(pc), total, _ptr(offs), _ptr(count2),
                                        (Stats * nsig)())
    assert rc == m.OK
    assert np.array_equal(count, count2)
    for i in range(nsig):
        a, b = int(offs[i]), int(offs[i + 1])
        assert b - a == count[i]
        assert np.array_equal(pk[a:b], ks[i][:count[i]])
        assert np.array_equal(pc[a:b].view(np.uint64), cs[i][:count[i]].view(np.uint64))
    # packed, one entry short of the last signal
    short = int(count[:-1].sum() + count[-1] - 1)
    offs3, count3 = np.zeros(nsig + 1, np.int64), np.zeros(nsig, np.int32)
    st3 = (Stats * nsig)()
    rngs, ra = rng_arr()
    rc = lib.mpsft_solve_batched_packed(ctx._h, sig_arr, opt_arr, nsig, ra, _ptr(pk),
                                        _ptr(pc), short, _ptr(offs3), _ptr(count3), st3)
    assert rc == m.ERR_CAPACITY
    assert np.array_equal(count3, count)
    assert [st3[i].status for i in range(nsig)] == [0, 0, m.ERR_CAPACITY]
    assert offs3[-1] == short and np.array_equal(offs3[:-1], offs[:-1])
    for s in sigs:
        s.free()
