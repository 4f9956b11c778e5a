"""The binning entry point that allocates nothing (mpsft_bin_in_time_noalloc).

It exists for callers that cannot call cudaMalloc, such as code running inside
a caller-managed memory pool or a plugin host that forbids allocation after
start-up: they pass their own device buffers for the samples and the bins, and
the library works in a fixed scratch array compiled into it. These tests call it
through the C ABI with device buffers owned by the test and compare its bins
with those of mpsft_bin_in_time (which allocates its own work buffers) on two
calls in a row (the second with other sizes, so stale scratch from the first
would show). Both entry points run the same kernels on the same descriptor,
window and twiddles, so the bins must be equal bit for bit: a tolerance would
hide an offset or stride fault in the array's hand-made layout.

This file is collected last on purpose: it runs after every other test.
"""
from __future__ import annotations

import ctypes

import numpy as np
import pytest

import cases
import mpsft_gb300 as m

pytestmark = pytest.mark.gpu


def _noalloc_fn(lib):
    fn = lib.mpsft_bin_in_time_noalloc
    fn.restype = ctypes.c_int
    fn.argtypes = [ctypes.c_void_p, ctypes.c_int64, ctypes.c_int, ctypes.c_int32,
                   ctypes.c_int32, ctypes.c_double, ctypes.c_int32, ctypes.c_int32,
                   ctypes.c_int32, ctypes.c_int32, ctypes.c_int, ctypes.c_void_p,
                   ctypes.c_void_p]
    return fn


def _noalloc_bins(fn, x_dev, n, dtype, bins, bits, delta, a, b, c, q, prec, stream):
    import torch

    out = torch.zeros((1 + 2 * bits, bins), dtype=torch.complex128, device="cuda")
    rc = fn(x_dev.data_ptr(), n, dtype, bins, bits, delta, a, b, c, q, prec,
            out.data_ptr(), stream.cuda_stream)
    assert rc == m.OK, rc
    stream.synchronize()
    return out.cpu().numpy()


@pytest.mark.parametrize("prec", [m.FP64, m.FP32], ids=["fp64", "fp32"])
def test_noalloc_matches_allocating_entry_point(ctx, prec):
    torch = pytest.importorskip("torch")
    lib = m.load_library()
    fn = _noalloc_fn(lib)
    stream = torch.cuda.Stream()
    calls = [
        # (n, bins, delta, a, b, c, q, seed, dtype)
        (1 << 20, 2001, 1e-5, 987653, 31337, 271828, 99991, 13, np.complex64),
        (65537, 101, 1e-6, 12345, 678, 910, 4444, 12, np.complex128),
    ]
    for n, bins, delta, a, b, c, q, seed, dt in calls:
        x = cases.random_signal(n, seed).astype(dt)
        dtype = m.C64 if dt == np.complex64 else m.C128
        bits = lib.mpsft_num_bits(n, bins)
        want = ctx.bin_in_time(ctx.upload(x), bins, bits, delta, a, b, c, q,
                               precision=prec)
        x_dev = torch.from_numpy(x).to("cuda")
        got = _noalloc_bins(fn, x_dev, n, dtype, bins, bits, delta, a, b, c, q,
                            prec, stream)
        assert np.array_equal(got, want), (
            n, bins, np.abs(got - want).max() / np.abs(want).max())


def test_noalloc_rejects_sizes_beyond_its_scratch(lib):
    torch = pytest.importorskip("torch")
    fn = _noalloc_fn(lib)
    x = torch.zeros(1 << 16, dtype=torch.complex64, device="cuda")
    out = torch.zeros((3, 4095), dtype=torch.complex128, device="cuda")
    rc = fn(x.data_ptr(), 1 << 16, m.C64, 4095, 1, 1e-5, 3, 1, 1, 1, m.FP32,
            out.data_ptr(), None)
    assert rc == m.ERR_CAPACITY
    rc = fn(x.data_ptr(), 1 << 16, m.C64, 101, 21, 1e-5, 3, 1, 1, 1, m.FP32,
            out.data_ptr(), None)
    assert rc == m.ERR_CAPACITY
    # the lengths of mpsft_bin_in_time: prime or a power of two
    rc = fn(x.data_ptr(), 60000, m.C64, 101, 2, 1e-5, 7, 1, 1, 1, m.FP32,
            out.data_ptr(), None)
    assert rc == m.ERR_UNSUPPORTED_N
