"""mpsft_gb300: GB300 (sm_103a) MPSFT recovery loop behind a C ABI.

This module is a thin ctypes binding of ``include/mpsft.h`` (the library is
``mpsft_gb300/_lib/libmpsft_gb300.so``, built by ``mpsft_gb300.build``). It
mirrors the reference's entry points (jiaweichiu/mpsft):

=====================  =========================================  ==============================
this module            reference                                  file:line
=====================  =========================================  ==============================
``bin_in_time``        ``BinInTime::Run``                         src/binner.h:30-41
``bin_in_freq``        ``BinInFreq::Run``                         src/binner.h:123-133
``mat_pencil``         ``MatPencil``                              src/freqid.h:28
``iterate``            ``Iterate``                                src/iterate.h:65
``solve``              ``Demo1::Run``                             src/demo1.cc:36-59
``Rng``                ``RandomSeed`` / ``RandomInt32``           src/base.cc:52-53
=====================  =========================================  ==============================

There is no CPU fallback: if the library is missing or no GPU is present, the
calls raise.
"""
from __future__ import annotations

import collections.abc
import ctypes
import os
import weakref
from dataclasses import dataclass, field

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_lib", "libmpsft_gb300.so")
# launch shapes of the FP32 binning chosen by the autotuner on GB300
# (python -m mpsft_gb300.tune); MPSFT_TUNING_FILE overrides, "none" disables
TUNING_PATH = os.path.join(_HERE, "tuning", "gb300_fold_shapes.tsv")

OK, ERR_INVALID, ERR_UNSUPPORTED_N, ERR_CUDA, ERR_CAPACITY, ERR_ITER_CAP, \
    ERR_NONFINITE, ERR_NOMEM = range(8)
C64, C128 = 1, 2
FP32, FP64, FP64_DIRECT = 0, 1, 2


class MpsftError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"mpsft status {status}: {msg}")
        self.status = status


class IterateOptions(ctypes.Structure):
    _fields_ = [("bins", ctypes.c_int32), ("window_delta", ctypes.c_double),
                ("trials", ctypes.c_int32), ("bin_threshold", ctypes.c_double),
                ("window_threshold", ctypes.c_double),
                ("sv_threshold", ctypes.c_double), ("precision", ctypes.c_int32),
                ("near_tie_margin", ctypes.c_double)]


class SolveOptions(ctypes.Structure):
    _fields_ = [("k", ctypes.c_int32), ("sigma", ctypes.c_double),
                ("trials", ctypes.c_int32), ("min_bins", ctypes.c_int32),
                ("window_delta", ctypes.c_double),
                ("window_threshold", ctypes.c_double),
                ("max_stale_iter", ctypes.c_int32), ("max_iter", ctypes.c_int32),
                ("precision", ctypes.c_int32), ("mode_capacity", ctypes.c_int32),
                ("near_tie_margin", ctypes.c_double)]


class EstimateSetup(ctypes.Structure):
    """The transform and shape of a fixed-set coefficient estimate."""
    _fields_ = [("bins", ctypes.c_int32), ("bits", ctypes.c_int32),
                ("trials", ctypes.c_int32), ("window_delta", ctypes.c_double),
                ("a", ctypes.c_int32), ("b", ctypes.c_int32), ("c", ctypes.c_int32),
                ("q", ctypes.c_int32 * 15)]


class Analysis(ctypes.Structure):
    """mpsft_analysis: Demo1::PostAnalyze's figures (src/demo1.cc:61-112)."""
    _fields_ = [("hit", ctypes.c_int32), ("miss", ctypes.c_int32),
                ("hit_l1", ctypes.c_double), ("hit_l2", ctypes.c_double),
                ("miss_l1", ctypes.c_double), ("miss_l2", ctypes.c_double),
                ("l1", ctypes.c_double), ("l2", ctypes.c_double),
                ("max_err", ctypes.c_double)]

    def as_dict(self) -> dict:
        return {name: getattr(self, name) for name, _ in self._fields_}


class BinLaunch(ctypes.Structure):
    """One timed binning launch (mpsft_bin_launch)."""
    _fields_ = [("iteration", ctypes.c_int32), ("signals", ctypes.c_int32),
                ("max_bins", ctypes.c_int32), ("min_bins", ctypes.c_int32),
                ("precision", ctypes.c_int32),
                ("gathers", ctypes.c_int64), ("bytes", ctypes.c_int64),
                ("ms", ctypes.c_double)]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


class Stats(ctypes.Structure):
    _fields_ = [("iterations", ctypes.c_int32), ("found", ctypes.c_int32),
                ("gathers", ctypes.c_int64), ("bin_bytes", ctypes.c_int64),
                ("bin_launches", ctypes.c_int32), ("bin_ms", ctypes.c_double),
                ("escalated", ctypes.c_int32), ("status", ctypes.c_int32),
                ("kernel_launches", ctypes.c_int64), ("unresolved", ctypes.c_int32),
                ("fp64_iterations", ctypes.c_int32), ("loop_ms", ctypes.c_double)]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


class BatchStats(collections.abc.Sequence):
    """The Stats of a batched solve, one dict per signal, made when read (a
    caller that drops them, or reads a few, pays no conversion of the rest)."""

    def __init__(self, arr):
        self._arr = arr

    def __len__(self) -> int:
        return len(self._arr)

    def __getitem__(self, i):
        if isinstance(i, slice):
            return [self._arr[j].as_dict() for j in range(*i.indices(len(self._arr)))]
        return self._arr[i].as_dict()

    def __eq__(self, other) -> bool:
        return list(self) == list(other)

    def __repr__(self) -> str:
        return repr(list(self))


_lib = None


def load_library(path: str | None = None) -> ctypes.CDLL:
    """Loads the CUDA library; raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or LIB_PATH
    if not os.path.exists(path):
        raise FileNotFoundError(
            f"{path} is missing: build it with `python -m mpsft_gb300.build`")
    lib = ctypes.CDLL(path)
    P = ctypes.c_void_p
    I32, I64, D, I = ctypes.c_int32, ctypes.c_int64, ctypes.c_double, ctypes.c_int
    PP = ctypes.POINTER(ctypes.c_void_p)
    sigs = {
        "mpsft_ctx_create": (I, [I, PP]),
        "mpsft_ctx_destroy": (I, [P]),
        "mpsft_ctx_set_stream": (I, [P, P]),
        "mpsft_ctx_set_profiling": (I, [P, I]),
        "mpsft_ctx_bin_launches": (I, [P, P, I32, P]),
        "mpsft_fold_shape_count": (I32, []),
        "mpsft_ctx_set_timeline": (I, [P, I]),
        "mpsft_ctx_timeline": (I, [P, P, P, I32, P]),
        "mpsft_ctx_set_fold_shape": (I, [P, I32]),
        "mpsft_autotune": (I, [P, P, ctypes.POINTER(SolveOptions), I32, I32, I32]),
        "mpsft_tuning_save": (I, [P, ctypes.c_char_p]),
        "mpsft_tuning_load": (I, [P, ctypes.c_char_p]),
        "mpsft_tuning_size": (I32, [P]),
        "mpsft_last_error": (ctypes.c_char_p, [P]),
        "mpsft_status_string": (ctypes.c_char_p, [I]),
        "mpsft_rng_create": (I, [I32, PP]),
        "mpsft_rng_destroy": (I, [P]),
        "mpsft_rng_seed": (I, [P, I32]),
        "mpsft_rng_seed_many": (I, [P, P, I32]),
        "mpsft_rng_int32": (I32, [P]),
        "mpsft_rng_normals": (I, [P, I64, P]),
        "mpsft_num_bits": (I32, [I32, I32]),
        "mpsft_window_support": (I32, [I32, I32, D]),
        "mpsft_window_table": (I, [P, I32, I32, D, P, I32]),
        "mpsft_signal_upload": (I, [P, P, I64, I, PP]),
        "mpsft_signal_wrap_device": (I, [P, P, I64, I, PP]),
        "mpsft_signal_free": (I, [P]),
        "mpsft_signal_write": (I, [P, P, P]),
        "mpsft_signal_write_many": (I, [P, P, P, I32, P]),
        "mpsft_signal_read": (I, [P, P, P]),
        "mpsft_bin_in_time": (I, [P, P, I32, I32, D, I32, I32, I32, I32, I, P, I]),
        "mpsft_bin_in_freq": (I, [P, I32, I32, I32, D, I32, I32, I32, I32, P, P,
                                  I64, P]),
        "mpsft_bin_in_time_wt": (I, [P, P, I32, I32, I32, P, I32, I32, I32, I32, I,
                                     P, I]),
        "mpsft_bin_in_freq_wf": (I, [P, I32, I32, I32, I32, I32, I32, I32, P, P, P,
                                     I64, P]),
        "mpsft_iterate_draws": (I, [P, P, ctypes.POINTER(IterateOptions), I32, I32,
                                    I32, I32, P, P, P, P, I32, P]),
        "mpsft_mat_pencil": (I, [P, P, I64, P, P]),
        "mpsft_estimate": (I, [P, P, ctypes.POINTER(EstimateSetup), P, I64, P]),
        "mpsft_adjoint": (I, [P, I32, ctypes.POINTER(EstimateSetup), P, I64, P, P]),
        "mpsft_iterate": (I, [P, P, ctypes.POINTER(IterateOptions), P, P, P, P,
                              I32, P]),
        "mpsft_solve_options_default": (None, [ctypes.POINTER(SolveOptions)]),
        "mpsft_solve": (I, [P, P, ctypes.POINTER(SolveOptions), P, P, P, I32, P,
                            ctypes.POINTER(Stats)]),
        "mpsft_solve_batched": (I, [P, P, ctypes.POINTER(SolveOptions), I32, P, P,
                                    P, P, P, ctypes.POINTER(Stats)]),
        "mpsft_solve_batched_packed": (I, [P, P, ctypes.POINTER(SolveOptions), I32, P,
                                           P, P, I64, P, P, ctypes.POINTER(Stats)]),
        "mpsft_generate_mode_map": (I, [P, I32, I32, P, P]),
        "mpsft_signal_generate": (I, [P, I64, P, P, I64, D, ctypes.c_uint64, I, PP]),
        "mpsft_signal_spectrum": (I, [P, P, P]),
        "mpsft_post_analyze": (I, [P, P, P, I64, P, P, I64,
                                   ctypes.POINTER(Analysis)]),
    }
    for name, (res, args) in sigs.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def num_bits(n: int, bins: int) -> int:
    """NumBits (src/iterate.cc:30-42): halvings of n while n >= bins."""
    return int(load_library().mpsft_num_bits(int(n), int(bins)))


def exported_symbols() -> list[str]:
    """Names declared in include/mpsft.h (used by the load test)."""
    import re
    hdr = os.path.join(os.path.dirname(_HERE), "include", "mpsft.h")
    txt = open(hdr).read()
    decl = r"(?m)^(?:int|int32_t|void|const char\s*\*)\s*\*?\s*(mpsft_[a-z0-9_]+)\s*\("
    return sorted(set(re.findall(decl, txt)))


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(ctypes.c_void_p)


class Rng:
    """The reference's global RNG made explicit (std::mt19937 +
    uniform_int_distribution<int32_t>); Rng(123534) is MainInit's state."""

    def __init__(self, seed: int = 123534):
        lib = load_library()
        h = ctypes.c_void_p()
        _check(None, lib.mpsft_rng_create(int(seed), ctypes.byref(h)))
        self._h = h
        self._lib = lib

    def seed(self, s: int) -> None:
        self._lib.mpsft_rng_seed(self._h, int(s))

    @staticmethod
    def seed_many(rngs: list, seeds) -> None:
        """Reseeds rngs[i] with seeds[i] in one call."""
        seeds = np.ascontiguousarray(seeds, np.int32)
        if seeds.size != len(rngs):
            raise ValueError("one seed per generator")
        arr = (ctypes.c_void_p * len(rngs))(*[r._h.value for r in rngs])
        _check(None, load_library().mpsft_rng_seed_many(arr, _ptr(seeds), len(rngs)))

    def int32(self) -> int:
        return int(self._lib.mpsft_rng_int32(self._h))

    def normals(self, count: int, keep: bool = True):
        """count RandomNormal draws (returned, or only consumed)."""
        out = np.empty(count if keep else 0, np.float64)
        _check(None, self._lib.mpsft_rng_normals(self._h, int(count),
                                                 _ptr(out) if keep else None))
        return out if keep else None

    def mode_map(self, n: int, count: int):
        """GenerateModeMap (src/gen.cc:27-39) from this RNG: (positions in
        draw order, unit-modulus complex128 coefficients)."""
        k = np.zeros(count, np.int32)
        c = np.zeros(count, np.complex128)
        _check(None, self._lib.mpsft_generate_mode_map(self._h, int(n), int(count),
                                                       _ptr(k), _ptr(c)))
        return k, c

    def __del__(self):
        if getattr(self, "_h", None):
            self._lib.mpsft_rng_destroy(self._h)
            self._h = None


def _check(ctx, rc: int) -> None:
    if rc != OK:
        lib = load_library()
        msg = lib.mpsft_last_error(ctx._h).decode() if ctx is not None else \
            lib.mpsft_status_string(rc).decode()
        raise MpsftError(rc, msg)


class Context:
    """One CUDA device, one stream, reusable work buffers."""

    def __init__(self, device: int = 0):
        lib = load_library()
        h = ctypes.c_void_p()
        rc = lib.mpsft_ctx_create(int(device), ctypes.byref(h))
        if rc != OK:
            raise MpsftError(rc, "mpsft_ctx_create failed (is a GPU present?)")
        self._h = h
        self._lib = lib
        # grow-only host buffers that batched solves write their modes into
        self._out_k = np.empty(0, np.int32)
        self._out_c = np.empty(0, np.complex128)
        # live signals of this context: freed before the context itself
        self._signals = weakref.WeakSet()
        tuning = os.environ.get("MPSFT_TUNING_FILE", TUNING_PATH)
        if tuning != "none" and os.path.exists(tuning):
            self.tuning_load(tuning)

    # ---- launch shapes of the FP32 binning (autotuner) ----------------------
    def autotune(self, sigs: list, opts: list, seed: int = 4242, repeats: int = 2) -> None:
        """Times every launch shape of the FP32 binning on one batched solve of
        these signals and records the fastest per bins class (mpsft_autotune)."""
        nsig = len(sigs)
        sig_arr = (ctypes.c_void_p * nsig)(*[s_._h.value for s_ in sigs])
        opt_arr = (SolveOptions * nsig)(*opts)
        _check(self, self._lib.mpsft_autotune(self._h, sig_arr, opt_arr, nsig,
                                              int(seed), int(repeats)))

    def tuning_save(self, path: str) -> None:
        _check(self, self._lib.mpsft_tuning_save(self._h, path.encode()))

    def tuning_load(self, path: str) -> None:
        _check(self, self._lib.mpsft_tuning_load(self._h, path.encode()))

    def tuning_size(self) -> int:
        return int(self._lib.mpsft_tuning_size(self._h))

    def set_timeline(self, on: bool) -> None:
        """Record the device clock at the end of every solve-graph iteration."""
        _check(self, self._lib.mpsft_ctx_set_timeline(self._h, int(bool(on))))

    TIMELINE_KERNELS = {1: "plan", 2: "window32", 3: "fold", 4: "bluestein",
                        5: "mode_prep", 6: "bucket", 7: "row_fft", 8: "decide",
                        9: "listed_terms", 10: "merge", 11: "rebin",
                        12: "decide_listed", 13: "finish", 14: "window64"}

    def timeline(self):
        """The last solve graph's kernel starts: (kernel ids, microseconds
        after the first), in start order."""
        count = np.zeros(1, np.int32)
        _check(self, self._lib.mpsft_ctx_timeline(self._h, None, None, 0, _ptr(count)))
        ids = np.zeros(int(count[0]), np.int32)
        us = np.zeros(int(count[0]), np.float64)
        _check(self, self._lib.mpsft_ctx_timeline(self._h, _ptr(ids), _ptr(us),
                                                  ids.size, _ptr(count)))
        return ids, us

    def set_fold_shape(self, shape: int) -> None:
        """Forces one FP32 binning launch shape (-1: the tuning table's)."""
        _check(self, self._lib.mpsft_ctx_set_fold_shape(self._h, int(shape)))

    def close(self) -> None:
        if getattr(self, "_h", None):
            for sg in list(getattr(self, "_signals", ())):
                sg.free()
            self._lib.mpsft_ctx_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()

    def set_stream(self, stream_handle: int | None) -> None:
        _check(self, self._lib.mpsft_ctx_set_stream(
            self._h, ctypes.c_void_p(stream_handle or 0)))

    def set_profiling(self, on: bool) -> None:
        _check(self, self._lib.mpsft_ctx_set_profiling(self._h, int(bool(on))))

    def bin_launches(self) -> list[dict]:
        """The timed binning launches of the last call made with profiling
        on (mpsft_ctx_bin_launches), in launch order."""
        count = np.zeros(1, np.int32)
        _check(self, self._lib.mpsft_ctx_bin_launches(self._h, None, 0, _ptr(count)))
        recs = (BinLaunch * max(1, int(count[0])))()
        _check(self, self._lib.mpsft_ctx_bin_launches(self._h, recs, int(count[0]),
                                                      _ptr(count)))
        return [recs[j].as_dict() for j in range(int(count[0]))]

    # ---- signals --------------------------------------------------------
    def upload(self, x: np.ndarray) -> "Signal":
        x = np.ascontiguousarray(x)
        if x.dtype == np.complex64:
            dt = C64
        elif x.dtype == np.complex128:
            dt = C128
        else:
            raise TypeError("x must be complex64 or complex128")
        h = ctypes.c_void_p()
        _check(self, self._lib.mpsft_signal_upload(self._h, _ptr(x), x.size, dt,
                                                   ctypes.byref(h)))
        sg = Signal(self, h, x.size, dt)
        self._signals.add(sg)
        return sg

    def wrap_device(self, ptr: int, n: int, dtype: int) -> "Signal":
        h = ctypes.c_void_p()
        _check(self, self._lib.mpsft_signal_wrap_device(
            self._h, ctypes.c_void_p(ptr), int(n), int(dtype), ctypes.byref(h)))
        sg = Signal(self, h, n, dtype)
        self._signals.add(sg)
        return sg

    def generate(self, n: int, k, coef, sigma: float, seed: int,
                 dtype: int = C64) -> "Signal":
        """A signal made on the device: sum_j coef_j e^{2 pi i k_j t/n} plus
        complex Gaussian noise of per-sample variance sigma^2 from a
        counter-based generator keyed by seed (mpsft_signal_generate)."""
        k = np.ascontiguousarray(k, np.int32)
        c = np.ascontiguousarray(coef, np.complex128)
        if k.size != c.size:
            raise ValueError("one coefficient per position")
        h = ctypes.c_void_p()
        _check(self, self._lib.mpsft_signal_generate(
            self._h, int(n), _ptr(k), _ptr(c), k.size, float(sigma),
            ctypes.c_uint64(int(seed) & (2**64 - 1)), int(dtype), ctypes.byref(h)))
        sg = Signal(self, h, int(n), int(dtype))
        self._signals.add(sg)
        return sg

    def spectrum(self, sig: "Signal") -> np.ndarray:
        """xhat = FFT(x) / n in FP64, computed on the device."""
        out = np.empty(sig.n, np.complex128)
        _check(self, self._lib.mpsft_signal_spectrum(self._h, sig._h, _ptr(out)))
        return out

    def post_analyze(self, sig: "Signal", true_k, found_k, found_c) -> dict:
        """Demo1::PostAnalyze (src/demo1.cc:61-112) on the device against the
        signal's spectrum FFT(x)/n."""
        tk = np.ascontiguousarray(true_k, np.int32)
        fk = np.ascontiguousarray(found_k, np.int32)
        fc = np.ascontiguousarray(found_c, np.complex128)
        if fk.size != fc.size:
            raise ValueError("one coefficient per found position")
        a = Analysis()
        _check(self, self._lib.mpsft_post_analyze(self._h, sig._h, _ptr(tk), tk.size,
                                                  _ptr(fk), _ptr(fc), fk.size,
                                                  ctypes.byref(a)))
        return a.as_dict()

    def write_many(self, sigs: list, xs: list, stream_handle: int | None = None) -> None:
        """Refills many signals from host arrays (pinned memory for an
        asynchronous copy) on the given CUDA stream (None = the context's).
        Safe to call from a second thread while a solve of this context runs,
        when it names its own stream; order the solve after it with an event."""
        if len(sigs) != len(xs):
            raise ValueError("one host array per signal")
        for sg, x in zip(sigs, xs):
            want = np.complex64 if sg.dtype == C64 else np.complex128
            if sg.ctx is not self or x.dtype != want or x.size != sg.n or \
                    not x.flags.c_contiguous:
                raise ValueError("x must match its signal's context, n and dtype")
        nsig = len(sigs)
        sig_arr = (ctypes.c_void_p * nsig)(*[s._h.value for s in sigs])
        x_arr = (ctypes.c_void_p * nsig)(*[x.ctypes.data for x in xs])
        _check(None, self._lib.mpsft_signal_write_many(
            self._h, sig_arr, x_arr, nsig, ctypes.c_void_p(stream_handle or 0)))

    # ---- operators -------------------------------------------------------
    def window_table(self, n: int, bins: int, delta: float) -> np.ndarray:
        p = int(self._lib.mpsft_window_support(n, bins, delta))
        if p <= 0:
            raise MpsftError(ERR_INVALID, "bad window arguments")
        wt = np.zeros(p, np.float64)
        _check(self, self._lib.mpsft_window_table(self._h, n, bins, delta, _ptr(wt), p))
        return wt

    def bin_in_time(self, sig: "Signal", bins: int, bits: int, delta: float,
                    a: int, b: int, c: int, q: int,
                    precision: int = FP32) -> np.ndarray:
        out = np.zeros((1 + 2 * bits, bins), np.complex128)
        _check(self, self._lib.mpsft_bin_in_time(
            self._h, sig._h, bins, bits, delta, a, b, c, q, precision, _ptr(out), 0))
        return out

    def bin_in_time_wt(self, sig: "Signal", bins: int, bits: int, wt: np.ndarray,
                       a: int, b: int, c: int, q: int,
                       precision: int = FP32) -> np.ndarray:
        """BinInTime::Run windowed by a Window's own table wt (p entries, the
        reference's index order t = 0, 1..p2, -p2..-1)."""
        wt = np.ascontiguousarray(wt, np.float64)
        out = np.zeros((1 + 2 * bits, bins), np.complex128)
        _check(self, self._lib.mpsft_bin_in_time_wt(
            self._h, sig._h, bins, bits, wt.size, _ptr(wt), a, b, c, q, precision,
            _ptr(out), 0))
        return out

    def bin_in_freq_wf(self, out: np.ndarray, n: int, bins: int, bits: int,
                       a: int, b: int, c: int, q: int, k0: np.ndarray,
                       coef: np.ndarray, wf: np.ndarray) -> np.ndarray:
        """BinInFreq::Run with each mode's window response wf given."""
        out = np.ascontiguousarray(out, np.complex128).copy()
        k0 = np.ascontiguousarray(k0, np.int32)
        coef = np.ascontiguousarray(coef, np.complex128)
        wf = np.ascontiguousarray(wf, np.float64)
        _check(self, self._lib.mpsft_bin_in_freq_wf(
            self._h, n, bins, bits, a, b, c, q, _ptr(k0), _ptr(coef), _ptr(wf),
            k0.size, _ptr(out)))
        return out

    def bin_in_freq(self, out: np.ndarray, n: int, bins: int, bits: int,
                    delta: float, a: int, b: int, c: int, q: int,
                    k0: np.ndarray, coef: np.ndarray) -> np.ndarray:
        out = np.ascontiguousarray(out, np.complex128).copy()
        k0 = np.ascontiguousarray(k0, np.int32)
        coef = np.ascontiguousarray(coef, np.complex128)
        _check(self, self._lib.mpsft_bin_in_freq(
            self._h, n, bins, bits, delta, a, b, c, q, _ptr(k0), _ptr(coef),
            k0.size, _ptr(out)))
        return out

    @staticmethod
    def estimate_setup(bins: int, bits: int, delta: float, a: int, b: int, c: int,
                       q) -> EstimateSetup:
        s = EstimateSetup()
        s.bins, s.bits, s.window_delta = bins, bits, delta
        s.a, s.b, s.c = a, b, c
        q = list(q)
        s.trials = len(q)
        for i, v in enumerate(q):
            s.q[i] = int(v)
        return s

    def estimate(self, sig: "Signal", setup: EstimateSetup,
                 k0: np.ndarray) -> np.ndarray:
        """Coefficient estimate of the fixed set k0 (a linear map of x)."""
        k0 = np.ascontiguousarray(k0, np.int32)
        out = np.zeros(k0.size, np.complex128)
        _check(self, self._lib.mpsft_estimate(self._h, sig._h, ctypes.byref(setup),
                                              _ptr(k0), k0.size, _ptr(out)))
        return out

    def adjoint(self, n: int, setup: EstimateSetup, k0: np.ndarray,
                g: np.ndarray) -> np.ndarray:
        """A^H g for the estimate of k0 (complex128, n entries)."""
        k0 = np.ascontiguousarray(k0, np.int32)
        g = np.ascontiguousarray(g, np.complex128)
        out = np.zeros(n, np.complex128)
        _check(self, self._lib.mpsft_adjoint(self._h, n, ctypes.byref(setup),
                                             _ptr(k0), k0.size, _ptr(g), _ptr(out)))
        return out

    def mat_pencil(self, u: np.ndarray):
        """u: (count, 3) complex128 rows (u0, u1, u2). Returns (sigma, vote)."""
        u = np.ascontiguousarray(u, np.complex128).reshape(-1, 3)
        sig = np.zeros((u.shape[0], 2), np.float64)
        vote = np.zeros(u.shape[0], np.int32)
        _check(self, self._lib.mpsft_mat_pencil(self._h, _ptr(u), u.shape[0],
                                                _ptr(sig), _ptr(vote)))
        return sig, vote.astype(bool)

    def iterate(self, sig: "Signal", rng: Rng, bins: int,
                window_delta: float = 1e-6, trials: int = 1,
                bin_threshold: float = 0.0, window_threshold: float = 0.1,
                sv_threshold: float = 0.0, mm: dict | None = None,
                precision: int = FP32):
        mm = dict(mm or {})
        cap = len(mm) + bins + 16
        k = np.zeros(cap, np.int32)
        c = np.zeros(cap, np.complex128)
        for i, (kk, cc) in enumerate(mm.items()):
            k[i] = kk
            c[i] = cc
        size = np.array([len(mm)], np.int32)
        found = np.zeros(1, np.int32)
        opt = IterateOptions(bins, window_delta, trials, bin_threshold,
                             window_threshold, sv_threshold, precision, 0.0)
        _check(self, self._lib.mpsft_iterate(self._h, sig._h, ctypes.byref(opt),
                                             rng._h, _ptr(k), _ptr(c), _ptr(size),
                                             cap, _ptr(found)))
        m = int(size[0])
        return bool(found[0]), {int(k[i]): complex(c[i]) for i in range(m)}

    def iterate_draws(self, sig: "Signal", a: int, b: int, c: int, a_inv: int,
                      q, bins: int, window_delta: float = 1e-6,
                      bin_threshold: float = 0.0, window_threshold: float = 0.1,
                      sv_threshold: float = 0.0, mm: dict | None = None,
                      precision: int = FP32):
        """Iterate on the caller's draws: transform (a, b, c, a_inv) and one q
        per trial (trials = len(q))."""
        mm = dict(mm or {})
        cap = len(mm) + bins + 16
        k = np.zeros(cap, np.int32)
        cc = np.zeros(cap, np.complex128)
        for i, (kk, v) in enumerate(mm.items()):
            k[i] = kk
            cc[i] = v
        qq = np.ascontiguousarray(q, np.int32)
        size = np.array([len(mm)], np.int32)
        found = np.zeros(1, np.int32)
        opt = IterateOptions(bins, window_delta, qq.size, bin_threshold,
                             window_threshold, sv_threshold, precision, 0.0)
        _check(self, self._lib.mpsft_iterate_draws(
            self._h, sig._h, ctypes.byref(opt), a, b, c, a_inv, _ptr(qq), _ptr(k),
            _ptr(cc), _ptr(size), cap, _ptr(found)))
        m = int(size[0])
        return bool(found[0]), {int(k[i]): complex(cc[i]) for i in range(m)}

    @staticmethod
    def solve_options(k: int, sigma: float, **kw) -> SolveOptions:
        o = SolveOptions()
        load_library().mpsft_solve_options_default(ctypes.byref(o))
        o.k = k
        o.sigma = sigma
        for name, v in kw.items():
            setattr(o, name, v)
        return o

    def solve(self, sig: "Signal", rng: Rng, opt: SolveOptions,
              cap: int | None = None):
        """Demo1::Run. Returns (modes dict, Stats)."""
        cap = cap or (4 * opt.k + 4096)
        k = np.zeros(cap, np.int32)
        c = np.zeros(cap, np.complex128)
        count = np.zeros(1, np.int32)
        st = Stats()
        _check(self, self._lib.mpsft_solve(self._h, sig._h, ctypes.byref(opt),
                                           rng._h, _ptr(k), _ptr(c), cap,
                                           _ptr(count), ctypes.byref(st)))
        m = int(count[0])
        return {int(k[i]): complex(c[i]) for i in range(m)}, st

    def solve_arrays(self, sig: "Signal", rng: Rng, opt: SolveOptions,
                     cap: int | None = None):
        """Like solve but returns (k int32 array, coef complex128 array, Stats)."""
        cap = cap or (4 * opt.k + 4096)
        k = np.zeros(cap, np.int32)
        c = np.zeros(cap, np.complex128)
        count = np.zeros(1, np.int32)
        st = Stats()
        _check(self, self._lib.mpsft_solve(self._h, sig._h, ctypes.byref(opt),
                                           rng._h, _ptr(k), _ptr(c), cap,
                                           _ptr(count), ctypes.byref(st)))
        m = int(count[0])
        return k[:m], c[:m], st

    def solve_batched(self, sigs: list, rngs: list, opts: list,
                      cap: int | None = None, raise_on_error: bool = True):
        """Many Demo1::Run solves advanced together. Returns
        (list of (k, coef) arrays, sequence of Stats dicts: BatchStats)."""
        nsig = len(sigs)
        total = sum(cap or (4 * o.k + 4096) for o in opts)
        if self._out_k.size < total:
            self._out_k = np.empty(total, np.int32)
            self._out_c = np.empty(total, np.complex128)
        count = np.zeros(nsig, np.int32)
        offs = np.zeros(nsig + 1, np.int64)
        stats = (Stats * nsig)()
        opt_arr = (SolveOptions * nsig)(*opts)
        sig_arr = (ctypes.c_void_p * nsig)(*[s._h.value for s in sigs])
        rng_arr = (ctypes.c_void_p * nsig)(*[r._h.value for r in rngs])
        rc = self._lib.mpsft_solve_batched_packed(
            self._h, sig_arr, opt_arr, nsig, rng_arr, _ptr(self._out_k),
            _ptr(self._out_c), total, _ptr(offs), _ptr(count), stats)
        if raise_on_error:
            _check(self, rc)
        # one copy of the packed results, handed out as one view per signal
        used = int(offs[-1])
        ks, cs = self._out_k[:used].copy(), self._out_c[:used].copy()
        bounds = offs.tolist()
        out = [(ks[a:b], cs[a:b]) for a, b in zip(bounds[:-1], bounds[1:])]
        return out, BatchStats(stats)


@dataclass(eq=False)
class Signal:
    ctx: Context
    _h: ctypes.c_void_p
    n: int
    dtype: int
    _freed: bool = field(default=False)

    def write(self, x: np.ndarray) -> None:
        """Refills the device copy from host memory (same n and dtype)."""
        want = np.complex64 if self.dtype == C64 else np.complex128
        if x.dtype != want or x.size != self.n or not x.flags.c_contiguous:
            raise ValueError("x must match the signal's n and dtype")
        _check(self.ctx, self.ctx._lib.mpsft_signal_write(self.ctx._h, self._h,
                                                          _ptr(x)))

    def read(self) -> np.ndarray:
        """The samples, copied to a new host array."""
        x = np.empty(self.n, np.complex64 if self.dtype == C64 else np.complex128)
        _check(self.ctx, self.ctx._lib.mpsft_signal_read(self.ctx._h, self._h, _ptr(x)))
        return x

    def free(self) -> None:
        if not self._freed and self._h:
            self.ctx._lib.mpsft_signal_free(self._h)
            self._freed = True

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass
