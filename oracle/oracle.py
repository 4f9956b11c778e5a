"""ctypes wrapper over the two CPU oracles (test infrastructure only).

Only tests, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` import this module, and only as the checker / CPU baseline; the
product path (``mpsft_gb300``) never does.

* ``Oracle("port")`` loads ``oracle/liboracle.so``, this project's restatement
  of the reference algorithm (``oracle/mpsft_oracle.cc``). It is built from
  this directory on any host (``make liboracle``).
* ``Oracle("port_fast")`` loads ``oracle/liboracle_fast.so``, the same
  restatement built with the reference's optimised flags (-O3 -ffast-math,
  ``make liboracle_fast``): for timing the CPU baseline only.
* ``Oracle("ref")`` / ``Oracle("ref_pow2")`` load ``oracle/_ref/libref*.so``,
  the reference's own sources compiled here against stand-in headers
  (``make ref``); they exist only where the reference tree was present at
  build time.

Both expose the C interface in ``oracle_capi.h``. Complex arrays are numpy
``complex128``; bin matrices have shape ``(1 + 2*bits, bins)``.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
_LIBS = {
    "port": os.path.join(HERE, "liboracle.so"),
    "port_fast": os.path.join(HERE, "liboracle_fast.so"),
    "ref": os.path.join(HERE, "_ref", "libref.so"),
    "ref_pow2": os.path.join(HERE, "_ref", "libref_pow2.so"),
}

_i32 = ctypes.c_int32
_dbl = ctypes.c_double
_int = ctypes.c_int
_p = ctypes.c_void_p


def build_port() -> str:
    """Compile oracle/liboracle.so (g++ only)."""
    subprocess.run(["make", "-s", "-C", HERE, "liboracle"], check=True)
    return _LIBS["port"]


def build_port_fast() -> str:
    """Compile oracle/liboracle_fast.so (g++ only; CPU-baseline timing)."""
    subprocess.run(["make", "-s", "-C", HERE, "liboracle_fast"], check=True)
    return _LIBS["port_fast"]


def available(kind: str) -> bool:
    return os.path.exists(_LIBS[kind])


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(_p)


class Oracle:
    def __init__(self, kind: str = "port"):
        path = _LIBS[kind]
        if not os.path.exists(path):
            raise FileNotFoundError(f"oracle library {path} is not built")
        self.kind = kind
        lib = ctypes.CDLL(path)
        sig = {
            "orc_seed": (None, [_i32]),
            "orc_random_int32": (_i32, []),
            "orc_random_normal": (_dbl, []),
            "orc_num_bits": (_i32, [_i32, _i32]),
            "orc_window": (_i32, [_i32, _i32, _dbl, _p, _i32]),
            "orc_window_sample_in_freq": (_dbl, [_i32, _i32, _dbl, _dbl]),
            "orc_transform": (None, [_i32, _p]),
            "orc_transform_inverse": (_i32, [_i32, _i32]),
            "orc_bin_in_time": (_int, [_int, _i32, _i32, _i32, _dbl, _i32, _i32,
                                       _i32, _i32, _p, _p]),
            "orc_bin_in_freq": (_int, [_int, _i32, _i32, _i32, _dbl, _i32, _i32,
                                       _i32, _i32, _p, _p, _i32, _p]),
            "orc_mat_pencil": (_int, [_p, _p]),
            "orc_iterate": (_int, [_i32, _p, _i32, _dbl, _i32, _dbl, _dbl, _dbl,
                                   _int, _int, _p, _p, _p, _i32]),
            "orc_demo1_run": (_int, [_i32, _p, _i32, _dbl, _i32, _i32, _dbl,
                                     _dbl, _i32, _i32, _p, _p, _i32, _p]),
            "orc_generate_mode_map": (_int, [_i32, _i32, _p, _p]),
            "orc_post_analyze": (None, [_i32, _p, _p, _i32, _p, _p, _i32, _p]),
            "orc_demo_signal": (_int, [_i32, _i32, _dbl, _int, _p, _p, _p]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        self.lib = lib

    # --- RNG -------------------------------------------------------------
    def seed(self, s: int) -> None:
        self.lib.orc_seed(int(s))

    def random_int32(self) -> int:
        return int(self.lib.orc_random_int32())

    def random_normal(self) -> float:
        return float(self.lib.orc_random_normal())

    # --- primitives --------------------------------------------------------
    def num_bits(self, n: int, bins: int) -> int:
        return int(self.lib.orc_num_bits(n, bins))

    def window(self, n: int, bins: int, delta: float) -> np.ndarray:
        p = int(self.lib.orc_window(n, bins, delta, None, 0))
        wt = np.zeros(p, np.float64)
        self.lib.orc_window(n, bins, delta, _ptr(wt), p)
        return wt

    def sample_in_freq(self, n: int, bins: int, delta: float, xi: float) -> float:
        return float(self.lib.orc_window_sample_in_freq(n, bins, delta, xi))

    def transform(self, n: int):
        out = np.zeros(4, np.int32)
        self.lib.orc_transform(n, _ptr(out))
        return tuple(int(v) for v in out)

    def transform_inverse(self, n: int, a: int) -> int:
        return int(self.lib.orc_transform_inverse(n, a))

    # --- operators ---------------------------------------------------------
    def bin_in_time(self, x: np.ndarray, bins: int, bits: int, delta: float,
                    a: int, b: int, c: int, q: int, btype: int = 4) -> np.ndarray:
        x = np.ascontiguousarray(x, np.complex128)
        out = np.zeros((1 + 2 * bits, bins), np.complex128)
        rc = self.lib.orc_bin_in_time(btype, x.size, bins, bits, delta, a, b, c,
                                      q, _ptr(x), _ptr(out))
        assert rc == 0
        return out

    def bin_in_freq(self, out: np.ndarray, n: int, bins: int, bits: int,
                    delta: float, a: int, b: int, c: int, q: int,
                    k0: np.ndarray, coef: np.ndarray, ftype: int = 1) -> np.ndarray:
        out = np.ascontiguousarray(out, np.complex128).copy()
        k0 = np.ascontiguousarray(k0, np.int32)
        coef = np.ascontiguousarray(coef, np.complex128)
        rc = self.lib.orc_bin_in_freq(ftype, n, bins, bits, delta, a, b, c, q,
                                      _ptr(k0), _ptr(coef), k0.size, _ptr(out))
        assert rc == 0
        return out

    def mat_pencil(self, u0: complex, u1: complex, u2: complex):
        u = np.array([u0, u1, u2], np.complex128)
        sig = np.zeros(2, np.float64)
        vote = self.lib.orc_mat_pencil(_ptr(u), _ptr(sig))
        return float(sig[0]), float(sig[1]), bool(vote)

    def iterate(self, x: np.ndarray, bins: int, window_delta: float = 1e-6,
                trials: int = 1, bin_threshold: float = 0.0,
                window_threshold: float = 0.0, sv_threshold: float = 0.0,
                mm: dict | None = None, btype: int = 4, ftype: int = 1,
                cap: int | None = None):
        x = np.ascontiguousarray(x, np.complex128)
        mm = dict(mm or {})
        cap = cap or (len(mm) + bins + 16)
        k = np.zeros(cap, np.int32)
        c = np.zeros(cap, np.complex128)
        for i, (kk, cc) in enumerate(mm.items()):
            k[i] = kk
            c[i] = cc
        size = np.array([len(mm)], np.int32)
        rc = self.lib.orc_iterate(x.size, _ptr(x), bins, window_delta, trials,
                                  bin_threshold, window_threshold, sv_threshold,
                                  btype, ftype, _ptr(k), _ptr(c), _ptr(size), cap)
        if rc < 0:
            raise RuntimeError("mode map capacity too small")
        m = int(size[0])
        return bool(rc), {int(k[i]): complex(c[i]) for i in range(m)}

    def demo1_run(self, x: np.ndarray, k: int, sigma: float, seed: int,
                  trials: int = 1, min_bins: int = 51, window_delta: float = 1e-5,
                  window_threshold: float = 0.1, max_stale_iter: int = 5,
                  cap: int | None = None):
        """Returns (modes dict, number of Iterate calls or -1 if unknown)."""
        x = np.ascontiguousarray(x, np.complex128)
        cap = cap or (4 * k + 4096)
        ok = np.zeros(cap, np.int32)
        oc = np.zeros(cap, np.complex128)
        iters = np.zeros(1, np.int32)
        m = self.lib.orc_demo1_run(x.size, _ptr(x), k, sigma, trials, min_bins,
                                   window_delta, window_threshold, max_stale_iter,
                                   seed, _ptr(ok), _ptr(oc), cap, _ptr(iters))
        if m < 0:
            raise RuntimeError("mode capacity too small")
        return {int(ok[i]): complex(oc[i]) for i in range(m)}, int(iters[0])

    # --- test data and analysis (src/gen.cc, src/demo1.cc) -----------------
    def generate_mode_map(self, n: int, k: int, seed: int):
        """GenerateModeMap after RandomSeed(seed): (positions sorted, coefs)."""
        self.seed(seed)
        ok = np.zeros(k, np.int32)
        oc = np.zeros(k, np.complex128)
        m = self.lib.orc_generate_mode_map(n, k, _ptr(ok), _ptr(oc))
        return ok[:m].copy(), oc[:m].copy()

    def demo_signal(self, n: int, k: int, sigma: float, seed: int, alt: bool = False):
        """RandomSeed(seed), then Demo1's signal construction (GenerateModeMap,
        GenerateXhat or GenerateXhatAlt, backward FFT): (x, positions sorted,
        coefficients). The RNG is left where the construction leaves it."""
        self.seed(seed)
        x = np.zeros(n, np.complex128)
        ok = np.zeros(k, np.int32)
        oc = np.zeros(k, np.complex128)
        m = self.lib.orc_demo_signal(n, k, sigma, 1 if alt else 0, _ptr(x), _ptr(ok),
                                     _ptr(oc))
        return x, ok[:m].copy(), oc[:m].copy()

    def post_analyze(self, xh: np.ndarray, true_k, found_k, found_c) -> dict:
        """Demo1::PostAnalyze on spectrum xh: hit/miss counts and errors."""
        xh = np.ascontiguousarray(xh, np.complex128)
        tk = np.ascontiguousarray(true_k, np.int32)
        fk = np.ascontiguousarray(found_k, np.int32)
        fc = np.ascontiguousarray(found_c, np.complex128)
        out = np.zeros(9, np.float64)
        self.lib.orc_post_analyze(xh.size, _ptr(xh), _ptr(tk), tk.size, _ptr(fk),
                                  _ptr(fc), fk.size, _ptr(out))
        names = ["hit", "hit_l1", "hit_l2", "miss", "miss_l1", "miss_l2", "l1",
                 "l2", "max_err"]
        d = dict(zip(names, out.tolist()))
        d["hit"] = int(d["hit"])
        d["miss"] = int(d["miss"])
        return d
