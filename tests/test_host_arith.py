"""Host-side integer helpers of the kernels, compiled for the host with
nvcc and run without a GPU (tests/host/arith_check.cu): the division-free
k1 rounding of the decide kernels equals the rounding by a 64-bit division
(src/iterate.cc:133-134 evaluates it in FP64; the exact integer form and
its FP64 tie-break are the library's), and the rows the FP32 fold stashes
stay within the stash's capacity."""
from __future__ import annotations

import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def test_integer_helpers(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not available")
    exe = str(tmp_path / "arith_check")
    subprocess.run([nvcc, "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"),
                    os.path.join(HERE, "host", "arith_check.cu"), "-o", exe],
                   check=True, capture_output=True, text=True)
    out = subprocess.run([exe], capture_output=True, text=True)
    assert out.returncode == 0, out.stdout + out.stderr
    lines = out.stdout.split("\n")
    assert any(ln.startswith("round_k1 checked") and ln.endswith("mismatches 0") for ln in lines)
    assert any(ln.startswith("stash_rows checked") and ln.endswith("mismatches 0") for ln in lines)
