"""The drop-in adapter (mpsft_gb300/adapter) builds against the reference's
own headers and sources: the factory patch applies to the reference's
src/binner.cc, the patched factory and the GPU binners compile, and an example
caller links them with the reference's other objects and libmpsft_gb300.so.

The reference's third-party headers are the oracle's stand-ins (oracle/shim).
Runs where the reference tree is (it is not on GPU hosts). Without a GPU the
example caller's GPU work stops with the adapter's error, as the reference's
own checks abort; where a GPU is present it gives the known-answer bin of
src/binner_test.cc:74-75 and BinInFreq's exact negative.
"""
from __future__ import annotations

import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF_SRC = os.environ.get("MPSFT_REFERENCE_SRC", "/root/reference/src")
ADAPTER = os.path.join(ROOT, "mpsft_gb300", "adapter")
REF_OBJ = os.path.join(ROOT, "oracle", "_ref", "obj")
REF_OBJS = ["base", "window", "sincos", "magic", "freqid", "iterate", "gen",
            "demo1", "integer"]

pytestmark = pytest.mark.skipif(not os.path.isdir(REF_SRC),
                                reason="the reference tree is not on this host")


def _gpu_present() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except ImportError:
        return False


@pytest.fixture(scope="module")
def driver(lib, tmp_path_factory):
    subprocess.run(["make", "-s", "-j8", "-C", os.path.join(ROOT, "oracle"), "ref",
                    f"REF={REF_SRC}"], check=True, capture_output=True)
    out = tmp_path_factory.mktemp("adapter")
    objs = " ".join(os.path.join(REF_OBJ, o + ".o") for o in REF_OBJS)
    r = subprocess.run(
        ["make", "-s", "-C", ADAPTER, "driver", f"REF={REF_SRC}", f"OUT={out}",
         f"DEPS=-I{os.path.join(ROOT, 'oracle', 'shim')}",
         f"REFOBJS={objs}",
         f"DRIVER={os.path.join(ROOT, 'tests', 'adapter', 'adapter_driver.cc')}"],
        capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    return os.path.join(out, "adapter_driver"), out


def test_patch_adds_the_gpu_factory_types(driver):
    _, out = driver
    src = open(os.path.join(out, "src", "binner.cc")).read()
    assert '#include "binner_gpu.h"' in src
    assert "new BinInTimeGPU(win, bits)" in src
    assert "new BinInFreqGPU(win, bits)" in src


def test_factory_returns_the_gpu_binners(driver):
    exe, _ = driver
    r = subprocess.run([exe], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "factory: BinInTimeGPU, BinInFreqGPU" in r.stdout


def test_gpu_binning_through_the_factory(driver):
    exe, _ = driver
    r = subprocess.run([exe, "bin"], capture_output=True, text=True, timeout=120)
    if not _gpu_present():
        # the reference aborts on a failed check; so does the adapter
        assert r.returncode != 0
        assert "mpsft-gb300 context" in r.stderr
        return
    assert r.returncode == 0, r.stdout + r.stderr
    m = re.search(r"bin 0,1: (\S+) (\S+)", r.stdout)
    assert abs(float(m.group(1)) - 1.12652) < 2e-5
    assert abs(float(m.group(2)) + 0.108838) < 2e-5
    m = re.search(r"time \+ freq max: (\S+)", r.stdout)
    assert float(m.group(1)) < 1e-5
