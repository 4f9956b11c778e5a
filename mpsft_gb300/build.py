"""Builds the in-tree shared library mpsft_gb300/_lib/libmpsft_gb300.so.

Every CUDA source in mpsft_gb300/csrc is compiled for sm_103a only
(``-gencode arch=compute_103a,code=sm_103a``), in parallel, and linked with
``nvcc -shared``. No cmake, no torch extension machinery: the product is a
plain C-ABI library that any FFI (ctypes, cgo, JNI) can load. The C++ adapter
that plugs the library into the reference's own binner factory
(mpsft_gb300/adapter) is compiled against the reference's headers by its user,
not here.
"""
from __future__ import annotations

import glob
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_lib")
LIB = os.path.join(OUT_DIR, "libmpsft_gb300.so")
OBJ_DIR = os.path.join(HERE, "_build")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + [
    "-O3", "-lineinfo", "-std=c++17",
    # host code: IEEE arithmetic without FMA contraction so that host-side
    # scalars (window widths, thresholds) match the reference on x86 and Arm
    "-Xcompiler", "-fPIC,-ffp-contract=off",
    "-I" + os.path.join(ROOT, "include"),
]


def _nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found; the CUDA toolkit is required")
    return cand


def _sources() -> list[str]:
    srcs = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    return srcs


def _stale(obj: str, deps: list[str]) -> bool:
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose: bool = False, jobs: int | None = None) -> str:
    nvcc = _nvcc()
    os.makedirs(OUT_DIR, exist_ok=True)
    os.makedirs(OBJ_DIR, exist_ok=True)
    headers = glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(
        os.path.join(CSRC, "*.h")) + [
        os.path.join(ROOT, "include", "mpsft.h")]
    srcs = _sources()
    objs = []
    cmds = []
    for src in srcs:
        obj = os.path.join(OBJ_DIR, os.path.basename(src) + ".o")
        objs.append(obj)
        if _stale(obj, [src] + headers):
            cmds.append([nvcc] + NVCC_FLAGS + ["-c", src, "-o", obj])

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if verbose or r.returncode != 0:
            sys.stderr.write(" ".join(cmd) + "\n" + r.stdout + r.stderr)
        if r.returncode != 0:
            raise RuntimeError(f"compile failed: {cmd[-3]}")

    with ThreadPoolExecutor(max_workers=jobs or min(8, os.cpu_count() or 4)) as ex:
        list(ex.map(run, cmds))
    if cmds or not os.path.exists(LIB):
        tmp = LIB + ".tmp"
        link = [nvcc] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart", "-lpthread"]
        r = subprocess.run(link, capture_output=True, text=True)
        if r.returncode != 0:
            sys.stderr.write(" ".join(link) + "\n" + r.stdout + r.stderr)
            raise RuntimeError("link failed")
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
