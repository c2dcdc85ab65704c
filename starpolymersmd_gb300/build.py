"""Builds the in-tree CUDA library ``starpolymersmd_gb300/_lib/libsmpc.so``.

nvcc for sm_103a only (``-gencode arch=compute_103a,code=sm_103a``), one
translation unit per precision so the FP64 parity kernels can be compiled
with ``-fmad=false`` (no contraction, the reference's rounding order) while the
FP32 fast path keeps FMA. Host code is compiled with ``-ffp-contract=off`` so
the FP64 Lees-Edwards offset is advanced exactly like the reference's on every
host architecture. Translation units compile in parallel.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
LIBDIR = os.path.join(HERE, "_lib")
OBJDIR = os.path.join(HERE, "_build")
LIB = os.path.join(LIBDIR, "libsmpc.so")
ROOT = os.path.dirname(HERE)

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler",
          "-ffp-contract=off", "--expt-relaxed-constexpr", "-I", os.path.join(ROOT, "include")]
UNITS = {
    "kernels_fp64.cu": ["-fmad=false"],
    "kernels_fp32.cu": [],
    "scan.cu": [],
    "smpc_capi.cu": ["-fmad=false"],
}


def nvcc() -> str:
    path = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(path):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libsmpc")
    return path


def _sources_newer_than(target: str) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    deps.append(os.path.join(ROOT, "include", "smpc.h"))
    deps.append(__file__)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose: bool = False) -> str:
    """Compiles (if needed) and returns the path of libsmpc.so."""
    if not force and not _sources_newer_than(LIB):
        return LIB
    os.makedirs(OBJDIR, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    cc = nvcc()

    def compile_unit(name: str) -> str:
        obj = os.path.join(OBJDIR, name.replace(".cu", ".o"))
        cmd = [cc] + ARCH + COMMON + UNITS[name] + ["-c", os.path.join(CSRC, name), "-o", obj]
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"nvcc failed for {name}:\n{res.stdout}\n{res.stderr}")
        if verbose:
            sys.stderr.write(res.stderr)
        return obj

    with cf.ThreadPoolExecutor(max_workers=len(UNITS)) as ex:
        objs = list(ex.map(compile_unit, UNITS))
    tmp = LIB + ".tmp%d" % os.getpid()
    cmd = [cc] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"link failed:\n{res.stdout}\n{res.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
