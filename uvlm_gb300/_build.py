"""Build the CUDA library (uvlm_gb300/libvfmm.so) with nvcc for sm_103a.

Translation units compile in parallel into uvlm_gb300/_build/ and link into
one shared library; a unit is recompiled when it or a header is newer than its
object.  Each unit's ptxas resource report (registers, spills, static shared
memory per kernel) is kept beside its object.  No CMake and no torch extension machinery: plain nvcc, so that the
library has a C ABI (include/vfmm.h) and no dependency on PyTorch.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import re
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libvfmm.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
              "-I" + os.path.join(ROOT, "include")]


def nvcc() -> str:
    exe = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(exe):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libvfmm.so")
    return exe


def _newest_header() -> float:
    hdrs = glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(ROOT, "include", "*.h"))
    return max((os.path.getmtime(h) for h in hdrs), default=0.0)


def ptxas_report(name: str) -> str:
    """Path of the ptxas resource report (registers, spills, static shared
    memory per kernel) that the build keeps beside csrc/<name>.cu's object."""
    return os.path.join(OUT_DIR, name + ".ptxas.txt")


def _compile(src: str, extra: list[str], verbose: bool) -> str:
    obj = os.path.join(OUT_DIR, os.path.basename(src).replace(".cu", ".o"))
    report = ptxas_report(os.path.basename(src)[:-3])
    if os.path.exists(obj) and os.path.exists(report) and \
            os.path.getmtime(obj) >= max(os.path.getmtime(src), _newest_header()):
        return obj
    cmd = [nvcc(), *ARCH, *NVCC_FLAGS, "-Xptxas", "-v", *extra, "-c", src, "-o", obj]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, stderr=subprocess.PIPE, text=True)
    with open(report, "w") as f:
        f.write(r.stderr)
    # the resource lines go to the report; anything else the compiler says is shown
    other = [ln for ln in r.stderr.splitlines() if not ln.startswith("ptxas info") and not re.match(r"^\s+\d+ bytes", ln)]
    if other:
        sys.stderr.write("\n".join(other) + "\n")
    if r.returncode != 0:
        raise subprocess.CalledProcessError(r.returncode, cmd)
    return obj


def build(verbose: bool = False, extra: list[str] | None = None, jobs: int | None = None) -> str:
    """Compile every csrc/*.cu for sm_103a and link libvfmm.so; returns its path."""
    os.makedirs(OUT_DIR, exist_ok=True)
    srcs = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    jobs = jobs or min(len(srcs), os.cpu_count() or 4)
    with cf.ThreadPoolExecutor(jobs) as ex:
        objs = list(ex.map(lambda s: _compile(s, extra or [], verbose), srcs))
    if not os.path.exists(LIB) or os.path.getmtime(LIB) < max(os.path.getmtime(o) for o in objs):
        cmd = [nvcc(), *ARCH, "-shared", "-o", LIB, *objs]
        if verbose:
            print(" ".join(cmd), flush=True)
        subprocess.run(cmd, check=True)
    return LIB


if __name__ == "__main__":
    print(build(verbose=True))
