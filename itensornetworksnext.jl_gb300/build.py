"""Build recipe for libitn_gpu.so (sm_103a).

Each CUDA translation unit is compiled with nvcc in parallel, then linked into
``itensornetworksnext.jl_gb300/lib/libitn_gpu.so``.  No cmake, no torch: the library
depends only on the CUDA runtime (statically linked) so that any FFI (Julia ``ccall``,
Python ``ctypes``, C) can load it.

    python itensornetworksnext.jl_gb300/build.py [--force] [--jobs N]
"""
from __future__ import annotations

import argparse
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OBJ = os.path.join(HERE, "_build")
LIB_DIR = os.path.join(HERE, "lib")
LIB = os.path.join(LIB_DIR, "libitn_gpu.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-O2",
              "--expt-relaxed-constexpr", "-I", INCLUDE, "-I", CSRC]

SOURCES = ["itn_api.cu", "bp_generic.cu", "bp_tc.cu", "bp_z3.cu", "noalloc.cu", "contract.cu", "apply_gates.cu"]
HEADERS = ["itn_common.cuh", "itn_internal.h", "itn_tc.h", "tc_ptx.cuh", "itn_conv.cuh", "itn_contract.h", "itn_apply.h", "itn_z3.h"]


def nvcc() -> str:
    p = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(p):
        raise RuntimeError("nvcc not found")
    return p


def _newest_dep() -> float:
    files = [os.path.join(CSRC, f) for f in SOURCES + HEADERS]
    files += [os.path.join(INCLUDE, "itn_gpu.h"), os.path.abspath(__file__)]
    return max(os.path.getmtime(f) for f in files if os.path.exists(f))


def _compile(src: str, extra: list[str]) -> str:
    obj = os.path.join(OBJ, os.path.splitext(src)[0] + ".o")
    cmd = [nvcc(), *ARCH, *NVCC_FLAGS, *extra, "-c", os.path.join(CSRC, src), "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    return obj


def build(force: bool = False, jobs: int | None = None, verbose: bool = False,
          extra: list[str] | None = None) -> str:
    """Compile every CUDA source for sm_103a and link libitn_gpu.so; returns its path."""
    os.makedirs(OBJ, exist_ok=True)
    os.makedirs(LIB_DIR, exist_ok=True)
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= _newest_dep():
        return LIB
    extra = list(extra or [])
    jobs = jobs or min(len(SOURCES), os.cpu_count() or 1)
    with cf.ThreadPoolExecutor(max_workers=jobs) as ex:
        objs = list(ex.map(lambda s: _compile(s, extra), SOURCES))
    tmp = LIB + f".tmp{os.getpid()}"
    cmd = [nvcc(), *ARCH, "-shared", "-o", tmp, *objs]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    if verbose:
        print(f"built {LIB}")
    return LIB


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--force", action="store_true")
    ap.add_argument("--jobs", type=int, default=None)
    ap.add_argument("--ptxas-verbose", action="store_true")
    a = ap.parse_args()
    ex = ["-Xptxas", "-v"] if a.ptxas_verbose else []
    try:
        build(force=a.force or a.ptxas_verbose, jobs=a.jobs, verbose=True, extra=ex)
    except RuntimeError as e:
        print(e, file=sys.stderr)
        sys.exit(1)
