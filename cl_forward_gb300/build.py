"""Build recipe of the native library and the standalone driver.

Outputs (in-tree, git-ignored), under ``cl_forward_gb300/_build/``:

* ``libclforward_gb300.so`` -- the sm_103a kernels, the C ABI of
  ``include/velo_search.h`` and the reference-signature C++ entry points of
  ``include/GpuPixelSearchByTriplet.h`` (CUDA runtime linked statically);
* ``clpixel`` -- the standalone driver (IndependentEntrypoint counterpart);
* ``libvelo_api_bench.so`` -- the timing harness of the reference-signature
  entry points (bench.py's end-to-end leg through them).

The kernels are compiled for ``sm_103a`` only, with ``--fmad=false`` so that no
multiply-add contraction can change an FP32 cut (the kernel also spells every
operation with round-to-nearest intrinsics).  Translation units compile in
parallel; a unit is rebuilt only when a source or header it depends on is
newer than its object.
"""
from __future__ import annotations

import argparse
import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(ROOT, "include")
BUILD = os.path.join(PKG, "_build")
OBJ = os.path.join(BUILD, "obj")
LIB = os.path.join(BUILD, "libclforward_gb300.so")
DRIVER = os.path.join(BUILD, "clpixel")
API_BENCH = os.path.join(BUILD, "libvelo_api_bench.so")
# sources outside the library: the driver and the timing harness
NOT_IN_LIB = ("clpixel_main.cpp", "velo_api_bench.cpp")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "--fmad=false", "-Xcompiler", "-fPIC",
              "-Xcompiler", "-ffp-contract=off"]
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-Wall", "-Wextra",
             "-Wno-unused-parameter"]


def cuda_home() -> str:
    for c in (os.environ.get("CUDA_HOME"), os.environ.get("CUDA_PATH"), "/usr/local/cuda"):
        if c and os.path.isdir(c):
            return c
    nvcc = shutil.which("nvcc")
    if nvcc:
        return os.path.dirname(os.path.dirname(os.path.realpath(nvcc)))
    raise RuntimeError("CUDA toolkit not found (nvcc)")


def _headers():
    return glob.glob(os.path.join(CSRC, "*.h")) + glob.glob(os.path.join(CSRC, "*.cuh")) + \
        glob.glob(os.path.join(INCLUDE, "*.h"))


def _stale(target: str, deps) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _run(cmd, verbose):
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"build step failed ({r.returncode}): {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return r.stdout + r.stderr


def build(force: bool = False, verbose: bool = False, ptxas_info: bool = False) -> str:
    os.makedirs(OBJ, exist_ok=True)
    cuda = cuda_home()
    nvcc = os.path.join(cuda, "bin", "nvcc")
    inc = ["-I", os.path.join(cuda, "include"), "-I", INCLUDE, "-I", CSRC]
    hdrs = _headers()
    jobs = []
    objs = []
    for src in sorted(glob.glob(os.path.join(CSRC, "*.cu"))):
        obj = os.path.join(OBJ, os.path.basename(src) + ".o")
        objs.append(obj)
        if force or _stale(obj, [src, *hdrs, __file__]):
            extra = ["-Xptxas", "-v"] if ptxas_info else []
            jobs.append([nvcc, *ARCH, *NVCC_FLAGS, *extra, *inc, "-c", src, "-o", obj])
    for src in sorted(glob.glob(os.path.join(CSRC, "*.cpp"))):
        obj = os.path.join(OBJ, os.path.basename(src) + ".o")
        if os.path.basename(src) not in NOT_IN_LIB:
            objs.append(obj)
        if force or _stale(obj, [src, *hdrs, __file__]):
            jobs.append(["g++", *CXX_FLAGS, *inc, "-c", src, "-o", obj])
    logs = []
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(8, len(jobs))) as ex:
            for out in ex.map(lambda c: _run(c, verbose), jobs):
                logs.append(out)
    if ptxas_info:
        for l in logs:
            if l.strip():
                print(l)
    if force or jobs or not os.path.exists(LIB):
        tmp = LIB + f".tmp{os.getpid()}"
        _run([nvcc, *ARCH, "-shared", "-cudart", "static", "-o", tmp, *objs,
              "-Xlinker", "-z,defs", "-lpthread", "-ldl", "-lrt"], verbose)
        os.replace(tmp, LIB)
    drv_obj = os.path.join(OBJ, "clpixel_main.cpp.o")
    if force or _stale(DRIVER, [LIB, drv_obj]):
        _run(["g++", "-o", DRIVER, drv_obj, "-L", BUILD, "-lclforward_gb300",
              "-Wl,-rpath,$ORIGIN"], verbose)
    bench_obj = os.path.join(OBJ, "velo_api_bench.cpp.o")
    if force or _stale(API_BENCH, [LIB, bench_obj]):
        _run(["g++", "-shared", "-o", API_BENCH, bench_obj, "-L", BUILD, "-lclforward_gb300",
              "-Wl,-rpath,$ORIGIN"], verbose)
    return LIB


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--force", action="store_true")
    ap.add_argument("-v", "--verbose", action="store_true")
    ap.add_argument("--ptxas-info", action="store_true", help="print -Xptxas -v register/smem usage")
    a = ap.parse_args()
    print(build(a.force, a.verbose, a.ptxas_info))
    sys.exit(0)
