"""Build recipe for oracle/_ref/libref_emu.so: the reference's own kernel on the CPU.

TEST INFRASTRUCTURE ONLY.  Compiles the reference's ``KernelDefinitions.h`` +
``Kernel.cl`` exactly where they lie in the reference checkout (the same
concatenation KernelInvoker.cpp:41-45 JIT-compiles), as plain C11 through
``ref_shim.h``, and links it with the fiber work-group emulator
``ref_emu.c``.  The reference's host ``Tools.cpp`` and ``Logger.cpp`` are
compiled too (against the OpenCL declarations in ``ref_cl/CL/cl.h``, whose
entry points are never called) so that ``ref_sort_glue.cpp`` can run the
reference's own ``preorder_by_x``.  Only output: ``oracle/_ref/libref_emu.so``
(git-ignored).

One mechanical edit is applied in the pipe to gcc (nothing is written to
disk): the two work-group-shared arrays declared in the kernel body
(Kernel.cl:656-657, ``__local int sh_hit_process[...]`` and
``__local int sensor_data[6]``) become ``static _Thread_local``, which is
work-group-shared under the emulator because all fibers of a work-group run
on one OS thread.  Everything else is the reference's code, unmodified.

Usage: ``python oracle/build_ref.py [--reference DIR]``; the reference
checkout is ``$CL_FORWARD_REFERENCE`` when set, else a checkout named
``reference`` beside this repository; where neither exists, nothing is built
and the tests that need the reference skip.
"""
from __future__ import annotations

import argparse
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_ref")
OUT_LIB = os.path.join(OUT_DIR, "libref_emu.so")

_EDITS = [
    ("__local int sh_hit_process [NUMTHREADS_X];",
     "static _Thread_local int sh_hit_process [NUMTHREADS_X];"),
    ("__local int sensor_data [6];", "static _Thread_local int sensor_data [6];"),
]

CFLAGS = ["-O2", "-std=gnu11", "-fPIC", "-ffp-contract=off", "-fno-strict-aliasing",
          "-w"]


def default_reference() -> str:
    env = os.environ.get("CL_FORWARD_REFERENCE")
    if env:
        return env
    return os.path.normpath(os.path.join(HERE, "..", "..", "reference"))


def available(reference: str | None = None) -> bool:
    ref = reference or default_reference()
    return all(os.path.isfile(os.path.join(ref, f)) for f in ("Kernel.cl", "KernelDefinitions.h"))


def kernel_source(reference: str) -> str:
    with open(os.path.join(reference, "KernelDefinitions.h")) as f:
        defs = f.read()
    with open(os.path.join(reference, "Kernel.cl")) as f:
        kern = f.read()
    for old, new in _EDITS:
        if kern.count(old) != 1:
            raise RuntimeError(f"expected exactly one occurrence of {old!r} in Kernel.cl")
        kern = kern.replace(old, new)
    return f'#include "ref_shim.h"\n#line 1 "KernelDefinitions.h"\n{defs}\n#line 1 "Kernel.cl"\n{kern}\n'


def build(reference: str | None = None, force: bool = False, quiet: bool = False) -> str | None:
    ref = reference or default_reference()
    if not available(ref):
        if not quiet:
            print(f"reference sources not found under {ref}; oracle/_ref not built", file=sys.stderr)
        return None
    srcs = [os.path.join(ref, f) for f in ("Kernel.cl", "KernelDefinitions.h", "Tools.cpp", "Logger.cpp")]
    srcs += [os.path.join(HERE, f) for f in ("ref_emu.c", "ref_shim.h", "ref_sort_glue.cpp",
                                               "ref_cl/CL/cl.h", "ref_cl/ref_cl_stubs.c")]
    srcs.append(__file__)
    if (not force and os.path.exists(OUT_LIB)
            and os.path.getmtime(OUT_LIB) >= max(os.path.getmtime(s) for s in srcs)):
        return OUT_LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    kobj = os.path.join(OUT_DIR, "ref_kernel.o")
    eobj = os.path.join(OUT_DIR, "ref_emu.o")
    subprocess.run(["gcc", *CFLAGS, "-I", HERE, "-x", "c", "-c", "-", "-o", kobj],
                   input=kernel_source(ref).encode(), check=True)
    subprocess.run(["gcc", *CFLAGS, "-c", os.path.join(HERE, "ref_emu.c"), "-o", eobj], check=True)
    objs = [kobj, eobj]
    cl_inc = ["-I", os.path.join(HERE, "ref_cl"), "-I", ref]
    for src, comp in ((os.path.join(ref, "Tools.cpp"), "g++"), (os.path.join(ref, "Logger.cpp"), "g++"),
                      (os.path.join(HERE, "ref_sort_glue.cpp"), "g++"),
                      (os.path.join(HERE, "ref_cl", "ref_cl_stubs.c"), "gcc")):
        obj = os.path.join(OUT_DIR, os.path.basename(src) + ".o")
        std = ["-std=gnu++14"] if comp == "g++" else ["-std=gnu11"]
        subprocess.run([comp, "-O2", "-fPIC", "-w", *std, *cl_inc, "-c", src, "-o", obj], check=True)
        objs.append(obj)
    subprocess.run(["g++", "-shared", "-o", OUT_LIB, *objs, "-lpthread", "-lm"], check=True)
    return OUT_LIB


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=None)
    ap.add_argument("--force", action="store_true")
    a = ap.parse_args()
    out = build(a.reference, a.force)
    print(out or "not built")
