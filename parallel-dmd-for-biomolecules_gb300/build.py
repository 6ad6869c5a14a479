"""Builds the GB300 engine library in-tree: _build/libdmd_gb300.so.

nvcc compiles every CUDA translation unit for sm_103a only, with
--fmad=false so that the device arithmetic keeps the reference's separate
multiply and add (bit-identical to the host restatement), and the host
C++ of the library with -ffp-contract=off for the same reason.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
# DMD_CHECKED=1: the checked build (-DDMD_BOUNDS: device index checks that
# record the first out-of-range index instead of faulting), kept apart
CHECKED = os.environ.get("DMD_CHECKED", "") == "1"
OUT = os.path.join(PKG, "_build_checked" if CHECKED else "_build")
LIB = os.path.join(OUT, "libdmd_gb300.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "--fmad=false", "-lineinfo", "-Xcompiler", "-fPIC,-ffp-contract=off",
              "-I" + os.path.join(REPO, "include"), "-I" + CSRC]
CU_SOURCES = ["engine.cu", "capi.cu", "sidechain.cu"]
CPP_SOURCES = ["generate.cpp"]


def nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _run(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed:\n" + " ".join(cmd) + "\n" + r.stdout)
    return r.stdout


def build(verbose: bool = False, extra: list | None = None) -> str:
    os.makedirs(OUT, exist_ok=True)
    if CHECKED:
        extra = list(extra or []) + ["-DDMD_BOUNDS"]
        stamp = os.path.join(OUT, "checked.stamp")
        newest_src = max(os.path.getmtime(os.path.join(CSRC, f)) for f in os.listdir(CSRC))
        if os.path.exists(LIB) and os.path.exists(stamp) and os.path.getmtime(stamp) >= newest_src:
            return LIB
    nv = nvcc()
    srcs = CU_SOURCES + CPP_SOURCES
    newest = max(os.path.getmtime(os.path.join(CSRC, f)) for f in os.listdir(CSRC))
    newest = max(newest, os.path.getmtime(os.path.join(REPO, "include", "dmd.h")), os.path.getmtime(__file__))
    # the extra flags the library was built with: a library built with
    # other flags (a debug build with timers, say) is rebuilt, not reused
    flags_file = os.path.join(OUT, "build.flags")
    want_flags = " ".join(extra or [])
    try:
        with open(flags_file) as fh:
            have_flags = fh.read()
    except OSError:
        have_flags = None
    if os.path.exists(LIB) and os.path.getmtime(LIB) >= newest and not extra and have_flags == want_flags:
        return LIB
    objs, cmds = [], []
    for s in srcs:
        obj = os.path.join(OUT, s + ".o")
        objs.append(obj)
        if s.endswith(".cu"):
            cmds.append([nv] + ARCH + NVCC_FLAGS + (extra or []) + ["-c", os.path.join(CSRC, s), "-o", obj])
        else:
            cmds.append([nv] + ["-O3", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off",
                                "-I" + os.path.join(REPO, "include"), "-I" + CSRC, "-c", os.path.join(CSRC, s), "-o", obj])
    with cf.ThreadPoolExecutor(max_workers=len(cmds)) as ex:
        outs = list(ex.map(_run, cmds))
    if verbose:
        for o in outs:
            sys.stdout.write(o)
    tmp = LIB + ".tmp"
    _run([nv] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart"])
    os.replace(tmp, LIB)
    with open(flags_file, "w") as fh:
        fh.write(want_flags)
    if CHECKED:
        open(os.path.join(OUT, "checked.stamp"), "w").close()
    return LIB


if __name__ == "__main__":
    print(build(verbose=True, extra=sys.argv[1:] or None))
