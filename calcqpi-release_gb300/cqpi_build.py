"""Build libcqpi.so (CUDA, sm_103a) and the host tools (calcqpi, mkwavefunctions) in-tree,
under _build/.

Every translation unit is compiled in parallel with
``nvcc -gencode arch=compute_103a,code=sm_103a -O3 -lineinfo``; objects are reused
when they are newer than their sources and headers.  The C++ host CLI links the
shared library with an $ORIGIN rpath.  No cmake, no torch extension machinery.
"""
from __future__ import annotations

import glob
import os
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
HOST = os.path.join(PKG, "host")
BUILD = os.path.join(PKG, "_build")
OBJ = os.path.join(BUILD, "obj")
LIB = os.path.join(BUILD, "libcqpi.so")
CLI = os.path.join(BUILD, "calcqpi")
MKWF = os.path.join(BUILD, "mkwavefunctions")
INCLUDE = os.path.join(ROOT, "include")

NVCC = os.environ.get("NVCC", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVFLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-O2", "-I" + INCLUDE, "-I" + CSRC]
CXX = os.environ.get("CXX", "g++")
CXXFLAGS = ["-O2", "-std=c++17", "-fopenmp", "-I" + INCLUDE, "-I" + HOST]


def _newer(target: str, deps) -> bool:
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(d) <= t for d in deps)


def _run_parallel(cmds, verbose=False):
    procs = []
    for c in cmds:
        if verbose:
            print(" ".join(c), flush=True)
        procs.append((c, subprocess.Popen(c, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)))
    errors = []
    for c, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            errors.append((c, out.decode(errors="replace")))
        elif verbose and out:
            sys.stdout.write(out.decode(errors="replace"))
    if errors:
        msg = "\n".join(" ".join(c) + "\n" + o for c, o in errors)
        raise RuntimeError("build failed:\n" + msg)


def build_lib(verbose=False, extra_flags=()) -> str:
    os.makedirs(OBJ, exist_ok=True)
    headers = (glob.glob(os.path.join(CSRC, "*.h")) + glob.glob(os.path.join(CSRC, "*.cuh")) +
               glob.glob(os.path.join(INCLUDE, "*.h")))
    srcs = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    objs, cmds = [], []
    for s in srcs:
        o = os.path.join(OBJ, os.path.basename(s)[:-3] + ".o")
        objs.append(o)
        if not _newer(o, [s] + headers):
            cmds.append([NVCC] + NVFLAGS + list(extra_flags) + ["-c", s, "-o", o])
    for s in sorted(glob.glob(os.path.join(CSRC, "*.cc"))):
        o = os.path.join(OBJ, os.path.basename(s)[:-3] + ".host.o")
        objs.append(o)
        if not _newer(o, [s] + headers):
            cmds.append([CXX, "-O2", "-std=c++17", "-fPIC", "-I" + INCLUDE, "-I" + CSRC, "-c", s, "-o", o])
    _run_parallel(cmds, verbose)
    if cmds or not _newer(LIB, objs):
        tmp = LIB + ".tmp%d" % os.getpid()
        _run_parallel([[NVCC] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart", "-lpthread"]], verbose)
        os.replace(tmp, LIB)
    return LIB


def build_cli(verbose=False) -> str:
    """One executable per host/<tool>_main.cc (calcqpi, mkwavefunctions), linked against
    libcqpi.so; the other host/*.cc files are shared by all tools."""
    srcs = sorted(glob.glob(os.path.join(HOST, "*.cc")))
    mains = [s for s in srcs if s.endswith("_main.cc")]
    if not mains:
        return ""
    shared = [s for s in srcs if s not in mains]
    headers = glob.glob(os.path.join(HOST, "*.h")) + glob.glob(os.path.join(INCLUDE, "*.h"))
    cmds, moves = [], []
    for m in mains:
        exe = os.path.join(BUILD, os.path.basename(m)[: -len("_main.cc")])
        if _newer(exe, [m] + shared + headers + [LIB]):
            continue
        tmp = exe + ".tmp%d" % os.getpid()
        cmds.append([CXX] + CXXFLAGS + [m] + shared + ["-o", tmp, "-L" + BUILD, "-lcqpi", "-Wl,-rpath,$ORIGIN"])
        moves.append((tmp, exe))
    _run_parallel(cmds, verbose)
    for tmp, exe in moves:
        os.replace(tmp, exe)
    return CLI


def build(verbose=False) -> dict:
    lib = build_lib(verbose)
    cli = build_cli(verbose)
    return {"lib": lib, "cli": cli, "mkwavefunctions": MKWF if cli else ""}


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
