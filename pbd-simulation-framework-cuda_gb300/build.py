"""Build recipe for libpbd.so (the GB300 PBD step behind include/pbd.h).

nvcc compiles the CUDA translation units for sm_103a only and g++ the config reader; the
shared library links the CUDA runtime statically, so it depends on nothing but the driver.
Objects go to _build/ beside this file and the library to this folder (both git-ignored).
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OBJ = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libpbd.so")
INCLUDE = os.path.join(HERE, "..", "include")
NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

CU = ["pbd_sim.cu", "pbd_noalloc.cu"]
CPP = ["pbd_config.cpp"]


def _newer(out, deps):
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps)


def _deps():
    d = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    d.append(os.path.join(INCLUDE, "pbd.h"))
    d.append(os.path.abspath(__file__))
    return d


def build(force=False, verbose=False, extra_nvcc=()):
    os.makedirs(OBJ, exist_ok=True)
    deps = _deps()
    jobs = []
    objs = []
    for f in CU:
        o = os.path.join(OBJ, f + ".o")
        objs.append(o)
        if force or _newer(o, deps):
            # -prec-div/-prec-sqrt=false: the neighbour passes use the hardware approximations
            # (as the reference's FastMath build does); bit-exact steps use explicit _rn intrinsics
            cmd = [NVCC, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-prec-div=false", "-prec-sqrt=false",
                   "-Xcompiler", "-fPIC,-O2", "-I", INCLUDE,
                   *extra_nvcc, "-c", os.path.join(CSRC, f), "-o", o]
            jobs.append(cmd)
    for f in CPP:
        o = os.path.join(OBJ, f + ".o")
        objs.append(o)
        if force or _newer(o, deps):
            jobs.append(["g++", "-O2", "-std=c++17", "-fPIC", "-I", INCLUDE, "-c", os.path.join(CSRC, f), "-o", o])
    procs = []
    for cmd in jobs:
        if verbose:
            print(" ".join(cmd), flush=True)
        procs.append((cmd, subprocess.Popen(cmd)))
    for cmd, p in procs:
        if p.wait() != 0:
            raise RuntimeError("build failed: " + " ".join(cmd))
    if force or jobs or not os.path.exists(LIB):
        cmd = [NVCC, *ARCH, "-shared", "-o", LIB + ".tmp", *objs, "-cudart", "static"]
        if verbose:
            print(" ".join(cmd), flush=True)
        subprocess.check_call(cmd)
        os.replace(LIB + ".tmp", LIB)
    build_examples(force or bool(jobs))
    return LIB


EXAMPLES = os.path.join(HERE, "examples")


def build_examples(force=False):
    """The C++ host examples, linked against libpbd.so (found beside them through the rpath)."""
    for src in sorted(os.listdir(EXAMPLES)):
        if not src.endswith(".cpp"):
            continue
        exe = os.path.join(EXAMPLES, src[:-4])
        s = os.path.join(EXAMPLES, src)
        if force or _newer(exe, [s, LIB, os.path.join(INCLUDE, "pbd.h")]):
            # no FMA contraction: the host arithmetic (the spawn lattice) rounds as numpy does
            subprocess.check_call(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-I", INCLUDE, s, "-o", exe,
                                   "-L", HERE, "-lpbd", "-Wl,-rpath,$ORIGIN/.."])


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
