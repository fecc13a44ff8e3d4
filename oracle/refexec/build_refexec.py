"""Build recipe of oracle/_ref/librefexec.so: the reference's own kernel code, run on the CPU.

TEST INFRASTRUCTURE ONLY.  Reads the reference's kernel headers where they lie
(<reference>/src/app/simulation/kernel, <reference> = $PBD_REFERENCE_ROOT or the
reference/PBD-Simulation-Framework-CUDA checkout beside this repository), rewrites in memory
the one construct a host compiler cannot parse -- the launch syntax `kernel<<<grid, block>>>(args);`
becomes `refx::launch(grid, block, [&]{ kernel(args); });` -- drops the includes of sibling
headers that are concatenated in order, and pipes the result, between refexec_shim.h and
refexec_harness.cpp, to g++ on standard input.  Nothing derived from the reference is written to
disk except the shared library in oracle/_ref/ (git-ignored).  Needs the reference sources, so it
runs only where they are mounted; the golden fixtures it produces are committed.
"""
import os
import re
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
# the reference checkout: PBD_REFERENCE_ROOT, else reference/PBD-Simulation-Framework-CUDA beside this repository
REF = os.environ.get("PBD_REFERENCE_ROOT") or os.path.join(os.path.dirname(ROOT), "reference", "PBD-Simulation-Framework-CUDA")
KDIR = os.path.join(REF, "src", "app", "simulation", "kernel")
OUT_DIR = os.path.join(ROOT, "oracle", "_ref")
OUT = os.path.join(OUT_DIR, "librefexec.so")
FILES = ["Kernels.h", "Globals.h", "Hash.h", "SortReorder.h", "Forces.h", "Collision.h", "Density.h", "Update.h"]
SIBLINGS = {"Kernels.h", "Globals.h", "Hash.h", "Communication.h", "SortReorder.h", "Forces.h",
            "Collision.h", "Density.h", "Update.h"}
LAUNCH = re.compile(r"(\w+)\s*<<<(.+?)>>>\s*\((.*)\)\s*;")
INCLUDE = re.compile(r'\s*#\s*include\s+"([^"]+)"')


def available():
    return all(os.path.exists(os.path.join(KDIR, f)) for f in FILES)


def translation_unit():
    parts = ['#include "refexec_shim.h"\n']
    for f in FILES:
        path = os.path.join(KDIR, f)
        parts.append(f'#line 1 "{path}"\n')
        for line in open(path, encoding="latin-1").read().splitlines():
            m = INCLUDE.match(line)
            if m and os.path.basename(m.group(1)) in SIBLINGS:
                parts.append("\n")
                continue
            parts.append(LAUNCH.sub(r"refx::launch(\2, [&] { \1(\3); });", line) + "\n")
    harness = os.path.join(HERE, "refexec_harness.cpp")
    parts.append(f'#line 1 "{harness}"\n')
    parts.append(open(harness).read())
    return "".join(parts)


def build(force=False, verbose=False):
    if not available():
        raise FileNotFoundError(f"reference kernel sources not found under {KDIR}")
    deps = [os.path.join(HERE, n) for n in ("refexec_shim.h", "refexec_harness.cpp", "build_refexec.py")]
    if not force and os.path.exists(OUT) and all(os.path.getmtime(OUT) >= os.path.getmtime(d) for d in deps):
        return OUT
    os.makedirs(OUT_DIR, exist_ok=True)
    cmd = ["g++", "-std=c++17", "-O2", "-fPIC", "-shared", "-w", "-mfma", "-ffp-contract=fast",
           "-I", os.path.join(HERE, "include"), "-I", HERE, "-I", "/usr/local/cuda/include",
           "-I", os.path.join(REF, "src"), "-I", os.path.join(ROOT, "include"),
           "-x", "c++", "-", "-o", OUT + ".tmp"]
    if verbose:
        print(" ".join(cmd))
    p = subprocess.run(cmd, input=translation_unit().encode("latin-1"), capture_output=True)
    if p.returncode != 0:
        raise RuntimeError("refexec build failed:\n" + p.stderr.decode(errors="replace")[-6000:])
    os.replace(OUT + ".tmp", OUT)
    return OUT


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
