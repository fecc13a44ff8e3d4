"""Build recipe for the CPU oracle (test infrastructure only).

Compiles oracle/pbd_oracle.c twice with gcc into oracle/_build/:
  liboracle_f32.so  -- FP32 transliteration of the reference step (also the timed CPU baseline)
  liboracle_f64.so  -- FP64 oracle with the same semantics
Both are built with -ffp-contract=off (the only fused multiply-adds are the explicit ones in
the source) and OpenMP over particles.  No -march flags: the same source gives the same
results on x86_64 and aarch64.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_build")
SRC = os.path.join(HERE, "pbd_oracle.c")


def targets():
    return {"f32": os.path.join(OUT, "liboracle_f32.so"), "f64": os.path.join(OUT, "liboracle_f64.so")}


def build(force=False, verbose=False):
    os.makedirs(OUT, exist_ok=True)
    procs = []
    for tag, real in (("f32", "float"), ("f64", "double")):
        out = targets()[tag]
        if not force and os.path.exists(out) and os.path.getmtime(out) >= max(
            os.path.getmtime(SRC), os.path.getmtime(os.path.join(HERE, "..", "include", "pbd.h"))
        ):
            continue
        cmd = ["gcc", "-O2", "-std=c11", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
               "-fno-fast-math", f"-DORC_REAL={real}", SRC, "-o", out + ".tmp", "-lm"]
        if verbose:
            print(" ".join(cmd))
        procs.append((subprocess.Popen(cmd), out))
    for p, out in procs:
        if p.wait() != 0:
            raise RuntimeError(f"oracle build failed for {out}")
        os.replace(out + ".tmp", out)
    return targets()


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
