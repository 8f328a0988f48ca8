"""Build recipe for the CPU oracle (test infrastructure only).

Compiles oracle/srpic_oracle.c, grpic_oracle.c, inject_oracle.c and
output_oracle.c with gcc into oracle/_build/:
  liboracle_f32.so      (real = float, the reference's SINGLE_PRECISION build)
  liboracle_f64.so      (real = double)
all with -ffp-contract=off so every operation is rounded as written, and
OpenMP so the CPU-baseline leg can use every host core.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_build")

SOURCES = ["srpic_oracle.c", "grpic_oracle.c", "inject_oracle.c", "output_oracle.c"]
FLAGS = ["-O2", "-std=c11", "-fPIC", "-shared", "-ffp-contract=off", "-fno-fast-math",
         "-fopenmp", "-Wall", "-Wno-unused-function"]


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose=False):
    os.makedirs(OUT, exist_ok=True)
    deps = [os.path.join(HERE, s) for s in SOURCES] + [
        os.path.join(HERE, h) for h in ("srpic_oracle.h", "grpic_oracle.h", "grpic_metric.inc",
                                        "inject_oracle.h", "output_oracle.h")]
    libs = {}
    for tag, defs in (("f32", ["-DORC_SINGLE"]), ("f64", [])):
        target = os.path.join(OUT, f"liboracle_{tag}.so")
        if _stale(target, deps):
            cmd = ["gcc", *FLAGS, *defs, "-o", target, *deps[:len(SOURCES)], "-lm"]
            if verbose:
                print(" ".join(cmd))
            subprocess.check_call(cmd)
        libs[tag] = target
    return libs


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
