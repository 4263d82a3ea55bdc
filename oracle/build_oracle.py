"""Build the CPU oracle shared library (test infrastructure only).

The oracle is the checker for the CUDA path; it is compiled with
-ffp-contract=off so that float expressions are evaluated op by op on both
x86-64 and aarch64 (GCC contracts a*b+c into FMA by default on aarch64).
Output: oracle/_build/liboracle_fl.so
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "liboracle_fl.so")
SRCS = [os.path.join(HERE, "fl_oracle.c")]
DEPS = SRCS + [os.path.join(HERE, "fl_oracle_step.inc"), os.path.join(HERE, "fl_oracle.h"),
               os.path.join(HERE, "..", "include", "fluidgb.h")]


def build(force=False, verbose=False):
    os.makedirs(OUT_DIR, exist_ok=True)
    if not force and os.path.exists(LIB):
        t = os.path.getmtime(LIB)
        if all(os.path.getmtime(d) <= t for d in DEPS):
            return LIB
    cc = os.environ.get("CC", "gcc")
    cmd = [cc, "-std=c11", "-O2", "-fPIC", "-shared", "-ffp-contract=off", "-fno-fast-math",
           "-fopenmp", "-Wall", "-Wno-unused-function", "-o", LIB + ".tmp"] + SRCS + ["-lm"]
    if verbose:
        print(" ".join(cmd))
    subprocess.run(cmd, check=True)
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
