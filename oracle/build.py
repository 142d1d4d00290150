"""Build recipe for the CPU oracle (test infrastructure only).

Compiles oracle/ati_oracle.c into oracle/_build/libati_oracle.so with gcc
-O3 and OpenMP.  -ffp-contract=off keeps x86 and Arm results identical (gcc
contracts to FMA by default on aarch64); without -ffast-math the vectoriser
leaves every floating-point result as written, so -O3 changes speed only.
There is no -march: the same flags build on the x86 container and the Arm
GPU host (CFLAGS is the flag list the timed CPU baseline reports).
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libati_oracle.so")
SRC = [os.path.join(HERE, "ati_oracle.c")]
DEPS = SRC + [os.path.join(HERE, "ati_oracle.h"), os.path.join(HERE, "..", "include", "ati.h")]
CFLAGS = ["-O3", "-std=gnu99", "-fPIC", "-fopenmp", "-ffp-contract=off", "-fno-fast-math", "-Wall",
          "-Wno-unused-function"]


def build(force=False, verbose=False):
    os.makedirs(OUT_DIR, exist_ok=True)
    if not force and os.path.exists(LIB):
        t = os.path.getmtime(LIB)
        if all(os.path.getmtime(d) <= t for d in DEPS):
            return LIB
    cmd = ["gcc", *CFLAGS, "-shared", "-o", LIB + ".tmp", *SRC, "-lm"]
    if verbose:
        print(" ".join(cmd), file=sys.stderr)
    subprocess.run(cmd, check=True)
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
