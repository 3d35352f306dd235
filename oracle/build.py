"""Build recipe for the oracle (test infrastructure only).

Compiles ``swe_oracle.c`` (the step) and ``swe_oracle_adapt.c`` (one adaption
step and the integrated bathymetry) into ``oracle/_build/libswe_oracle.so`` with strict IEEE
flags: no FMA contraction, no fast-math, OpenMP for the timed CPU baseline.
The reference itself is Fortran and is not compiled here (no Fortran compiler).
"""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libswe_oracle.so")
SRCS = [os.path.join(HERE, "swe_oracle.c"), os.path.join(HERE, "swe_oracle_adapt.c")]

CFLAGS = ["-O2", "-fPIC", "-shared", "-std=c11", "-fno-fast-math", "-ffp-contract=off",
          "-fno-strict-aliasing", "-fopenmp", "-Wall", "-Wno-unused-function"]


def build(force: bool = False) -> str:
    os.makedirs(OUT_DIR, exist_ok=True)
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= max(os.path.getmtime(s) for s in SRCS):
        return LIB
    tmp = LIB + ".tmp%d" % os.getpid()
    subprocess.check_call(["gcc", *CFLAGS, *SRCS, "-o", tmp, "-lm"])
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True))
