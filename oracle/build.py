"""Build recipe for the CPU oracle (test infrastructure only).

Compiles oracle/cliffs_oracle.c into oracle/_lib/libcliffs_oracle.so with
OpenMP.  -ffp-contract=off keeps the FP64 rounding identical on x86 and Arm.
No -march=native: the same flags must work on both hosts.
"""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
LIBDIR = os.path.join(HERE, "_lib")
LIB = os.path.join(LIBDIR, "libcliffs_oracle.so")
SRC = os.path.join(HERE, "cliffs_oracle.c")
HDR = os.path.join(HERE, "cliffs_oracle.h")


def build(force: bool = False) -> str:
    os.makedirs(LIBDIR, exist_ok=True)
    if (not force and os.path.exists(LIB)
            and os.path.getmtime(LIB) >= max(os.path.getmtime(SRC), os.path.getmtime(HDR))):
        return LIB
    tmp = LIB + ".tmp"
    cmd = ["gcc", "-O2", "-std=c11", "-fopenmp", "-fPIC", "-shared",
           "-ffp-contract=off", "-Wall", "-Wno-unknown-pragmas",
           SRC, "-o", tmp, "-lm"]
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True))
