"""Build recipe for the CPU oracle (test infrastructure only).

Compiles oracle/cliffs_oracle.c into oracle/_lib/libcliffs_oracle.so with
OpenMP.  -ffp-contract=off keeps the FP64 rounding identical on x86 and Arm.
No -march=native: the same flags must work on both hosts.  The same source
with -DORC_REAL=float -fsingle-precision-constant becomes
oracle/_lib/libcliffs_oracle_f32.so, the FP32 variant of the CPU time loop
(a timed baseline only).
"""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
LIBDIR = os.path.join(HERE, "_lib")
LIB = os.path.join(LIBDIR, "libcliffs_oracle.so")
LIB32 = os.path.join(LIBDIR, "libcliffs_oracle_f32.so")
SRC = os.path.join(HERE, "cliffs_oracle.c")
HDR = os.path.join(HERE, "cliffs_oracle.h")


def _build_one(lib, extra, force):
    if (not force and os.path.exists(lib)
            and os.path.getmtime(lib) >= max(os.path.getmtime(SRC), os.path.getmtime(HDR))):
        return lib
    tmp = lib + ".tmp"
    cmd = ["gcc", "-O2", "-std=c11", "-fopenmp", "-fPIC", "-shared",
           "-ffp-contract=off", "-Wall", "-Wno-unknown-pragmas", *extra,
           SRC, "-o", tmp, "-lm"]
    subprocess.run(cmd, check=True)
    os.replace(tmp, lib)
    return lib


def build(force: bool = False) -> str:
    os.makedirs(LIBDIR, exist_ok=True)
    _build_one(LIB32, ["-DORC_REAL=float", "-fsingle-precision-constant"], force)
    return _build_one(LIB, [], force)


if __name__ == "__main__":
    print(build(force=True))
