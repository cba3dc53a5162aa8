"""Build recipe of the CUDA library behind include/cliffs_gpu.h.

nvcc compiles csrc/cliffs_gpu.cu for sm_103a only (GB300) into
_lib/libcliffs_gpu.so, in the source tree.  No torch, no cmake.
"""
import glob
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
LIBDIR = os.path.join(HERE, "_lib")
LIB = os.path.join(LIBDIR, "libcliffs_gpu.so")
SRC = os.path.join(HERE, "csrc", "cliffs_gpu.cu")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _deps():
    return glob.glob(os.path.join(HERE, "csrc", "*")) + [os.path.join(ROOT, "include", "cliffs_gpu.h")]


def nvcc():
    cand = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")
    return cand if os.path.exists(cand) else "nvcc"


def build(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(LIBDIR, exist_ok=True)
    if not force and os.path.exists(LIB):
        if os.path.getmtime(LIB) >= max(os.path.getmtime(p) for p in _deps()):
            return LIB
    tmp = LIB + ".tmp"
    cmd = [nvcc(), "-O3", "-std=c++17", *ARCH, "-lineinfo", "-Xcompiler", "-fPIC",
           "-shared", SRC, "-o", tmp]
    if verbose:
        cmd.insert(1, "-Xptxas=-v")
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True, verbose=True))
