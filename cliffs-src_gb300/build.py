"""Build recipe of the CUDA library behind include/cliffs_gpu.h and of the
driver executable above it.

nvcc compiles csrc/cliffs_gpu.cu for sm_103a only (GB300) into
_lib/libcliffs_gpu.so; g++ compiles host/*.cpp (the Cliffs driver with its
NetCDF classic I/O) into _lib/cliffs_gb300, and the offline tools depth_ssl
and ComputeBoundaryInput into _lib/depth_ssl_gb300 and _lib/cmpboundary_gb300,
all linked against that library.
Both stay in the source tree.  No torch, no cmake.
"""
import glob
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
LIBDIR = os.path.join(HERE, "_lib")
LIB = os.path.join(LIBDIR, "libcliffs_gpu.so")
SRC = [os.path.join(HERE, "csrc", "cliffs_gpu.cu"), os.path.join(HERE, "csrc", "mlp.cu")]
DRIVER = os.path.join(LIBDIR, "cliffs_gb300")
# the offline tools: executable -> its main source (each linked with nc3.cpp)
TOOLS = {os.path.join(LIBDIR, "depth_ssl_gb300"): os.path.join(HERE, "host", "depth_ssl_main.cpp"),
         os.path.join(LIBDIR, "cmpboundary_gb300"): os.path.join(HERE, "host", "cmpboundary_main.cpp")}
HOST_SRC = sorted(p for p in glob.glob(os.path.join(HERE, "host", "*.cpp")) if p not in TOOLS.values())
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _deps():
    return glob.glob(os.path.join(HERE, "csrc", "*")) + glob.glob(os.path.join(ROOT, "include", "*.h"))


def nvcc():
    cand = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")
    return cand if os.path.exists(cand) else "nvcc"


def build(force: bool = False, verbose: bool = False) -> str:
    """Build the library, then the driver; returns the library's path."""
    lib = build_lib(force, verbose)
    build_driver(force)
    for exe, main in TOOLS.items():
        build_tool(exe, main, force)
    return lib


def build_tool(exe: str, main: str, force: bool = False) -> str:
    src = [main, os.path.join(HERE, "host", "nc3.cpp")]
    deps = src + glob.glob(os.path.join(HERE, "host", "*.hpp")) + [LIB, os.path.join(ROOT, "include", "cliffs_gpu.h")]
    if not force and os.path.exists(exe):
        if os.path.getmtime(exe) >= max(os.path.getmtime(p) for p in deps):
            return exe
    tmp = exe + ".tmp"
    cmd = ["g++", "-O2", "-std=c++17", "-Wall", "-Wextra", *src, "-L" + LIBDIR, "-lcliffs_gpu",
           "-Wl,-rpath,$ORIGIN", "-o", tmp]
    subprocess.run(cmd, check=True)
    os.replace(tmp, exe)
    return exe


def build_driver(force: bool = False) -> str:
    deps = HOST_SRC + glob.glob(os.path.join(HERE, "host", "*.hpp")) + [LIB, os.path.join(ROOT, "include", "cliffs_gpu.h")]
    if not force and os.path.exists(DRIVER):
        if os.path.getmtime(DRIVER) >= max(os.path.getmtime(p) for p in deps):
            return DRIVER
    tmp = DRIVER + ".tmp"
    cmd = ["g++", "-O2", "-std=c++17", "-Wall", "-Wextra", *HOST_SRC, "-L" + LIBDIR, "-lcliffs_gpu",
           "-Wl,-rpath,$ORIGIN", "-o", tmp]
    subprocess.run(cmd, check=True)
    os.replace(tmp, DRIVER)
    return DRIVER


def build_lib(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(LIBDIR, exist_ok=True)
    if not force and os.path.exists(LIB):
        if os.path.getmtime(LIB) >= max(os.path.getmtime(p) for p in _deps()):
            return LIB
    tmp = LIB + ".tmp"
    cmd = [nvcc(), "-O3", "-std=c++17", *ARCH, "-lineinfo", "-Xcompiler", "-fPIC", "--threads", "2",
           "-shared", *SRC, "-o", tmp]
    if verbose:
        cmd.insert(1, "-Xptxas=-v")
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True, verbose=True))
