"""GB300-native implementation of the Cliffs time-stepping hot path.

The compute lives in the CUDA library behind include/cliffs_gpu.h
(csrc/cliffs_gpu.cu, built for sm_103a by build.py); cliffs_gpu.GpuGrid is its
Python binding.  workloads holds seeded synthetic inputs shaped like the
benchmark configurations.
"""
from . import build, workloads  # noqa: F401
from .cliffs_gpu import GpuGrid, Batch, CliffsError, load, metrics  # noqa: F401
