"""GB300-native (sm_103a) implementation of range_libc's batched ray-casting path.

* ``range_libc_gb300.range_libc`` -- the reference's Python API (PyOMap,
  PyBresenhamsLine, PyRayMarching, PyCDDTCast, PyGiantLUTCast, PyRayMarchingGPU) over the GPU.
* ``include/rangelibc.h`` -- the C ABI; ``include/RangeLib.h`` -- the C++ API.
* ``range_libc_gb300.build`` -- nvcc build of ``_build/librangelibc_gb300.so``.
* ``range_libc_gb300.workloads`` -- seeded synthetic maps, poses and tables.
"""
from .build import build, LIB_PATH  # noqa: F401

__all__ = ["build", "LIB_PATH"]
