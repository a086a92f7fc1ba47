"""GB300-native execution backend for ComputeQL's GPU operators.

libcqlcuda.so  - the backend behind include/cqlcuda.h (drop-in for the reference's src/gpu backend)
libcqlops.so   - the C99 operator layer over it (include/cqlops.h)
"""
from . import native  # noqa: F401

__all__ = ["native", "ops", "build"]
