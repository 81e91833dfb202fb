"""lvr2_gb300: the lvr2 surface-reconstruction hot path on GB300 (sm_103a).

LBVH kNN, point normals (flip + interpolation), signed distance at grid
vertices and marching cubes, behind the C ABI of include/lvrgb.h
(liblvrgb.so).  This package holds the build recipe, the ctypes binding and a
Python mirror of lvr2's PointsetSurface / CudaSurface calls; the C++ mirror is
in lvr2_gb300/cpp.
"""
from ._lib import LvrgbError, load
from .surface import Batch, Surface

__all__ = ["Surface", "Batch", "LvrgbError", "load"]
