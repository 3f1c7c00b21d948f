"""vecgeom_gb300 -- GB300-native (sm_103a) batched BVH navigation for VecGeom geometries.

The compute path is libvgnav.so (C ABI in include/vgnav.h): hand-written CUDA
kernels for the navigation step, safety, point location and the per-shape
distance/safety queries.  This package holds its in-tree build, a ctypes
binding, a Python mirror of VecGeom's batched navigator interface and the
seeded synthetic workloads.
"""
from .navigator import SOA3D, BVHNavigator, Geometry, NavStatePool, StepBatch  # noqa: F401
from .workloads import GeometryBuilder, GeometryDescription  # noqa: F401

__all__ = ["SOA3D", "BVHNavigator", "Geometry", "NavStatePool", "StepBatch", "GeometryBuilder",
           "GeometryDescription"]
