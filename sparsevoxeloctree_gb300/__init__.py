"""GB300-native sparse-voxel-octree engine: voxelize -> build -> ray march, in hand-written sm_103a CUDA.

The compute lives in libsvo.so (C ABI: include/svo.h).  This package holds its ctypes binding, the
host-side mirror of the reference's Voxelizer / OctreeBuilder / Octree / OctreeTracer / PathTracer classes, the
binary formats and the synthetic benchmark scenes.
"""
import importlib

from .formats import CAMERA_DTYPE, HIT_DTYPE, RAY_DTYPE, TRIANGLE_DTYPE  # noqa: F401

_API_NAMES = ("Voxelizer", "OctreeBuilder", "Octree", "OctreeTracer", "PathTracer", "Lighting", "EnvironmentMap",
              "BatchBuilder", "Server", "voxelize", "raycast")


def __getattr__(name):
    # the torch-dependent API is imported lazily so the formats and scenes work without torch/CUDA
    if name in _API_NAMES:
        return getattr(importlib.import_module(__name__ + ".api"), name)
    raise AttributeError(name)
