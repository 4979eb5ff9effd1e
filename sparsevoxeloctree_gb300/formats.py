"""Binary formats shared by the C ABI (include/svo.h) and Python callers.

numpy dtypes mirror the C structs byte for byte; helpers pack and unpack the reference's fragment and
node-word encodings:

* fragment (shader/voxelizer.frag:40-42): x = vx | vy<<12 | (vz&0xff)<<24, y = (vz>>8)<<28 | rgb24,
  stored as one little-endian uint64 (low word x, high word y);
* node word (shader/octree_tag_node.comp:10-16,59, shader/octree_alloc_node.comp:21): 0 = empty,
  bit31 = non-empty, interior bits 0-29 = child block word index, leaf = 0xC0000000 | min(n,63)<<24 | rgb.
"""
from __future__ import annotations

import numpy as np

TRIANGLE_DTYPE = np.dtype([("v", "<f4", (9,)), ("rgb", "<u4", (3,))], align=True)
RAY_DTYPE = np.dtype([("o", "<f4", (3,)), ("d", "<f4", (3,))], align=True)
CAMERA_DTYPE = np.dtype([("pos", "<f4", (4,)), ("look", "<f4", (4,)), ("side", "<f4", (4,)),
                         ("up", "<f4", (4,))], align=True)
HIT_DTYPE = np.dtype([("t", "<f4"), ("pos", "<f4", (3,)), ("node", "<u4"), ("iter", "<u4"),
                      ("voxel", "<u2", (3,)), ("flags", "<u2")], align=True)

assert TRIANGLE_DTYPE.itemsize == 48
assert RAY_DTYPE.itemsize == 24
assert CAMERA_DTYPE.itemsize == 64
assert HIT_DTYPE.itemsize == 32

LEVEL_MIN = 1
LEVEL_MAX = 12
MAX_POOL_WORDS = 1 << 30
STACK_SIZE = 23

HIT_FLAG_HIT = 1
HIT_NORMAL_NEG = 8
HIT_FLAG_ABORTED = 16  # malformed pool: pointer outside the range, interior word below the level, or the iteration bound

NODE_NONEMPTY = 0x80000000
NODE_LEAF = 0x40000000
NODE_PTR_MASK = 0x3FFFFFFF


def pack_fragments(x: np.ndarray, y: np.ndarray, z: np.ndarray, rgb: np.ndarray) -> np.ndarray:
    """Encode voxel coordinates and colours the way shader/voxelizer.frag:40-42 does."""
    x = np.asarray(x, np.uint64)
    y = np.asarray(y, np.uint64)
    z = np.asarray(z, np.uint64)
    rgb = np.asarray(rgb, np.uint64)
    fx = x | (y << np.uint64(12)) | ((z & np.uint64(0xFF)) << np.uint64(24))
    fy = ((z >> np.uint64(8)) << np.uint64(28)) | (rgb & np.uint64(0xFFFFFF))
    return fx | (fy << np.uint64(32))


def unpack_fragments(frags: np.ndarray):
    """Inverse of pack_fragments: returns (x, y, z, rgb) as uint32 arrays."""
    f = np.asarray(frags, np.uint64)
    fx = (f & np.uint64(0xFFFFFFFF)).astype(np.uint32)
    fy = (f >> np.uint64(32)).astype(np.uint32)
    x = fx & 0xFFF
    y = (fx >> 12) & 0xFFF
    z = (fx >> 24) | ((fy >> 28) << 8)
    return x, y, z, fy & 0xFFFFFF


def fragment_keys(frags: np.ndarray) -> np.ndarray:
    """Sorted uint64 keys of a fragment list: multiset comparison is array equality of these."""
    return np.sort(np.asarray(frags, np.uint64), kind="stable")


def rays_from_arrays(o: np.ndarray, d: np.ndarray) -> np.ndarray:
    rays = np.zeros(len(d), RAY_DTYPE)
    rays["o"] = o
    rays["d"] = d
    return rays
