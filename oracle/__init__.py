"""CPU oracle of the sparse-voxel-octree hot path — TEST INFRASTRUCTURE ONLY.

A plain-C restatement (oracle/oracle.c) of the reference's voxelize / build / march logic, loaded with
ctypes.  Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may import this package;
the engine (sparsevoxeloctree_gb300) never does.  Its parity with the reference's own shader source is
pinned by tests/test_oracle_pin.py against oracle/_ref (built by oracle/build_ref.py) and by the
fixtures in tests/golden/.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

from sparsevoxeloctree_gb300.formats import CAMERA_DTYPE, HIT_DTYPE, RAY_DTYPE, TRIANGLE_DTYPE

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")

COLOR_DET = 0
COLOR_REF = 1


def build(force: bool = False) -> str:
    """Compile liboracle.so with the committed Makefile (gcc, seconds)."""
    if force or not os.path.exists(LIB_PATH) or _stale():
        subprocess.run(["make", "-s", "-C", HERE, "-B" if force else "liboracle.so"], check=True)
    return LIB_PATH


def _stale() -> bool:
    t = os.path.getmtime(LIB_PATH)
    for f in ("oracle.c", "oracle.h", "svo_trig.h", os.path.join("..", "include", "svo.h")):
        if os.path.getmtime(os.path.join(HERE, f)) > t:
            return True
    return False


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB_PATH)
        P = ctypes.c_void_p
        u32, u64, i32 = ctypes.c_uint32, ctypes.c_uint64, ctypes.c_int
        L.oracle_set_threads.argtypes = [i32]
        L.oracle_get_threads.restype = i32
        L.oracle_voxelize_count.argtypes = [P, u32, u32, P]
        L.oracle_voxelize_count.restype = u64
        L.oracle_voxelize_emit.argtypes = [P, u32, u32, P, P]
        L.oracle_triangle_info.argtypes = [P, u32, P]
        L.oracle_build.argtypes = [P, u64, u32, i32, P, u64, P, ctypes.POINTER(i32)]
        L.oracle_build.restype = u64
        L.oracle_canonicalize.argtypes = [P, u64, P]
        L.oracle_canonicalize.restype = i32
        L.oracle_raycast.argtypes = [P, u64, u32, P, u64, P, P]
        L.oracle_camera_rays.argtypes = [P, u32, u32, P]
        L.oracle_occlude.argtypes = [P, u64, u32, P, u64, P]
        L.oracle_beam.argtypes = [P, u64, u32, P, u32, u32, u32, P]
        L.oracle_camera_rays_beam.argtypes = [P, u32, u32, P, u32, P]
        L.oracle_bounce_rays.argtypes = [P, u64, u64, P]
        L.oracle_diffuse_sample.argtypes = [P, ctypes.c_float, ctypes.c_float, P]
        f32 = ctypes.c_float
        L.oracle_pt_render.argtypes = [P, u64, u32, P, u32, u32, u32, u32, P, f32, f32, P, P, u32, u32, P, P, P,
                                       P, P]
        L.oracle_sobol_next.argtypes = [P, P, u32]
        L.oracle_envmap_build.argtypes = [P, u32, u32, P]
        L.oracle_envmap_build.restype = i32
        L.oracle_trig.argtypes = [f32, f32, P]
        L.oracle_texture_mips.argtypes = [P, u32, u32, P]
        L.oracle_texture_mips.restype = u32
        L.oracle_voxelize_textured.argtypes = [P, P, u32, u32, P, P, P, u32, P]
        L.oracle_voxelize_textured.restype = u64
        _lib = L
    return _lib


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(ctypes.c_void_p)


def set_threads(n: int) -> None:
    lib().oracle_set_threads(int(n))


def threads() -> int:
    return int(lib().oracle_get_threads())


def voxelize(tris: np.ndarray, level: int, return_counts: bool = False):
    """Fragments of `tris` (TRIANGLE_DTYPE) in canonical order, as uint64."""
    tris = np.ascontiguousarray(tris, TRIANGLE_DTYPE)
    n = len(tris)
    counts = np.zeros(max(n, 1), np.uint32)
    total = lib().oracle_voxelize_count(_ptr(tris), n, level, _ptr(counts))
    offsets = np.zeros(n + 1, np.uint64)
    np.cumsum(counts[:n], out=offsets[1:])
    frags = np.zeros(max(int(total), 1), np.uint64)
    lib().oracle_voxelize_emit(_ptr(tris), n, level, _ptr(offsets), _ptr(frags))
    frags = frags[: int(total)]
    return (frags, counts[:n]) if return_counts else frags


TRI_INFO_DTYPE = np.dtype([(k, "<i4") for k in ("axis", "i0", "i1", "j0", "j1", "z0", "z1", "cols",
                                                 "degenerate")] + [("rgb", "<u4")])


def triangle_info(tri: np.ndarray, level: int) -> dict:
    tri = np.ascontiguousarray(np.asarray(tri, TRIANGLE_DTYPE).reshape(1))
    info = np.zeros(1, TRI_INFO_DTYPE)
    lib().oracle_triangle_info(_ptr(tri), level, _ptr(info))
    return {k: int(info[k][0]) for k in TRI_INFO_DTYPE.names}


def pool_bound(count: int, level: int) -> int:
    """Upper bound on the words a build can use (every fragment adds at most one node per depth)."""
    words = 8
    for i in range(1, level):
        words += 8 * min(8 ** i, count)
    return min(words, 1 << 30)


def build_octree(frags: np.ndarray, level: int, color_mode: int = COLOR_DET, capacity: int | None = None,
                 return_level_nodes: bool = False):
    """Octree node pool (uint32, exactly `range` words) of a fragment list."""
    frags = np.ascontiguousarray(frags, np.uint64)
    cap = pool_bound(len(frags), level) if capacity is None else int(capacity)
    pool = np.zeros(max(cap, 8), np.uint32)
    level_nodes = np.zeros(12, np.uint32)
    status = ctypes.c_int(0)
    rng = lib().oracle_build(_ptr(frags), len(frags), level, color_mode, _ptr(pool), cap, _ptr(level_nodes),
                             ctypes.byref(status))
    if status.value != 0:
        raise RuntimeError(f"oracle_build failed with status {status.value}")
    pool = pool[: int(rng)].copy()
    return (pool, level_nodes[:level].copy()) if return_level_nodes else pool


def canonicalize(pool: np.ndarray) -> np.ndarray:
    pool = np.ascontiguousarray(pool, np.uint32)
    out = np.zeros_like(pool)
    if lib().oracle_canonicalize(_ptr(pool), len(pool), _ptr(out)) != 0:
        raise ValueError("malformed octree pool")
    return out


def raycast(pool: np.ndarray, level: int, rays: np.ndarray, return_fetches: bool = False):
    pool = np.ascontiguousarray(pool, np.uint32)
    rays = np.ascontiguousarray(rays, RAY_DTYPE)
    hits = np.zeros(len(rays), HIT_DTYPE)
    fetches = np.zeros(max(len(rays), 1), np.uint32)
    lib().oracle_raycast(_ptr(pool), len(pool), level, _ptr(rays), len(rays), _ptr(hits), _ptr(fetches))
    return (hits, fetches[: len(rays)]) if return_fetches else hits


def camera_rays(cam: np.ndarray, width: int, height: int) -> np.ndarray:
    cam = np.ascontiguousarray(np.asarray(cam, CAMERA_DTYPE).reshape(1))
    rays = np.zeros(width * height, RAY_DTYPE)
    lib().oracle_camera_rays(_ptr(cam), width, height, _ptr(rays))
    return rays


def occlude(pool: np.ndarray, level: int, rays: np.ndarray) -> np.ndarray:
    """Octree_RayMarchOcclude per ray (1 = the ray hits a leaf)."""
    pool = np.ascontiguousarray(pool, np.uint32)
    rays = np.ascontiguousarray(rays, RAY_DTYPE)
    out = np.zeros(len(rays), np.uint32)
    lib().oracle_occlude(_ptr(pool), len(pool), level, _ptr(rays), len(rays), _ptr(out))
    return out


BEAM_SIZE = 8  # kBeamSize: pixels per beam tile edge


def beam(pool: np.ndarray, level: int, cam: np.ndarray, width: int, height: int, beam_size: int = BEAM_SIZE):
    """Beam pre-pass: start distance per tile corner, shape ((H+bs-1)//bs+1, (W+bs-1)//bs+1)."""
    pool = np.ascontiguousarray(pool, np.uint32)
    cam = np.ascontiguousarray(np.asarray(cam, CAMERA_DTYPE).reshape(1))
    bw, bh = (width + beam_size - 1) // beam_size + 1, (height + beam_size - 1) // beam_size + 1
    out = np.zeros((bh, bw), np.float32)
    lib().oracle_beam(_ptr(pool), len(pool), level, _ptr(cam), width, height, beam_size, _ptr(out))
    return out


def camera_rays_beam(cam: np.ndarray, width: int, height: int, beam_img: np.ndarray, beam_size: int = BEAM_SIZE):
    """Primary rays advanced by the beam image (o += d * min of the 4 texels around the pixel's tile)."""
    cam = np.ascontiguousarray(np.asarray(cam, CAMERA_DTYPE).reshape(1))
    rays = np.zeros(width * height, RAY_DTYPE)
    lib().oracle_camera_rays_beam(_ptr(cam), width, height, _ptr(np.ascontiguousarray(beam_img, np.float32)),
                                  beam_size, _ptr(rays))
    return rays


def bounce_rays(hits: np.ndarray, seed: int) -> np.ndarray:
    hits = np.ascontiguousarray(hits, HIT_DTYPE)
    rays = np.zeros(len(hits), RAY_DTYPE)
    lib().oracle_bounce_rays(_ptr(hits), len(hits), seed & 0xFFFFFFFFFFFFFFFF, _ptr(rays))
    return rays


def diffuse_sample(normal, u1: float, u2: float) -> np.ndarray:
    n = np.ascontiguousarray(normal, np.float32)
    out = np.zeros(3, np.float32)
    lib().oracle_diffuse_sample(_ptr(n), u1, u2, _ptr(out))
    return out


# ---------------------------------------------------------------------------------------------- path tracer
class PathTraceState:
    """Accumulation targets and Sobol state of one path-traced image, advanced by render()."""

    def __init__(self, width: int, height: int, bounce: int, matrices: np.ndarray, noise: np.ndarray):
        self.width, self.height, self.bounce = width, height, bounce
        self.color = np.zeros((height, width, 4), np.float32)
        self.albedo = np.zeros((height, width), np.uint32)
        self.normal = np.zeros((height, width), np.uint32)
        self.sobol = np.zeros(65, np.uint32)
        self.matrices = np.ascontiguousarray(matrices, np.uint32).reshape(64 * 32)
        self.noise = np.ascontiguousarray(noise, np.uint8).reshape(256 * 256 * 2)

    def render(self, pool: np.ndarray, level: int, cam: np.ndarray, light_type: int = 0, const_color=(5.0, 5.0, 5.0),
               rotation: float = 0.0, multiplier: float = 1.0, env=None, samples: int = 1) -> None:
        """`samples` x (one sample per pixel, then the Sobol step).  env: (texels (h, w, 4) float32 with the
        pdf weight in alpha, alias (h, w, 2) uint32) from envmap_build."""
        pool = np.ascontiguousarray(pool, np.uint32)
        cam = np.ascontiguousarray(np.asarray(cam, CAMERA_DTYPE).reshape(1))
        cc = np.ascontiguousarray(const_color, np.float32)
        if env is None:
            tex, alias, ew, eh = np.zeros(4, np.float32), np.zeros(2, np.uint32), 0, 0
        else:
            tex, alias = np.ascontiguousarray(env[0], np.float32), np.ascontiguousarray(env[1], np.uint32)
            eh, ew = tex.shape[0], tex.shape[1]
        dim = 2 * (self.bounce + 1)
        for _ in range(samples):
            lib().oracle_pt_render(_ptr(pool), len(pool), level, _ptr(cam), self.width, self.height, self.bounce,
                                   light_type, _ptr(cc), rotation, multiplier, _ptr(tex), _ptr(alias), ew, eh,
                                   _ptr(self.sobol), _ptr(self.noise), _ptr(self.color), _ptr(self.albedo),
                                   _ptr(self.normal))
            lib().oracle_sobol_next(_ptr(self.sobol), _ptr(self.matrices), dim)


def sobol_next(sobol: np.ndarray, matrices: np.ndarray, dim: int) -> None:
    """Sobol::CmdNext in place on a uint32 state array."""
    assert sobol.dtype == np.uint32 and sobol.flags.c_contiguous
    lib().oracle_sobol_next(_ptr(sobol), _ptr(np.ascontiguousarray(matrices, np.uint32)), dim)


def envmap_build(rgba: np.ndarray):
    """(texels with the pdf weight in alpha, alias table (h, w, 2)) of an (h, w, 4) float32 image, or None
    when the image has no positive luminance."""
    tex = np.array(rgba, np.float32, copy=True, order="C")
    h, w = tex.shape[:2]
    alias = np.zeros((h, w, 2), np.uint32)
    if not lib().oracle_envmap_build(_ptr(tex), w, h, _ptr(alias)):
        return None
    return tex, alias


def trig(x: float, y: float) -> np.ndarray:
    """(sin x, cos x, atan2(y, x), acos x) by the engine's float restatements."""
    out = np.zeros(4, np.float32)
    lib().oracle_trig(x, y, _ptr(out))
    return out


UV_DTYPE = np.dtype([("uv", "<f4", (6,)), ("texture", "<u4"), ("reserved", "<u4")])


def texture_mips(rgba: np.ndarray) -> list:
    """Mip chain of an (h, w, 4) uint8 texture: a list of (h_l, w_l, 4) uint8 levels."""
    img = np.ascontiguousarray(rgba, np.uint8)
    h, w = img.shape[:2]
    out = np.zeros(w * h * 4 * 2 + 256, np.uint8)
    levels = lib().oracle_texture_mips(_ptr(img), w, h, _ptr(out))
    res, off = [], 0
    for lv in range(levels):
        wl, hl = max(1, w >> lv), max(1, h >> lv)
        res.append(out[off: off + wl * hl * 4].reshape(hl, wl, 4).copy())
        off += wl * hl * 4
    return res


def voxelize_textured(tris: np.ndarray, uvs: np.ndarray, level: int, textures: list) -> np.ndarray:
    """Fragments with texture-sampled colour (textures: (h, w, 4) uint8 images)."""
    tris = np.ascontiguousarray(tris, TRIANGLE_DTYPE)
    uvs = np.ascontiguousarray(uvs, UV_DTYPE)
    imgs = [np.ascontiguousarray(t, np.uint8) for t in textures]
    ptrs = (ctypes.c_void_p * max(1, len(imgs)))(*[i.ctypes.data for i in imgs])
    ws = np.array([i.shape[1] for i in imgs] + [0], np.uint32)
    hs = np.array([i.shape[0] for i in imgs] + [0], np.uint32)
    total = lib().oracle_voxelize_count(_ptr(tris), len(tris), level, None)
    out = np.zeros(max(int(total), 1), np.uint64)
    n = lib().oracle_voxelize_textured(_ptr(tris), _ptr(uvs), len(tris), level, ptrs, _ptr(ws), _ptr(hs), len(imgs),
                                       _ptr(out))
    return out[: int(n)]
