"""ctypes binding of oracle/_ref/libsvo_ref.so — the reference's own shader code compiled for the CPU.

TEST INFRASTRUCTURE ONLY.  The library is built by oracle/build_ref.py from the reference checkout and
exists only where that checkout does; `available()` says whether it can be loaded.  It is used to pin
the oracle (tests/test_oracle_pin.py) and to generate the fixtures in tests/golden/.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_ref", "libsvo_ref.so")
from .build_ref import DEFAULT_REFERENCE as REFERENCE_DIR  # noqa: E402  (the recipe owns the location)

_lib = None
_lib_etrig = None
LIB_ETRIG_PATH = os.path.join(HERE, "_ref", "libsvo_ref_etrig.so")


def build() -> bool:
    """Build the library when the reference checkout is present; True if it is available afterwards."""
    if os.path.isdir(os.path.join(REFERENCE_DIR, "shader")):
        subprocess.run([sys.executable, os.path.join(HERE, "build_ref.py"), "--reference", REFERENCE_DIR],
                       check=True, stdout=subprocess.DEVNULL)
    return os.path.exists(LIB_PATH)


def available() -> bool:
    try:
        lib()
        return True
    except OSError:
        return False


def lib(engine_trig: bool = False):
    """The reference build; engine_trig selects the one whose GLSL sin / cos / atan / acos are the
    engine's restatements instead of libm's."""
    global _lib, _lib_etrig
    cached = _lib_etrig if engine_trig else _lib
    if cached is None:
        path = LIB_ETRIG_PATH if engine_trig else LIB_PATH
        if not os.path.exists(path):
            build()
        L = ctypes.CDLL(path)
        P, u32, u64, i32, f32 = ctypes.c_void_p, ctypes.c_uint32, ctypes.c_uint64, ctypes.c_int, ctypes.c_float
        L.ref_build.argtypes = [P, u32, u32, P, u64]
        L.ref_build.restype = u64
        L.ref_raycast.argtypes = [P, u32, P, P, i32, P, P, P, P, P]
        L.ref_occlude.argtypes = [P, u32, P, P, P]
        L.ref_camera_rays.argtypes = [P, u32, u32, P]
        L.ref_beam.argtypes = [P, P, u32, u32, u32, f32, P]
        L.ref_diffuse_sample.argtypes = [P, f32, f32, P]
        L.ref_voxelize_triangle.argtypes = [P, u32, u32, i32, P, u64]
        L.ref_voxelize_triangle.restype = u64
        L.ref_voxelize_triangle_texel.argtypes = [P, P, u32, i32, P, u64]
        L.ref_voxelize_triangle_texel.restype = u64
        L.ref_sobol_matrices.argtypes = [P]
        L.ref_sobol_next.argtypes = [P, u32]
        L.ref_envmap_build.argtypes = [P, u32, u32, P]
        L.ref_envmap_build.restype = i32
        L.ref_path_trace.argtypes = [P, P, u32, u32, u32, u32, P, f32, f32, P, P, u32, u32, P, P, P, P, P, u32, P]
        if engine_trig:
            _lib_etrig = L
        else:
            _lib = L
        cached = L
    return cached


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def build_octree(frags: np.ndarray, level: int, capacity: int) -> np.ndarray:
    frags = np.ascontiguousarray(frags, np.uint64)
    pool = np.zeros(capacity, np.uint32)
    rng = lib().ref_build(_p(frags), len(frags), level, _p(pool), capacity)
    if rng == 0:
        raise RuntimeError("reference build overflowed the pool")
    return pool[:rng].copy()


def raycast(pool: np.ndarray, o: np.ndarray, d: np.ndarray, with_iter: bool = True) -> dict:
    pool = np.ascontiguousarray(pool, np.uint32)
    o = np.ascontiguousarray(o, np.float32)
    d = np.ascontiguousarray(d, np.float32)
    n = len(o)
    out = dict(hit=np.zeros(n, np.uint32), pos=np.zeros((n, 3), np.float32), color=np.zeros((n, 3), np.float32),
               normal=np.zeros((n, 3), np.float32), iter=np.zeros(n, np.uint32))
    lib().ref_raycast(_p(pool), n, _p(o), _p(d), int(with_iter), _p(out["hit"]), _p(out["pos"]), _p(out["color"]),
                      _p(out["normal"]), _p(out["iter"]))
    return out


def occlude(pool: np.ndarray, o: np.ndarray, d: np.ndarray) -> np.ndarray:
    pool = np.ascontiguousarray(pool, np.uint32)
    o = np.ascontiguousarray(o, np.float32)
    d = np.ascontiguousarray(d, np.float32)
    hit = np.zeros(len(o), np.uint32)
    lib().ref_occlude(_p(pool), len(o), _p(o), _p(d), _p(hit))
    return hit


def beam(pool: np.ndarray, cam, width: int, height: int, level: int, beam_size: int = 8) -> np.ndarray:
    """Beam image (start distance per tile corner) of the reference's beam pre-pass."""
    c = np.ascontiguousarray(np.frombuffer(np.asarray(cam).tobytes(), np.float32))
    bw, bh = (width + beam_size - 1) // beam_size + 1, (height + beam_size - 1) // beam_size + 1
    out = np.zeros((bh, bw), np.float32)
    lib().ref_beam(_p(np.ascontiguousarray(pool)), _p(c), width, height, beam_size,
                   float(np.ldexp(np.float32(1.0), 1 - level)), _p(out))
    return out


def camera_dirs(cam, width: int, height: int) -> np.ndarray:
    c = np.ascontiguousarray(np.concatenate([cam["pos"], cam["look"], cam["side"], cam["up"]]).astype(np.float32))
    dirs = np.zeros((width * height, 3), np.float32)
    lib().ref_camera_rays(_p(c), width, height, _p(dirs))
    return dirs


def diffuse_sample(normal, u1: float, u2: float) -> np.ndarray:
    n = np.ascontiguousarray(normal, np.float32)
    out = np.zeros(3, np.float32)
    lib().ref_diffuse_sample(_p(n), u1, u2, _p(out))
    return out


def voxelize_triangle(v9_ref: np.ndarray, albedo: int, level: int, conservative_sw: bool) -> np.ndarray:
    """Fragments of one triangle given in the reference's [-1,1] space."""
    v = np.ascontiguousarray(v9_ref, np.float32)
    cap = 1 << 16
    while True:
        out = np.zeros(cap, np.uint64)
        n = lib().ref_voxelize_triangle(_p(v), albedo, level, int(conservative_sw), _p(out), cap)
        if n <= cap:
            return out[:n]
        cap = int(n)


def sobol_matrices() -> np.ndarray:
    """kMatrices of shader/sobol.comp, (64, 32) uint32."""
    out = np.zeros((64, 32), np.uint32)
    lib().ref_sobol_matrices(_p(out))
    return out


def sobol_next(sobol: np.ndarray, dim: int) -> None:
    """shader/sobol.comp (one group of 64 invocations) on a uint32 state array, in place."""
    assert sobol.dtype == np.uint32 and sobol.flags.c_contiguous
    lib().ref_sobol_next(_p(sobol), dim)


def envmap_build(rgba: np.ndarray):
    """EnvironmentMap::weigh_hdr_image + generate_alias_table: (texels with the weight in alpha, alias
    table (h, w, 2)), or None for an image of zero weight."""
    tex = np.array(rgba, np.float32, copy=True, order="C")
    h, w = tex.shape[:2]
    alias = np.zeros((h, w, 2), np.uint32)
    if not lib().ref_envmap_build(_p(tex), w, h, _p(alias)):
        return None
    return tex, alias


def path_trace(pool: np.ndarray, cam, width: int, height: int, bounce: int, sobol: np.ndarray, noise: np.ndarray,
               color: np.ndarray, albedo: np.ndarray, normal: np.ndarray, light_type: int = 0,
               const_color=(5.0, 5.0, 5.0), rotation: float = 0.0, multiplier: float = 1.0, env=None,
               samples: int = 1, engine_trig: bool = False, matrices: np.ndarray | None = None) -> None:
    """shader/path_tracer.comp + shader/sobol.comp, `samples` times, updating the targets and the Sobol
    state in place (color (h, w, 4) float32; albedo / normal (h, w) uint32 rgba8 words).  matrices: other
    Sobol direction numbers (64 x 32) for sobol.comp to run with."""
    cam16 = np.ascontiguousarray(np.frombuffer(np.asarray(cam).tobytes(), np.float32))
    cc = np.ascontiguousarray(const_color, np.float32)
    if env is None:
        tex, alias, ew, eh = np.zeros(4, np.float32), np.zeros(2, np.uint32), 0, 0
    else:
        tex, alias = np.ascontiguousarray(env[0], np.float32), np.ascontiguousarray(env[1], np.uint32)
        eh, ew = tex.shape[0], tex.shape[1]
    for a in (sobol, color, albedo, normal):
        assert a.flags.c_contiguous
    lib(engine_trig).ref_path_trace(_p(np.ascontiguousarray(pool, np.uint32)), _p(cam16), width, height, bounce,
                                    light_type,
                         _p(cc), rotation, multiplier, _p(tex), _p(alias), ew, eh, _p(sobol),
                         _p(np.ascontiguousarray(noise, np.uint8)), _p(color), _p(albedo), _p(normal), samples,
                         None if matrices is None else _p(np.ascontiguousarray(matrices, np.uint32)))


def voxelize_triangle_texel(v9_ref: np.ndarray, texel_linear, level: int, conservative_sw: bool) -> np.ndarray:
    """voxelizer.frag with a 1x1 texture of linear rgba `texel_linear` bound (alpha discard, packUnorm4x8)."""
    v = np.ascontiguousarray(v9_ref, np.float32)
    t = np.ascontiguousarray(texel_linear, np.float32)
    cap = 1 << 16
    out = np.zeros(cap, np.uint64)
    n = lib().ref_voxelize_triangle_texel(_p(v), _p(t), level, int(conservative_sw), _p(out), cap)
    return out[: min(int(n), cap)]
