"""ctypes binding of libsvo.so (the C ABI in include/svo.h).

The library is the only compute path: if it cannot be loaded, every entry point raises.  There is no
CPU fallback.
"""
from __future__ import annotations

import ctypes
import os
import re

from . import build as _build

LIB_PATH = _build.LIB
HEADER = os.path.join(_build.ROOT, "include", "svo.h")

SVO_OK, SVO_ERR_INVALID, SVO_ERR_CAPACITY, SVO_ERR_OOM, SVO_ERR_TIMEOUT, SVO_ERR_CUDA = range(6)
STATUS_NAMES = {0: "SVO_OK", 1: "SVO_ERR_INVALID", 2: "SVO_ERR_CAPACITY", 3: "SVO_ERR_OOM", 4: "SVO_ERR_TIMEOUT",
                5: "SVO_ERR_CUDA"}

u32, u64, i32, f32, sz = ctypes.c_uint32, ctypes.c_uint64, ctypes.c_int, ctypes.c_float, ctypes.c_size_t
P = ctypes.c_void_p


class SvoError(RuntimeError):
    def __init__(self, code: int, message: str):
        super().__init__(f"{STATUS_NAMES.get(code, code)}: {message}")
        self.code = code


class Fraglist(ctypes.Structure):
    _fields_ = [("data", P), ("count", u32), ("level", u32), ("capacity", u64), ("owned", u32), ("units", u32)]


class OctreeC(ctypes.Structure):
    _fields_ = [("words", P), ("capacity", u64), ("range_words", u32), ("level", u32), ("owned", u32),
                ("reserved", u32)]


class BuildInfo(ctypes.Structure):
    _fields_ = [("level", u32), ("fragments", u32), ("range_words", u32), ("leaves", u32),
                ("level_nodes", u32 * 12)]


class CameraC(ctypes.Structure):
    _fields_ = [("pos", f32 * 4), ("look", f32 * 4), ("side", f32 * 4), ("up", f32 * 4)]


class LightingC(ctypes.Structure):
    """svo_lighting: light type, sun radiance, environment-map rotation / multiplier and handle."""
    _fields_ = [("type", ctypes.c_uint32), ("sun_radiance", ctypes.c_float * 3), ("envmap_rotation", ctypes.c_float),
                ("envmap_multiplier", ctypes.c_float), ("envmap", ctypes.c_void_p)]


class BatchMesh(ctypes.Structure):
    _fields_ = [("tris", P), ("n_tris", u32), ("level", u32)]


class ServerConfig(ctypes.Structure):
    _fields_ = [("hbm_budget_bytes", u64), ("lanes", u32), ("max_batch_rays", u32), ("max_batch_requests", u32),
                ("flags", u32)]


SVO_SERVER_COUNT_FETCHES = 1


class TraceRequest(ctypes.Structure):
    _fields_ = [("scene", u32), ("mode", u32), ("camera", CameraC), ("width", u32), ("height", u32),
                ("n_primary", u32), ("n_rays", u32), ("rays", P), ("hits", P), ("seed", u64)]


class RequestResult(ctypes.Structure):
    _fields_ = [("status", i32), ("batch_requests", u32), ("submit_us", ctypes.c_double),
                ("launch_us", ctypes.c_double), ("done_us", ctypes.c_double)]


class ServerStats(ctypes.Structure):
    _fields_ = [(n, u64) for n in ("submitted", "completed", "failed", "batches", "batched_requests", "rays",
                                   "rebuilds", "resident_bytes", "inflight_bytes", "pending", "node_fetches")]


SVO_REQUEST_CAMERA, SVO_REQUEST_RAYS = 0, 1

ALLOC_FN = ctypes.CFUNCTYPE(P, P, sz)
RELEASE_FN = ctypes.CFUNCTYPE(None, P, P)


class Allocator(ctypes.Structure):
    _fields_ = [("alloc", ALLOC_FN), ("release", RELEASE_FN), ("user", P)]


_SIGNATURES = {
    "svo_last_error": ([], ctypes.c_char_p),
    "svo_version": ([], ctypes.c_char_p),
    "svo_kernel_launches": ([], u64),
    "svo_allocation_calls": ([], u64),
    "svo_debug_wait_fault": ([u32, u32], i32),
    "svo_device_alloc": ([ctypes.POINTER(P), sz, P], i32),
    "svo_device_free": ([P, P], None),
    "svo_upload": ([P, P, sz, P], i32),
    "svo_download": ([P, P, sz, i32, P], i32),
    "svo_stream_synchronize": ([P], i32),
    "svo_profile_enable": ([i32], None),
    "svo_profile_summary": ([ctypes.c_char_p, sz], sz),
    "svo_voxelize": ([P, u32, u32, ctypes.POINTER(Fraglist), P], i32),
    "svo_voxelize_ex": ([P, u32, u32, ctypes.POINTER(Allocator), ctypes.POINTER(Fraglist), P], i32),
    "svo_voxelize_count": ([P, u32, u32, ctypes.POINTER(u64), P], i32),
    "svo_voxelize_workspace_size": ([u32, u64], sz),
    "svo_voxelize_into": ([P, u32, u32, P, u64, P, P, sz, P], i32),
    "svo_fraglist_destroy": ([ctypes.POINTER(Fraglist), P], None),
    "svo_voxelize_static": ([P, u32, u32, P, u64, P, P], i32),
    "svo_build": ([P, u32, u32, ctypes.POINTER(OctreeC), ctypes.POINTER(BuildInfo), P], i32),
    "svo_build_ex": ([P, u32, u32, ctypes.POINTER(Allocator), ctypes.POINTER(OctreeC), ctypes.POINTER(BuildInfo), P],
                     i32),
    "svo_build_fraglist": ([ctypes.POINTER(Fraglist), ctypes.POINTER(OctreeC), ctypes.POINTER(BuildInfo), P], i32),
    "svo_build_workspace_size": ([u32, u32, u64, u64], sz),
    "svo_build_pool_bound": ([u32, u32], u64),
    "svo_build_into": ([P, u32, u32, P, u64, P, sz, P, P], i32),
    "svo_octree_destroy": ([ctypes.POINTER(OctreeC), P], None),
    "svo_raycast": ([ctypes.POINTER(OctreeC), P, u32, P, P, P], i32),
    "svo_raycast_camera": ([ctypes.POINTER(OctreeC), ctypes.POINTER(CameraC), u32, u32, P, P, P], i32),
    "svo_raycast_camera_download": ([ctypes.POINTER(OctreeC), ctypes.POINTER(CameraC), u32, u32, P, P, P, P], i32),
    "svo_bounce_rays": ([P, u32, u64, P, P], i32),
    "svo_batcher_create": ([ctypes.POINTER(P)], i32),
    "svo_batcher_destroy": ([P], None),
    "svo_batcher_build": ([P, ctypes.POINTER(BatchMesh), u32, P], i32),
    "svo_batcher_meshes": ([P], u32),
    "svo_batcher_result": ([P, u32, ctypes.POINTER(Fraglist), ctypes.POINTER(OctreeC), ctypes.POINTER(BuildInfo)], i32),
    "svo_batcher_set_graph": ([P, i32], i32),
    "svo_batcher_stats": ([P, ctypes.POINTER(u64), ctypes.POINTER(u64)], None),
    "svo_server_create": ([ctypes.POINTER(ServerConfig), ctypes.POINTER(P)], i32),
    "svo_server_destroy": ([P], None),
    "svo_server_add_octree": ([P, ctypes.POINTER(OctreeC), ctypes.POINTER(u32)], i32),
    "svo_server_build_scene": ([P, P, u32, u32, ctypes.POINTER(u32)], i32),
    "svo_server_scene": ([P, u32, ctypes.POINTER(OctreeC)], i32),
    "svo_server_submit_trace": ([P, ctypes.POINTER(TraceRequest), ctypes.POINTER(u64)], i32),
    "svo_server_submit_rebuild": ([P, u32, P, u32, u32, ctypes.POINTER(u64)], i32),
    "svo_server_wait": ([P, u64, i32, ctypes.POINTER(RequestResult)], i32),
    "svo_server_get_stats": ([P, ctypes.POINTER(ServerStats)], None),
    "svo_beam_texels": ([u32, u32], u64),
    "svo_beam_prepass": ([ctypes.POINTER(OctreeC), ctypes.POINTER(CameraC), u32, u32, P, P], i32),
    "svo_raycast_camera_beam": ([ctypes.POINTER(OctreeC), ctypes.POINTER(CameraC), u32, u32, P, P, P, P], i32),
    "svo_occlude": ([ctypes.POINTER(OctreeC), P, u32, P, P], i32),
    "svo_load_obj": ([ctypes.c_char_p, ctypes.POINTER(P), ctypes.POINTER(u32)], i32),
    "svo_free_host": ([P], None),
    "svo_octree_write_host": ([P, u32, u32, ctypes.c_char_p], i32),
    "svo_octree_read_host": ([ctypes.c_char_p, ctypes.POINTER(P), ctypes.POINTER(u32), ctypes.POINTER(u32)], i32),
    "svo_octree_save": ([ctypes.POINTER(OctreeC), ctypes.c_char_p, P], i32),
    "svo_octree_load": ([ctypes.c_char_p, ctypes.POINTER(OctreeC), P], i32),
    "svo_tune_set": ([u32, u32, ctypes.c_int32, ctypes.c_int32], i32),
    "svo_tune_get": ([u32, u32, u64], i32),
    "svo_tune_size_class": ([u64], u32),
    "svo_tune_reset": ([], None),
    "svo_camera_from_angles": ([ctypes.POINTER(f32), f32, f32, f32, f32, ctypes.POINTER(CameraC)], None),
    "svo_texture_set_create": ([P, P, P, u32, ctypes.POINTER(P)], i32),
    "svo_texture_set_level": ([P, u32, u32, P, ctypes.POINTER(u32), ctypes.POINTER(u32)], i32),
    "svo_texture_set_destroy": ([P], None),
    "svo_voxelize_textured": ([P, P, u32, u32, P, ctypes.POINTER(Fraglist), P], i32),
    "svo_sobol_default_matrices": ([P], i32),
    "svo_envmap_create": ([P, u32, u32, ctypes.POINTER(P)], i32),
    "svo_envmap_tables": ([P, P, P], i32),
    "svo_envmap_destroy": ([P], None),
    "svo_path_tracer_create": ([u32, u32, u32, ctypes.POINTER(P)], i32),
    "svo_path_tracer_reset": ([P, u32, u32, u32, P], i32),
    "svo_path_tracer_set_noise": ([P, P, P], i32),
    "svo_path_tracer_set_sobol_matrices": ([P, P, P], i32),
    "svo_path_tracer_render": ([P, ctypes.POINTER(OctreeC), ctypes.POINTER(CameraC), ctypes.POINTER(LightingC), u32, P],
                               i32),
    "svo_path_tracer_info": ([P, ctypes.POINTER(u32), ctypes.POINTER(u32)], i32),
    "svo_path_tracer_images": ([P, ctypes.POINTER(P), ctypes.POINTER(P), ctypes.POINTER(P), ctypes.POINTER(P)], i32),
    "svo_path_tracer_extract": ([P, u32, P, P], i32),
    "svo_path_tracer_destroy": ([P], None),
}

_lib = None


def declared_symbols() -> list[str]:
    """Function names declared in include/svo.h."""
    with open(HEADER) as f:
        text = f.read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = re.findall(r"^[A-Za-z_][\w\s\*]*?\b(svo_\w+)\s*\(", text, flags=re.M)
    return sorted(set(names))


def load(build_if_needed: bool = True):
    """Load libsvo.so (building it first when sources are newer); raises if it cannot be loaded."""
    global _lib
    if _lib is not None:
        return _lib
    if build_if_needed and _build.needs_build():
        _build.build()
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(f"{LIB_PATH} is missing: build it with python -m sparsevoxeloctree_gb300.build")
    lib = ctypes.CDLL(LIB_PATH)
    for name, (args, res) in _SIGNATURES.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = res
    _lib = lib
    return lib


def check(code: int) -> None:
    if code != SVO_OK:
        raise SvoError(code, load().svo_last_error().decode())


def profile_summary() -> dict:
    """Per-kernel {name: {"launches": n, "ms": total}} since svo_profile_enable(1)."""
    import json
    lib = load()
    need = lib.svo_profile_summary(None, 0)
    buf = ctypes.create_string_buffer(need + 1)
    lib.svo_profile_summary(buf, need + 1)
    return json.loads(buf.value.decode())
