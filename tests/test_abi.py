"""The C ABI library: it loads, exports every function include/svo.h declares, and its host-side
argument checks and helpers behave (no kernel runs here)."""
import ctypes

import numpy as np
import pytest

from sparsevoxeloctree_gb300 import _lib


@pytest.fixture(scope="module")
def lib():
    return _lib.load()


def test_exports_every_declared_symbol(lib):
    names = _lib.declared_symbols()
    assert len(names) >= 20
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_version_and_counters(lib):
    assert b"sm_103a" in lib.svo_version()
    assert lib.svo_kernel_launches() >= 0


def test_invalid_arguments_are_rejected_before_any_launch(lib):
    before = lib.svo_kernel_launches()
    out = _lib.Fraglist()
    assert lib.svo_voxelize(None, 0, 0, ctypes.byref(out), None) == _lib.SVO_ERR_INVALID
    assert b"level" in lib.svo_last_error()
    assert lib.svo_voxelize(None, 0, 13, ctypes.byref(out), None) == _lib.SVO_ERR_INVALID
    assert lib.svo_voxelize(None, 5, 4, ctypes.byref(out), None) == _lib.SVO_ERR_INVALID
    assert lib.svo_voxelize(ctypes.c_void_p(8), 5, 4, ctypes.byref(out), None) == _lib.SVO_ERR_INVALID  # misaligned
    oc = _lib.OctreeC()
    assert lib.svo_build(None, 0, 0, ctypes.byref(oc), None, None) == _lib.SVO_ERR_INVALID
    assert lib.svo_build(ctypes.c_void_p(4), 3, 5, ctypes.byref(oc), None, None) == _lib.SVO_ERR_INVALID
    assert lib.svo_raycast(ctypes.byref(oc), None, 0, None, None, None) == _lib.SVO_ERR_INVALID  # null octree
    oc.words, oc.level, oc.range_words = 256, 5, 12  # range not a multiple of 8
    assert lib.svo_raycast(ctypes.byref(oc), None, 0, None, None, None) == _lib.SVO_ERR_INVALID
    oc.range_words = 16
    cam = _lib.CameraC()
    dl = lib.svo_raycast_camera_download
    assert dl(ctypes.byref(oc), None, 4, 4, None, None, None, None) == _lib.SVO_ERR_INVALID  # null camera
    assert dl(ctypes.byref(oc), ctypes.byref(cam), 4, 4, None, None, None, None) == _lib.SVO_ERR_INVALID  # no host buffer
    assert dl(ctypes.byref(oc), ctypes.byref(cam), 4, 4, None, ctypes.c_void_p(8), None, None) == _lib.SVO_ERR_INVALID
    assert b"aligned" in lib.svo_last_error()
    assert dl(ctypes.byref(oc), ctypes.byref(cam), 0, 4, None, None, None, None) == _lib.SVO_OK  # empty image
    assert lib.svo_build_into(ctypes.c_void_p(256), 1, 3, ctypes.c_void_p(256), 4, ctypes.c_void_p(256), 1 << 20,
                              ctypes.c_void_p(256), None) == _lib.SVO_ERR_CAPACITY
    assert lib.svo_build_into(ctypes.c_void_p(256), 1, 3, ctypes.c_void_p(256), 64, ctypes.c_void_p(256), 64,
                              ctypes.c_void_p(256), None) == _lib.SVO_ERR_CAPACITY  # workspace too small
    assert lib.svo_kernel_launches() == before


def test_pool_bound_and_workspace_sizes(lib):
    import oracle
    for count, level in [(0, 1), (1, 1), (5, 3), (1000, 8), (38_000_000, 10), (150_000_000, 12)]:
        assert lib.svo_build_pool_bound(count, level) == oracle.pool_bound(count, level)
    cap = lib.svo_build_pool_bound(1000, 8)
    # the bucketed fragment copy (8 B per fragment) dominates; the leaf level needs no device scratch
    assert lib.svo_build_workspace_size(1000, 8, cap, 0) == lib.svo_build_workspace_size(1000, 8, cap, 64) > 8000
    assert lib.svo_voxelize_workspace_size(1000, 0) > 8 * 1000
    assert lib.svo_voxelize_workspace_size(1000, 10**6) > lib.svo_voxelize_workspace_size(1000, 0)


def test_camera_from_angles_matches_python(lib):
    from sparsevoxeloctree_gb300 import scenes
    pos = (ctypes.c_float * 3)(1.5, 1.4, 1.3)
    cam = _lib.CameraC()
    lib.svo_camera_from_angles(pos, 0.3, -0.2, np.pi / 3, 1.5, ctypes.byref(cam))
    ref = scenes.camera_from_angles((1.5, 1.4, 1.3), 0.3, -0.2, np.pi / 3, 1.5)
    for k in ("pos", "look", "side", "up"):
        assert np.allclose(np.array(getattr(cam, k)[:3]), ref[k][:3], atol=1e-6)


def test_batcher_rejects_bad_batches_before_any_launch(lib):
    before = lib.svo_kernel_launches()
    h = ctypes.c_void_p()
    assert lib.svo_batcher_create(ctypes.byref(h)) == _lib.SVO_OK
    try:
        assert lib.svo_batcher_build(h, None, 0, None) == _lib.SVO_ERR_INVALID  # empty batch
        arr = (_lib.BatchMesh * 2)()
        arr[0].tris, arr[0].n_tris, arr[0].level = 256, 1, 8
        arr[1].tris, arr[1].n_tris, arr[1].level = 256, 1, 13  # level out of range
        assert lib.svo_batcher_build(h, arr, 2, None) == _lib.SVO_ERR_INVALID
        assert b"mesh 1" in lib.svo_last_error()
        arr[1].level, arr[1].tris = 8, 8  # misaligned triangles
        assert lib.svo_batcher_build(h, arr, 2, None) == _lib.SVO_ERR_INVALID
        arr[1].tris = None  # null buffer with triangles
        assert lib.svo_batcher_build(h, arr, 2, None) == _lib.SVO_ERR_INVALID
        assert lib.svo_batcher_meshes(h) == 0
        assert lib.svo_batcher_result(h, 0, None, None, None) == _lib.SVO_ERR_INVALID
        c, r = _lib.u64(), _lib.u64()
        lib.svo_batcher_stats(h, ctypes.byref(c), ctypes.byref(r))
        assert c.value == 0 and r.value == 0
    finally:
        lib.svo_batcher_destroy(h)
    assert lib.svo_kernel_launches() == before


def test_launch_parameter_table(lib):
    from sparsevoxeloctree_gb300 import autotune
    lib.svo_tune_reset()
    try:
        assert autotune.size_class(1000) == 0 and autotune.size_class(1 << 16) == 1
        assert autotune.size_class(38_000_000) == 5 and autotune.size_class(1 << 40) == 7
        assert autotune.get("march_block", 10, 2_000_000) == 128
        autotune.set_value("march_block", 10, autotune.size_class(2_000_000), 256)
        assert autotune.get("march_block", 10, 2_000_000) == 256
        assert autotune.get("march_block", 9, 2_000_000) == 128      # other level untouched
        assert autotune.get("march_block", 10, 20_000_000) == 128     # other size class untouched
        autotune.set_value("leaf_blocks", 0, -1, 8)                    # every level and class
        assert all(autotune.get("leaf_blocks", lv, 10 ** k) == 8 for lv in (1, 7, 12) for k in (3, 6, 9))
        assert autotune.get("build_streams", 10, 1000) == 2
        assert autotune.get("march_buffer_rays", 10, 1000) == 1
        assert autotune.get("download_bands", 10, 1000) == 0
        autotune.set_value("build_streams", 10, 0, 1)
        assert autotune.get("build_streams", 10, 1000) == 1
        for bad in ((0, 10, 3, 100), (1, 10, 3, 3), (2, 10, 3, 2), (3, 10, 3, 0), (3, 13, 3, 8), (3, 10, 8, 8),
                    (6, 10, 3, 3), (8, 10, 3, 3), (9, 10, 3, 8)):
            assert lib.svo_tune_set(*bad) == _lib.SVO_ERR_INVALID
        t = autotune.table()
        assert t["march_block"]["default"] == 128 and t["march_block"]["10:3"] == 256
        assert t["leaf_blocks"]["default"] == 8
    finally:
        lib.svo_tune_reset()
    assert autotune.get("leaf_blocks", 10, 1000) == 6
