"""svo_voxelize_static: voxelization for callers that cannot allocate device memory.

Such callers (a frame loop that forbids allocation after start-up, a thread that holds an allocator
lock, a device whose memory is carved up in advance) pass their own triangle and fragment buffers; the
engine's scratch is a fixed array in device memory.  The test calls the entry point through the C ABI
and checks its fragments against the allocating entry point (svo_voxelize_ex): bit-exact, order included
(both run the same kernels), on consecutive calls, so later calls run on the scratch the earlier ones
left behind.  Around every call it reads the library's allocation counter (svo_allocation_calls, bumped
by every device, pinned-host and caller-allocator request the library makes) and checks the call made
none.  It runs alone in a fresh process as well as after the rest of the suite.
"""
import ctypes

import numpy as np
import pytest

from sparsevoxeloctree_gb300 import scenes
from sparsevoxeloctree_gb300.formats import TRIANGLE_DTYPE

pytestmark = pytest.mark.gpu

STATIC_MAX_TRIS = 262144


def _fragments_allocating(tris_dev, n, level):
    """The existing allocating entry point (svo_voxelize_ex through the C ABI, torch-owned memory)."""
    from sparsevoxeloctree_gb300 import api
    v = api.Voxelizer.Create(tris_dev, level)
    assert v.GetVoxelFragmentCount() >= 0
    return v.GetVoxelFragmentList().cpu().numpy().view(np.uint64)


def _fragments_static(tris_dev, n, level, capacity):
    """The entry point under test, with caller-owned fragment and count buffers."""
    import torch

    from sparsevoxeloctree_gb300 import _lib
    lib = _lib.load()
    frags = torch.empty(max(capacity, 1), dtype=torch.int64, device=tris_dev.device)
    count = torch.full((2,), -1, dtype=torch.int64, device=tris_dev.device)
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    allocs = lib.svo_allocation_calls()
    rc = lib.svo_voxelize_static(ctypes.c_void_p(tris_dev.data_ptr()), n, level, ctypes.c_void_p(frags.data_ptr()),
                                 capacity, ctypes.c_void_p(count.data_ptr()), stream)
    assert rc == _lib.SVO_OK, lib.svo_last_error()
    assert lib.svo_allocation_calls() == allocs  # the call allocated nothing
    torch.cuda.synchronize()
    produced, status = (int(v) for v in count.cpu())
    assert status == 0
    return produced, frags[: min(produced, capacity)].cpu().numpy().view(np.uint64)


def _upload(tris):
    import torch
    return torch.from_numpy(np.ascontiguousarray(tris, TRIANGLE_DTYPE).view(np.uint8).reshape(-1)).cuda()


def test_static_matches_allocating_entry_point_on_consecutive_calls(cuda):
    small = scenes.plain_256()                  # 21,248 triangles at level 8
    room = scenes.room_1024()                   # 262,144 triangles at level 10: exactly the maximum
    assert len(room.tris) == STATIC_MAX_TRIS
    cases = [(small.tris, small.level), (room.tris, room.level), (small.tris, small.level)]
    first = None
    for tris, level in cases:
        dev = _upload(tris)
        want = _fragments_allocating(dev, len(tris), level)
        produced, got = _fragments_static(dev, len(tris), level, len(want))
        assert produced == len(want)
        assert np.array_equal(got, want)
        if first is None:
            first = got
    assert np.array_equal(got, first)  # the third call (same input as the first) repeats it exactly


def test_static_reports_required_count_when_buffer_is_short(cuda):
    s = scenes.plain_256()
    dev = _upload(s.tris)
    want = _fragments_allocating(dev, len(s.tris), s.level)
    produced, got = _fragments_static(dev, len(s.tris), s.level, len(want) // 2)
    assert produced == len(want)  # the count of a full run, so the caller can size its buffer


def test_allocation_counter_sees_the_allocating_entry_point(cuda):
    """The counter the other tests rely on moves when the library does allocate."""
    from sparsevoxeloctree_gb300 import _lib
    lib = _lib.load()
    s = scenes.plain_256()
    dev = _upload(s.tris)
    before = lib.svo_allocation_calls()
    _fragments_allocating(dev, len(s.tris), s.level)
    assert lib.svo_allocation_calls() > before


def test_static_reports_unit_overflow_without_writing_past_its_scratch(cuda):
    """32 full-size square planes (64 triangles) at level 12: a raster unit is one row piece of at most
    256 pixels of a triangle's bounding box, 4,096 rows x 16 pieces = 65,536 units per triangle, 4.2 million
    in all, beyond the roughly 1.29 million the fixed scratch holds beside 64 triangles.  The count pass reports it in
    count_dev[1]; the unit scan and unit emission skip their work, so no unit array is written past its
    end; the small-triangle fragments (none here) are still counted."""
    import torch

    from sparsevoxeloctree_gb300 import _lib
    lib = _lib.load()
    planes = 32
    tris = np.zeros(2 * planes, TRIANGLE_DTYPE)
    for k in range(planes):
        z = (k + 0.5) / planes
        tris["v"][2 * k] = [0.0, 0.0, z, 0.999, 0.0, z, 0.0, 0.999, z]
        tris["v"][2 * k + 1] = [0.999, 0.0, z, 0.999, 0.999, z, 0.0, 0.999, z]
    dev = _upload(tris)
    out = torch.zeros(16, dtype=torch.int64, device=dev.device)
    count = torch.full((2,), -1, dtype=torch.int64, device=dev.device)
    allocs = lib.svo_allocation_calls()
    rc = lib.svo_voxelize_static(ctypes.c_void_p(dev.data_ptr()), len(tris), 12, ctypes.c_void_p(out.data_ptr()), 16,
                                 ctypes.c_void_p(count.data_ptr()), None)
    assert rc == _lib.SVO_OK, lib.svo_last_error()
    assert lib.svo_allocation_calls() == allocs
    torch.cuda.synchronize()
    produced, status = (int(v) for v in count.cpu())
    assert status != 0          # the units did not fit: svo_voxelize must be used for this mesh
    assert produced == 0        # only small-triangle fragments are counted, and every triangle is large
    assert not out.any()        # nothing was emitted
    # the next call on the same scratch is unaffected
    s = scenes.plain_256()
    dev2 = _upload(s.tris)
    want = _fragments_allocating(dev2, len(s.tris), s.level)
    produced2, got = _fragments_static(dev2, len(s.tris), s.level, len(want))
    assert produced2 == len(want) and np.array_equal(got, want)


def test_static_rejects_more_triangles_than_its_scratch_holds(cuda):
    from sparsevoxeloctree_gb300 import _lib
    lib = _lib.load()
    g = np.random.default_rng(0)
    tris = np.zeros(STATIC_MAX_TRIS + 1, TRIANGLE_DTYPE)
    tris["v"] = g.uniform(0, 1, size=(len(tris), 9)).astype(np.float32)
    dev = _upload(tris)
    import torch
    out = torch.empty(16, dtype=torch.int64, device=dev.device)
    count = torch.zeros(2, dtype=torch.int64, device=dev.device)
    before = lib.svo_kernel_launches()
    allocs = lib.svo_allocation_calls()
    rc = lib.svo_voxelize_static(ctypes.c_void_p(dev.data_ptr()), len(tris), 6, ctypes.c_void_p(out.data_ptr()), 16,
                                 ctypes.c_void_p(count.data_ptr()), None)
    assert rc == _lib.SVO_ERR_CAPACITY
    assert b"262144" in lib.svo_last_error()
    assert lib.svo_allocation_calls() == allocs
    assert lib.svo_kernel_launches() == before
