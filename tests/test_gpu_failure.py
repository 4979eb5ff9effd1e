"""Failure paths of the bounded device waits, driven on the GPU without a fault.

The engine's single-pass scans (voxelize count, dense bitmap scan, bucket scan, sparse alloc) and the
fused beam march wait on values other warps publish; every wait is bounded and, when it gives up, sets
a status bit instead of trapping.  A correct run never reaches the bound, so these tests use the
library's test hook (svo_debug_wait_fault): it lowers the bound and withholds one scan tile or beam
texel, which then never publishes, so the waits on it run out.  Each test checks the reported status,
that nothing was written through the incomplete scan's offsets, and that the next call (hook cleared)
is correct again, i.e. the context stayed usable.  The reference has no such path: it logs an overflow
after the fact (src/Octree.cpp:30-33) and its shaders wait on nothing.
"""
import ctypes

import numpy as np
import pytest

import oracle
from sparsevoxeloctree_gb300 import scenes
from sparsevoxeloctree_gb300.formats import TRIANGLE_DTYPE

pytestmark = pytest.mark.gpu

SPIN_LIMIT = 2048  # iterations a wait takes before it gives up (each with a short sleep)


@pytest.fixture
def wait_fault(cuda):
    """Arms the hook for one tile/texel index; always disarmed again after the test."""
    from sparsevoxeloctree_gb300 import _lib
    lib = _lib.load()

    def arm(withheld):
        _lib.check(lib.svo_debug_wait_fault(SPIN_LIMIT, withheld))

    yield arm
    _lib.check(lib.svo_debug_wait_fault(0, 0))


def _upload_tris(tris):
    import torch
    return torch.from_numpy(np.ascontiguousarray(tris, TRIANGLE_DTYPE).view(np.uint8).reshape(-1)).cuda()


def test_voxelize_count_scan_timeout_is_reported(cuda, wait_fault):
    """Count pass: 21,248 triangles are 42 scan tiles of 512; tile 1 withheld, tiles after it give up."""
    from sparsevoxeloctree_gb300 import _lib
    lib = _lib.load()
    s = scenes.plain_256()
    dev = _upload_tris(s.tris)
    fl = _lib.Fraglist()
    allocs = lib.svo_allocation_calls()
    wait_fault(1)
    rc = lib.svo_voxelize(ctypes.c_void_p(dev.data_ptr()), len(s.tris), s.level, ctypes.byref(fl), None)
    assert rc == _lib.SVO_ERR_TIMEOUT, lib.svo_last_error()
    assert b"wait gave up" in lib.svo_last_error()
    assert fl.count == 0 and not fl.data  # no fragment list was handed out
    assert lib.svo_allocation_calls() > allocs  # (the count pass did allocate its workspace, and freed it)
    _lib.check(lib.svo_debug_wait_fault(0, 0))
    from sparsevoxeloctree_gb300 import api
    got = api.Voxelizer.Create(dev, s.level).GetVoxelFragmentList().cpu().numpy().view(np.uint64)
    assert np.array_equal(np.sort(got), np.sort(oracle.voxelize(s.tris, s.level)))


def test_build_scan_timeout_writes_nothing_through_its_offsets(cuda, wait_fault):
    """Build at level 8: tile 0 of every scan never publishes, so the look-backs of the tiles after it
    (the dense bitmap scan's ten 8192-word tiles, the bucket scan's two 2048-bucket tiles) give up.  The
    status word reports the timeout, and the caller's pool is left exactly as it was: the interior-word,
    sparse and leaf stages all skip once a scan is incomplete."""
    import torch

    from sparsevoxeloctree_gb300 import _lib, api
    lib = _lib.load()
    s = scenes.plain_256()
    frags = oracle.voxelize(s.tris, s.level)
    ft = torch.from_numpy(frags.view(np.int64)).cuda()
    b = api.OctreeBuilder.Create(fragments=ft, level=s.level)
    sentinel = np.int32(np.uint32(0xA5A5A5A5).view(np.int32))
    b.m_octree_buffer.fill_(int(sentinel))
    wait_fault(0)
    b.CmdBuild()
    torch.cuda.synchronize()
    status = int(b.m_result.cpu().numpy().view(np.uint32)[-1])
    assert status & 1, f"status {status:#x}: the timeout bit is not set"
    with pytest.raises(_lib.SvoError) as e:
        b.GetInfo()
    assert e.value.code == _lib.SVO_ERR_TIMEOUT
    assert bool((b.m_octree_buffer == int(sentinel)).all()), "a stage wrote the pool after the scan gave up"
    _lib.check(lib.svo_debug_wait_fault(0, 0))
    b.CmdBuild()
    info = b.GetInfo()
    ref = oracle.build_octree(frags, s.level)
    assert info["range_words"] == len(ref)
    assert np.array_equal(b.m_octree_buffer[: len(ref)].cpu().numpy().view(np.uint32), ref)


def test_sparse_alloc_timeout_through_allocating_entry_point(cuda, wait_fault):
    """Three walls of the room shell at level 11 (12.6 M fragments, below the 2^24 from which depth 10 is
    kept dense): depths 1..9 are dense (a 586-tile bitmap scan), the bucket scan has 128 tiles, and the
    sparse alloc of depth 10 has about 768 tiles of 8192 words (8 per occupied depth-9 cell, ~786 k cells
    on the walls).  Tile 700 exists only in that alloc, so only its look-back gives up.  svo_build returns
    SVO_ERR_TIMEOUT and hands out no octree; the same call with the hook cleared gives the octree of a
    fault-free build, word for word."""
    import torch

    from sparsevoxeloctree_gb300 import _lib, api
    lib = _lib.load()
    level = 11
    tris = scenes._soup(scenes.room_shell(level)[:6], scenes.random_colors(scenes.rng(9), 6))
    ft = api.voxelize(api.to_device(tris), level)
    n = int(ft.numel())

    def build():
        oc = _lib.OctreeC()
        rc = lib.svo_build(ctypes.c_void_p(ft.data_ptr()), n, level, ctypes.byref(oc), None, None)
        return rc, oc

    def words(oc):
        got = np.empty(oc.range_words, np.uint32)
        _lib.check(lib.svo_download(ctypes.c_void_p(got.ctypes.data), ctypes.c_void_p(oc.words), got.nbytes, 1, None))
        lib.svo_octree_destroy(ctypes.byref(oc), None)
        return got

    rc, oc = build()
    assert rc == _lib.SVO_OK, lib.svo_last_error()
    want = words(oc)
    assert n < (1 << 24)  # the depth-10 words are built by the sparse alloc
    assert len(want) > 8 * 700 * 8192 // 8  # the depth-10 range spans more than 700 alloc tiles
    wait_fault(700)
    rc, oc = build()
    assert rc == _lib.SVO_ERR_TIMEOUT, lib.svo_last_error()
    assert not oc.words
    _lib.check(lib.svo_debug_wait_fault(0, 0))
    rc, oc = build()
    assert rc == _lib.SVO_OK, lib.svo_last_error()
    assert np.array_equal(words(oc), want)
    torch.cuda.synchronize()


def test_beam_texel_wait_timeout_marches_from_the_camera(cuda, wait_fault):
    """Fused beam march on a 64 x 64 image: beam texel 10 (column 1, row 1 of the 9 x 9 texel grid) never
    publishes.  The 8 x 4 ray tiles that need it (pixels x < 16, y < 16) give up waiting, march from the
    camera and carry SVO_HIT_FLAG_BEAM_WAIT: apart from that bit their hits are svo_raycast_camera's.
    Every other ray is exactly the fault-free fused march's."""
    from sparsevoxeloctree_gb300 import _lib, api
    s = scenes.plain_256()
    o = api.Octree.FromFragments(api.voxelize(s.tris, s.level), s.level)
    w = h = 64
    tracer = api.OctreeTracer.Create(o, s.camera, w, h)
    clean = api.hits_numpy(tracer.CmdDrawPipelineBeam(None))
    plain = api.hits_numpy(tracer.CmdDrawPipeline())
    wait_fault(10)
    faulted = api.hits_numpy(tracer.CmdDrawPipelineBeam(None))
    _lib.check(_lib.load().svo_debug_wait_fault(0, 0))
    flagged = (faulted["flags"] & 32) != 0
    yy, xx = np.divmod(np.arange(w * h), w)
    expect = (xx < 16) & (yy < 16)
    assert np.array_equal(flagged, expect)
    assert not ((clean["flags"] & 32) != 0).any() and not ((plain["flags"] & 32) != 0).any()
    unflagged = faulted.copy()
    unflagged["flags"] &= ~np.uint16(32)
    assert np.array_equal(unflagged[expect], plain[expect])
    assert np.array_equal(faulted[~expect], clean[~expect])
    again = api.hits_numpy(tracer.CmdDrawPipelineBeam(None))
    assert np.array_equal(again, clean)
