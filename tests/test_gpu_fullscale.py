"""The benchmark workloads at their full sizes, engine against the oracle, through the C ABI.

The other parity tests run small scenes; these run the scenes the benchmark times, where the paths that
only large inputs take are exercised: segmented look-back scans over thousands of tiles, voxels crowded
past the packed colour accumulator (the exact 64-bit redo), 32^3-voxel buckets and sparse depths above
level 10, and millions of rays.

Bar (as everywhere): the fragment multiset and the node pool bit-exact, every ray's hit equal in every
field.  Fragment lists are compared as sorted int64 arrays on the device (sorting by the signed value is
a total order, so equal sorted arrays mean equal multisets); pools word for word.
"""
import numpy as np
import pytest

import oracle
from sparsevoxeloctree_gb300 import scenes
from sparsevoxeloctree_gb300.formats import HIT_DTYPE

pytestmark = pytest.mark.gpu


def _api():
    from sparsevoxeloctree_gb300 import api
    return api


def assert_same_multiset(frags_dev, ref):
    import torch
    r = torch.from_numpy(np.ascontiguousarray(ref).view(np.int64)).to(frags_dev.device)
    f = frags_dev.view(torch.int64)
    assert f.numel() == r.numel(), f"{f.numel()} fragments vs the oracle's {r.numel()}"
    assert torch.equal(torch.sort(f)[0], torch.sort(r)[0]), "fragment multisets differ"


def assert_same_pool(words_dev, ref):
    import torch
    r = torch.from_numpy(np.ascontiguousarray(ref).view(np.int32)).to(words_dev.device)
    assert words_dev.numel() == r.numel(), f"range {words_dev.numel()} vs the oracle's {r.numel()}"
    if not torch.equal(words_dev.view(torch.int32), r):
        bad = torch.nonzero(words_dev.view(torch.int32) != r)[:5].flatten().tolist()
        raise AssertionError(f"node words differ, first at {bad}")


def assert_hits_equal(got, want, what):
    assert len(got) == len(want)
    for f in HIT_DTYPE.names:
        same = (got[f] == want[f]).reshape(len(want), -1).all(axis=1)
        if not same.all():
            bad = np.nonzero(~same)[0]
            raise AssertionError(f"{what}: field {f} differs on {len(bad)} of {len(want)} rays, first {bad[:5]}")


def pipeline(tris, level, camera, width, height, bounce_seed=None):
    """voxelize -> build -> camera march (-> one diffuse bounce per hit) on the engine."""
    import torch
    api = _api()
    vox = api.Voxelizer.Create(api.to_device(tris), level)
    frags = vox.GetVoxelFragmentList()
    octree = api.Octree.FromFragments(frags, level)
    tracer = api.OctreeTracer.Create(octree, camera, width, height)
    hits = tracer.CmdDrawPipeline()
    bounce = None
    if bounce_seed is not None:
        bounce = tracer.Trace(api.OctreeTracer.Bounce(hits, bounce_seed))
    torch.cuda.synchronize()
    return frags, octree, api.hits_numpy(hits), (api.hits_numpy(bounce) if bounce is not None else None)


def test_room_1024_full_workload(cuda):
    """The benchmark's headline workload: 262,144 triangles at level 10 (38.4 M fragments, 87.1 M node
    words, walls of 1024^2 voxels crowding every leaf), 1920 x 1080 primary rays."""
    s = scenes.room_1024()
    frags, octree, hits, _ = pipeline(s.tris, s.level, s.camera, s.width, s.height)
    ref_frags = oracle.voxelize(s.tris, s.level)
    assert_same_multiset(frags, ref_frags)
    ref_pool = oracle.build_octree(ref_frags, s.level)
    del ref_frags
    assert_same_pool(octree.words(), ref_pool)
    ref_hits = oracle.raycast(ref_pool, s.level, oracle.camera_rays(s.camera, s.width, s.height))
    assert_hits_equal(hits, ref_hits, "room_1024 primary rays")
    assert (hits["flags"] & 1).mean() > 0.99  # an interior camera: nearly every ray hits a wall


def test_clusters_4096_4m_full_workload(cuda):
    """The 2^12 workload at the pointer format's limit: 4 M clustered triangles (145.7 M fragments,
    870 M node words; sparse depths 10 and 11, 32^3-voxel buckets), 3840 x 2160 primary rays plus one
    cosine-weighted diffuse bounce per hit."""
    s = scenes.clusters_4096(n_tris=4_000_000)
    frags, octree, hits, bounce = pipeline(s.tris, s.level, s.camera, s.width, s.height, bounce_seed=s.seed)
    ref_frags = oracle.voxelize(s.tris, s.level)
    assert_same_multiset(frags, ref_frags)
    del frags
    ref_pool = oracle.build_octree(ref_frags, s.level)
    del ref_frags
    assert_same_pool(octree.words(), ref_pool)
    ref_hits = oracle.raycast(ref_pool, s.level, oracle.camera_rays(s.camera, s.width, s.height))
    assert_hits_equal(hits, ref_hits, "clusters primary rays")
    ref_bounce = oracle.raycast(ref_pool, s.level, oracle.bounce_rays(ref_hits, s.seed))
    assert_hits_equal(bounce, ref_bounce, "clusters bounce rays")


def test_serving_level11_scene_through_the_server(cuda):
    """The largest level-11 scene of the serving workload (sphere + boxes + clutter), built by the
    server and traced by one 1 M-ray request (half camera rays, half their diffuse bounces), against the
    oracle's build and march of the same scene."""
    import torch
    api = _api()
    meshes = scenes.serving_scenes()
    tris, level = max((m for m in meshes if m[1] == 11), key=lambda m: len(m[0]))
    server = api.Server(lanes=2)
    try:
        sid = server.BuildScene(api.to_device(tris), level)
        words = server.Scene(sid).words()
        ref_frags = oracle.voxelize(tris, level)
        ref_pool = oracle.build_octree(ref_frags, level)
        del ref_frags
        assert_same_pool(words, ref_pool)
        w, h = 1024, 512
        n = w * h
        cam = scenes.camera_from_angles((1.35, 1.6, 1.2), 0.7, -0.2, aspect=w / h)
        buf = torch.empty(2 * n * HIT_DTYPE.itemsize, dtype=torch.uint8).pin_memory()
        t = server.SubmitCamera(sid, cam, w, h, n, 1234, buf)
        res = server.Wait(t)
        assert res["status"] == 0
        got = buf.numpy().view(HIT_DTYPE)
        ref_prim = oracle.raycast(ref_pool, level, oracle.camera_rays(cam, w, h))
        assert_hits_equal(got[:n], ref_prim, "served camera rays")
        ref_sec = oracle.raycast(ref_pool, level, oracle.bounce_rays(ref_prim, 1234))
        assert_hits_equal(got[n:], ref_sec, "served bounce rays")
    finally:
        server.close()
