"""The serving loop (svo_server) against the single-request path, through the C ABI.

Bar: every request's hits are bit-identical whether it ran alone, in a mix of concurrent requests of
other sizes and scenes (shared launches, several lanes in flight), or through svo_raycast_camera +
svo_bounce_rays + svo_raycast directly; requests after a rebuild see the new octree; requests that
cannot fit the HBM budget fail with SVO_ERR_CAPACITY instead of waiting forever.
"""
import math

import numpy as np
import pytest

from sparsevoxeloctree_gb300 import scenes
from sparsevoxeloctree_gb300.formats import HIT_DTYPE, RAY_DTYPE, TRIANGLE_DTYPE, rays_from_arrays

pytestmark = pytest.mark.gpu


def _api():
    from sparsevoxeloctree_gb300 import api
    return api


def small_scene(seed, n_clutter, level):
    sphere = scenes.icosphere(3, 0.3, (0.5, 0.5, 0.5))
    verts = np.concatenate([sphere, scenes.boxes(scenes.rng(seed, 1), 16),
                            scenes.clutter(scenes.rng(seed, 2), n_clutter, math.log(0.01), 0.7)], 0)
    return scenes._soup(verts, scenes.random_colors(scenes.rng(seed, 3), len(verts))), level


def pinned(nbytes):
    import torch
    return torch.empty(max(nbytes, 1), dtype=torch.uint8).pin_memory()


def direct_camera(octree, cam, width, height, n, seed):
    """The single-request path: full camera image, first n pixels, their bounce rays traced."""
    import torch
    api = _api()
    t = api.OctreeTracer.Create(octree, cam, width, height)
    prim = t.CmdDrawPipeline()[: n * HIT_DTYPE.itemsize].clone()
    rays = api.OctreeTracer.Bounce(prim, seed)
    sec = api.OctreeTracer.Create(octree).Trace(rays)
    torch.cuda.synchronize()
    return np.concatenate([api.hits_numpy(prim), api.hits_numpy(sec)])


def requests(n_scenes, count, seed=0):
    g = np.random.default_rng(seed)
    out = []
    for i in range(count):
        w = int(g.integers(8, 300))
        h = int(g.integers(8, 200))
        n = int(g.integers(1, w * h + 1))
        cam = scenes.camera_from_angles((float(g.uniform(1.2, 1.8)), float(g.uniform(1.2, 1.8)), 0.4),
                                        float(g.uniform(-0.4, 0.4)), float(g.uniform(-0.3, 0.3)), aspect=w / h)
        out.append({"scene": int(g.integers(0, n_scenes)), "cam": cam, "w": w, "h": h, "n": n,
                    "seed": int(g.integers(0, 2**62))})
    return out


def submit(server, req):
    buf = pinned(2 * req["n"] * HIT_DTYPE.itemsize)
    t = server.SubmitCamera(req["scene"], req["cam"], req["w"], req["h"], req["n"], req["seed"], buf)
    return t, buf


def hits_of(buf, n):
    return buf.numpy()[: n * HIT_DTYPE.itemsize].view(HIT_DTYPE).copy()


@pytest.fixture(scope="module")
def built(cuda):
    api = _api()
    server = api.Server(lanes=3)
    ids, octrees = [], []
    for k, (tris, level) in enumerate([small_scene(1, 3000, 6), small_scene(2, 6000, 8), small_scene(3, 9000, 9)]):
        ids.append(server.BuildScene(tris, level))
        octrees.append(server.Scene(ids[-1]))
    yield server, ids, octrees
    server.close()


def test_alone_equals_mix_equals_direct(built):
    server, ids, octrees = built
    reqs = requests(len(ids), 24, seed=5)
    alone = []
    for r in reqs:
        t, buf = submit(server, r)
        res = server.Wait(t)
        assert res["status"] == 0 and res["batch_requests"] == 1
        alone.append(hits_of(buf, 2 * r["n"]))
    # all at once: shared launches on several lanes
    sub = [submit(server, r) for r in reqs]
    mix = []
    batch_sizes = []
    for (t, buf), r in zip(sub, reqs):
        res = server.Wait(t)
        batch_sizes.append(res["batch_requests"])
        assert res["done_us"] >= res["launch_us"] >= res["submit_us"]
        mix.append(hits_of(buf, 2 * r["n"]))
    assert max(batch_sizes) > 1, "no request shared a launch"
    for i, r in enumerate(reqs):
        assert np.array_equal(alone[i], mix[i]), f"request {i}: alone and in the mix differ"
        ref = direct_camera(octrees[r["scene"]], r["cam"], r["w"], r["h"], r["n"], r["seed"])
        assert np.array_equal(alone[i], ref), f"request {i}: differs from the single-request path"


def pageable(nbytes):
    import torch
    return torch.empty(max(nbytes, 1), dtype=torch.uint8)


def test_pageable_and_mapped_buffers_agree(built):
    """Pinned (mapped) host buffers receive the bounce hits from the march in place; pageable ones get
    every hit through the lane's arena and copies.  A mix of both, in shared launches, gives the
    single-request hits."""
    server, ids, octrees = built
    reqs = requests(len(ids), 12, seed=11)
    sub = []
    for k, r in enumerate(reqs):
        buf = (pinned if k % 2 else pageable)(2 * r["n"] * HIT_DTYPE.itemsize)
        sub.append((server.SubmitCamera(r["scene"], r["cam"], r["w"], r["h"], r["n"], r["seed"], buf), buf))
    for (t, buf), r in zip(sub, reqs):
        assert server.Wait(t)["status"] == 0
        ref = direct_camera(octrees[r["scene"]], r["cam"], r["w"], r["h"], r["n"], r["seed"])
        assert np.array_equal(hits_of(buf, 2 * r["n"]), ref)


@pytest.mark.parametrize("alloc", ["pinned", "pageable", "pinned_offset"])
def test_ray_requests_match_svo_raycast(built, alloc):
    """pinned_offset: mapped buffers whose rays start 8 bytes in and hits 16 bytes in (still aligned
    for the march's stores) or 4 bytes in (unaligned: copied instead)."""
    import torch
    api = _api()
    server, ids, octrees = built
    g = np.random.default_rng(9)
    tickets = []
    for k in range(6):
        o, d = scenes.random_rays(g, int(g.integers(1, 5000)), inside=bool(k % 2))
        rays = rays_from_arrays(o, d)
        if alloc == "pageable":
            rh, hh = pageable(rays.nbytes), pageable(len(rays) * HIT_DTYPE.itemsize)
        elif alloc == "pinned":
            rh, hh = pinned(rays.nbytes), pinned(len(rays) * HIT_DTYPE.itemsize)
        else:
            hit_off = 16 if k % 2 else 4
            rh = pinned(rays.nbytes + 8)[8:]
            hh = pinned(len(rays) * HIT_DTYPE.itemsize + hit_off)[hit_off:]
        rh.numpy()[:] = rays.view(np.uint8)
        sc = k % len(ids)
        tickets.append((server.SubmitRays(sc, rh, hh), hh, rays, sc))
    for t, hh, rays, sc in tickets:
        server.Wait(t)
        got = hits_of(hh, len(rays))
        ref = api.hits_numpy(api.OctreeTracer.Create(octrees[sc]).Trace(api.to_device(rays)))
        torch.cuda.synchronize()
        assert np.array_equal(got, ref)


def test_rebuild_swaps_octree_while_tracing(built):
    import torch
    api = _api()
    server, ids, octrees = built
    reqs = [r for r in requests(len(ids), 12, seed=21)]
    for r in reqs:
        r["scene"] = 0
    before = [submit(server, r) for r in reqs[:6]]
    tris, level = small_scene(7, 5000, 7)
    tris_dev = api.to_device(tris)
    rb = server.SubmitRebuild(0, tris_dev, level)
    mid = [submit(server, r) for r in reqs[6:]]
    server.Wait(rb)
    after = [submit(server, r) for r in reqs[:4]]
    for t, _ in before + mid:
        assert server.Wait(t)["status"] == 0
    new = server.Scene(0)
    assert new.GetLevel() == level
    v = api.Voxelizer.Create(tris, level)
    direct_oct = api.Octree.FromFragments(v.GetVoxelFragmentList(), level)
    assert np.array_equal(new.words().cpu().numpy(), direct_oct.words().cpu().numpy())
    for (t, buf), r in zip(after, reqs[:4]):
        server.Wait(t)
        ref = direct_camera(direct_oct, r["cam"], r["w"], r["h"], r["n"], r["seed"])
        assert np.array_equal(hits_of(buf, 2 * r["n"]), ref)
    torch.cuda.synchronize()


def test_budget_admission(cuda):
    api = _api()
    tris, level = small_scene(4, 2000, 7)
    server = api.Server(hbm_budget_bytes=1 << 20, lanes=2)  # 1 MiB: the octree plus small requests
    try:
        sid = server.BuildScene(tris, level)
        st = server.stats()
        assert 0 < st["resident_bytes"] < (1 << 20)
        room = (1 << 20) - st["resident_bytes"]
        cam = scenes.camera_from_angles((1.5, 1.5, 0.4), 0.0, 0.0)
        big = (room // 88) + 64  # 88 device bytes per primary pixel (2 hits + 1 ray)
        t, _ = submit(server, {"scene": sid, "cam": cam, "w": 4096, "h": 4096, "n": big, "seed": 1})
        from sparsevoxeloctree_gb300 import _lib
        with pytest.raises(_lib.SvoError) as e:
            server.Wait(t)
        assert e.value.code == _lib.SVO_ERR_CAPACITY
        small = max(1, room // 88 // 4)
        ts = [submit(server, {"scene": sid, "cam": cam, "w": 512, "h": 512, "n": small, "seed": k}) for k in range(6)]
        for t, _ in ts:
            assert server.Wait(t)["status"] == 0
        st = server.stats()
        assert st["failed"] == 1 and st["inflight_bytes"] == 0
    finally:
        server.close()


def test_malformed_scene_fails_only_its_own_requests(cuda):
    """A scene added from a damaged pool (pointers past its range) shares launches with a healthy one:
    the requests that trace the damaged scene fail with SVO_ERR_INVALID, the co-batched requests on the
    healthy scene complete with the single-request path's hits."""
    import torch

    from sparsevoxeloctree_gb300 import _lib
    api = _api()
    server = api.Server(lanes=1)
    try:
        tris, level = small_scene(6, 3000, 7)
        good = server.BuildScene(tris, level)
        good_oct = server.Scene(good)
        bad_oct = api.Octree()
        bad_oct.m_buffer = torch.from_numpy(np.array([0x80000000 | 0x0FFF0000] * 8, np.uint32).view(np.int32)).cuda()
        bad_oct.m_range = 32
        bad_oct.m_level = 3
        bad = server.AddOctree(bad_oct)
        reqs = requests(2, 16, seed=31)
        for k, r in enumerate(reqs):
            r["scene"] = bad if k % 4 == 1 else good
        sub = [submit(server, r) for r in reqs]
        shared = False
        for (t, buf), r in zip(sub, reqs):
            if r["scene"] == bad:
                with pytest.raises(_lib.SvoError) as e:
                    server.Wait(t)
                assert e.value.code == _lib.SVO_ERR_INVALID
            else:
                res = server.Wait(t)
                assert res["status"] == 0
                shared |= res["batch_requests"] > 1
                ref = direct_camera(good_oct, r["cam"], r["w"], r["h"], r["n"], r["seed"])
                assert np.array_equal(hits_of(buf, 2 * r["n"]), ref)
        assert shared, "no healthy request shared a launch"
        assert server.stats()["failed"] == 4
    finally:
        server.close()
