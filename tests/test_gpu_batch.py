"""Batched voxelize + build (svo_batcher) against the single-mesh path and the oracle, through the C ABI.

Bar: per mesh, the batch's fragment list equals svo_voxelize of that mesh alone element for element
(same order), and its octree equals svo_build of those fragments word for word; both were checked
against the oracle by the single-mesh tests, and small meshes are checked against the oracle here too.
"""
import math

import numpy as np
import pytest

import oracle
from sparsevoxeloctree_gb300 import scenes
from sparsevoxeloctree_gb300.formats import TRIANGLE_DTYPE

pytestmark = pytest.mark.gpu


def _api():
    from sparsevoxeloctree_gb300 import api
    return api


def plain(tris, level):
    import torch
    api = _api()
    v = api.Voxelizer.Create(np.asarray(tris, TRIANGLE_DTYPE), level)
    frags = v.GetVoxelFragmentList()
    words = api.Octree.FromFragments(frags, level).words() if frags.numel() else None
    f = frags.cpu().numpy().view(np.uint64)
    if words is None:  # an empty mesh: the root block alone
        return f, np.zeros(8, np.uint32)
    torch.cuda.synchronize()
    return f, words.cpu().numpy().view(np.uint32)


def batch_results(bb, n):
    out = []
    for i in range(n):
        f = bb.GetVoxelFragmentList(i).cpu().numpy().view(np.uint64)
        w = bb.GetOctree(i).words().cpu().numpy().view(np.uint32)
        out.append((f, w))
    return out


def mixed_meshes(seed=7):
    g = scenes.rng(seed, 0)
    meshes = []
    sphere = scenes.icosphere(3, 0.3, (0.5, 0.5, 0.5))
    levels = [1, 2, 3, 5, 7, 8, 9, 10, 11, 12, 6, 10]
    for i, level in enumerate(levels):
        n = int(g.integers(50, 4000))
        verts = scenes.clutter(scenes.rng(seed, 1, i), n, math.log(0.02), 0.8)
        if i % 3 == 0:
            verts = np.concatenate([sphere, verts], 0)
        meshes.append((scenes._soup(verts, scenes.random_colors(scenes.rng(seed, 2, i), len(verts))), level))
    # an empty mesh and one of degenerate triangles (no fragments) in the middle of the batch
    meshes.insert(4, (np.zeros(0, TRIANGLE_DTYPE), 6))
    degenerate = np.zeros(5, TRIANGLE_DTYPE)
    degenerate["v"] = np.tile(np.float32([0.3, 0.3, 0.3]), 3)
    meshes.insert(7, (degenerate, 9))
    return meshes


def check_against_plain(meshes, got):
    for i, ((tris, level), (f, w)) in enumerate(zip(meshes, got)):
        pf, pw = plain(tris, level)
        assert np.array_equal(f, pf), f"mesh {i} (level {level}): fragment lists differ"
        assert np.array_equal(w, pw), f"mesh {i} (level {level}): octrees differ"


def test_batch_mixed_levels_match_single_builds(cuda):
    meshes = mixed_meshes()
    bb = _api().BatchBuilder()
    bb.Build(meshes)
    assert len(bb) == len(meshes)
    got = batch_results(bb, len(meshes))
    check_against_plain(meshes, got)
    # small meshes also against the oracle (canonical fragment order for the multiset)
    for i in (0, 1, 2, 5):
        tris, level = meshes[i]
        ref_f = oracle.voxelize(tris, level)
        assert np.array_equal(np.sort(got[i][0]), np.sort(ref_f))
        assert np.array_equal(got[i][1], oracle.build_octree(ref_f, level))
    info = bb.GetInfo(9)
    assert info["range_words"] == len(got[9][1])


def test_batch_graph_replay_and_shape_change(cuda):
    api = _api()
    meshes = mixed_meshes(11)[:8]
    bb = api.BatchBuilder(use_graph=True)
    bb.Build(meshes)
    first = batch_results(bb, len(meshes))
    bb.Build(meshes)  # same shape: the recorded graphs are replayed
    st = bb.stats()
    assert st["graph_replays"] >= 2, st
    second = batch_results(bb, len(meshes))
    for (f1, w1), (f2, w2) in zip(first, second):
        assert np.array_equal(f1, f2) and np.array_equal(w1, w2)
    # a different batch on the same batcher: re-recorded, still exact
    other = mixed_meshes(12)[3:10]
    bb.Build(other)
    check_against_plain(other, batch_results(bb, len(other)))
    # without graphs: same results
    nb = api.BatchBuilder(use_graph=False)
    nb.Build(meshes)
    for (f1, w1), (f2, w2) in zip(first, batch_results(nb, len(meshes))):
        assert np.array_equal(f1, f2) and np.array_equal(w1, w2)


def test_batch_clutter_workload_matches_single_builds(cuda):
    """The batched-build workload's mesh generator (clutter meshes, levels 7..10), scaled down."""
    meshes = scenes.batch_64(seed=3, n_meshes=12, t_lo=1e3, t_hi=3e4)
    bb = _api().BatchBuilder()
    bb.Build(meshes)
    check_against_plain(meshes, batch_results(bb, len(meshes)))


def test_batch_traced_octree_matches_single(cuda):
    """An octree from the batch's shared pool traces like the single build's octree."""
    api = _api()
    meshes = mixed_meshes(5)[6:10]
    bb = api.BatchBuilder()
    bb.Build(meshes)
    g = np.random.default_rng(3)
    o, d = scenes.random_rays(g, 4096)
    from sparsevoxeloctree_gb300.formats import rays_from_arrays
    rays = api.to_device(rays_from_arrays(o, d))
    for i, (tris, level) in enumerate(meshes):
        oct_b = bb.GetOctree(i)
        h_b = api.hits_numpy(api.OctreeTracer.Create(oct_b).Trace(rays))
        v = api.Voxelizer.Create(np.asarray(tris, TRIANGLE_DTYPE), level)
        if v.GetVoxelFragmentCount() == 0:
            continue
        oct_p = api.Octree.FromFragments(v.GetVoxelFragmentList(), level)
        h_p = api.hits_numpy(api.OctreeTracer.Create(oct_p).Trace(rays))
        assert np.array_equal(h_b, h_p)
