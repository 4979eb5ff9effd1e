"""CUDA engine vs the CPU oracle on the same seeded inputs, through the C ABI.

Bar: fragments (canonical order) and octrees bit-exact; ray hits bit-exact in every field (the march is
compiled without FMA contraction and follows the same float operations as the oracle), which is
stricter than the >= 99.99% voxel-id / |dt| <= 1e-5 tolerance the engine promises.
"""
import numpy as np
import pytest

import oracle
from sparsevoxeloctree_gb300 import scenes
from sparsevoxeloctree_gb300.formats import HIT_DTYPE, RAY_DTYPE, TRIANGLE_DTYPE, rays_from_arrays

pytestmark = pytest.mark.gpu

T_TOL = 1e-5  # |dt| bound, octree space (extent 1)


def _api():
    from sparsevoxeloctree_gb300 import api
    return api


def gpu_voxelize(tris, level):
    api = _api()
    v = api.Voxelizer.Create(np.asarray(tris, TRIANGLE_DTYPE), level)
    return v.GetVoxelFragmentList().cpu().numpy().view(np.uint64)


def gpu_build(frags, level):
    import torch
    api = _api()
    t = torch.from_numpy(np.ascontiguousarray(frags).view(np.int64)).cuda()
    o = api.Octree.FromFragments(t, level)
    return o, o.words().cpu().numpy().view(np.uint32)


def gpu_trace(octree, rays):
    api = _api()
    hits = api.OctreeTracer.Create(octree).Trace(api.to_device(np.asarray(rays, RAY_DTYPE)))
    return api.hits_numpy(hits)


def assert_same_fragments(got, ref):
    """Multiset equality of fragment lists (the engine's order is deterministic but differs from the
    oracle's triangle order: small triangles first, then large ones)."""
    assert len(got) == len(ref)
    assert np.array_equal(np.sort(got), np.sort(ref))


def assert_hits_equal(h_gpu, h_ref):
    for f in HIT_DTYPE.names:
        a, b = h_gpu[f], h_ref[f]
        if not np.array_equal(a, b):
            bad = np.nonzero((a != b).reshape(len(a), -1).any(axis=1))[0]
            raise AssertionError(f"hit field {f} differs on {len(bad)} rays, first {bad[:5]}: "
                                 f"{h_gpu[bad[:3]]} vs {h_ref[bad[:3]]}")


def single(v9, rgb=(0x112233, 0x445566, 0x778899)):
    t = np.zeros(1, TRIANGLE_DTYPE)
    t["v"] = np.asarray(v9, np.float32).reshape(1, 9)
    t["rgb"] = rgb
    return t


# ------------------------------------------------------------------------------------------- voxelize
def test_voxelize_plain_256_bit_exact(cuda):
    s = scenes.plain_256()
    ref = oracle.voxelize(s.tris, s.level)
    got = gpu_voxelize(s.tris, s.level)
    assert_same_fragments(got, ref)
    again = gpu_voxelize(s.tris, s.level)
    assert np.array_equal(again, got)  # run-to-run identical, order included


@pytest.mark.parametrize("level", [1, 2, 5, 8, 12])
def test_voxelize_random_triangles(cuda, level):
    g = np.random.default_rng(level)
    n = 3000
    c = g.uniform(0, 1, size=(n, 1, 3))
    size = np.exp(g.uniform(np.log(1e-4), np.log(0.7), size=(n, 1, 1)))
    verts = np.clip(c + g.normal(size=(n, 3, 3)) * size, -0.05, 1.05)
    tris = np.zeros(n, TRIANGLE_DTYPE)
    tris["v"] = verts.reshape(n, 9).astype(np.float32)
    tris["rgb"] = g.integers(0, 1 << 24, size=(n, 3))
    ref = oracle.voxelize(tris, level)
    got = gpu_voxelize(tris, level)
    assert_same_fragments(got, ref)


def test_voxelize_edge_cases(cuda):
    tris = np.concatenate([
        single([0.1, 0.1, 0.1, 0.1, 0.1, 0.1, 0.1, 0.1, 0.1]),          # a point: degenerate
        single([0.1, 0.1, 0.1, 0.5, 0.5, 0.5, 0.9, 0.9, 0.9]),          # collinear: degenerate
        single([0.0, 0.0, 0.5, 1.0, 0.0, 0.5, 0.0, 1.0, 0.5]),          # half the z = 0.5 plane
        single([0.0, 0.0, 0.0, 1.0, 1.0, 1.0, 1.0, 0.0, 0.0]),          # 45 degree diagonal
        single([np.nan, 0.2, 0.2, 0.3, np.inf, 0.2, 0.2, 0.3, -1.0]),  # non-finite / outside
        single([0.25, 0.25, 0.25, 0.75, 0.25, 0.25, 0.25, 0.75, 0.25]),  # on voxel boundaries
        single([0.5, 0.5, 0.5, 0.5 + 1e-7, 0.5, 0.5, 0.5, 0.5 + 1e-7, 0.5]),  # sub-voxel sliver
    ])
    for level in (1, 4, 10, 12):
        assert_same_fragments(gpu_voxelize(tris, level), oracle.voxelize(tris, level))


@pytest.mark.parametrize("level", [3, 7, 10, 12])
def test_voxelize_small_triangles_on_pixel_boundaries(cuda, level):
    """Small triangles (bounding boxes around the 256-pixel bound) whose vertices sit on pixel corners,
    pixel centres and sub-pixel steps, a third of them with an edge along an axis and many of them
    slivers or steep: the spans walked row by row with integer steps give the oracle's intervals
    exactly, on both sides of every edge."""
    g = np.random.default_rng(100 + level)
    R = 1 << level
    n = 6000
    base = g.integers(0, max(R - 17, 1), size=(n, 1, 3)).astype(np.float64)
    step = g.integers(0, 17, size=(n, 3, 3)).astype(np.float64)
    frac = g.choice([0.0, 0.5, 1 / 256, 255 / 256, 128 / 256], size=(n, 3, 3))
    pts = (base + step + frac) / R
    axis = g.integers(0, 3, size=n)
    for i in np.nonzero(np.arange(n) % 3 == 0)[0]:  # vertices 0 and 1 differ along one axis only
        others = [a for a in range(3) if a != axis[i]]
        pts[i, 1, others] = pts[i, 0, others]
    tris = np.zeros(n, TRIANGLE_DTYPE)
    tris["v"] = np.clip(pts, 0.0, 1.0).reshape(n, 9).astype(np.float32)
    tris["rgb"] = g.integers(0, 1 << 24, size=(n, 3))
    ref = oracle.voxelize(tris, level)
    assert len(ref) > n
    assert_same_fragments(gpu_voxelize(tris, level), ref)


def test_voxelize_repeated_mesh_with_changed_triangles(cuda):
    """svo_voxelize on the same triangle buffer again: the list is sized by the earlier count and the
    emission queued before the count is read back.  The buffer's triangles then change so that the
    count grows (the list is emitted again into an exact one) and then shrinks (the list keeps the
    larger capacity); every call returns exactly the oracle's fragments."""
    import ctypes

    import torch
    from sparsevoxeloctree_gb300 import _lib
    lib = _lib.load()
    s = scenes.plain_256()
    base = np.asarray(s.tris, TRIANGLE_DTYPE)
    bigger = base.copy()
    bigger["v"] = np.clip(0.5 + (bigger["v"] - 0.5) * 1.3, 0.0, 1.0)  # larger triangles: more fragments
    smaller = np.zeros(len(base), TRIANGLE_DTYPE)  # same triangle count: half of them, the rest degenerate
    smaller[: len(base) // 2] = base[: len(base) // 2]
    dev = torch.empty(base.nbytes, dtype=torch.uint8, device="cuda")
    counts, capacities = [], []
    for tris in (base, base, bigger, bigger, smaller):
        dev.copy_(torch.from_numpy(np.ascontiguousarray(tris).view(np.uint8).reshape(-1)))
        fl = _lib.Fraglist()
        _lib.check(lib.svo_voxelize(ctypes.c_void_p(dev.data_ptr()), len(tris), s.level, ctypes.byref(fl), None))
        got = np.empty(fl.count, np.uint64)
        if fl.count:
            _lib.check(lib.svo_download(ctypes.c_void_p(got.ctypes.data), ctypes.c_void_p(fl.data),
                                        fl.count * 8, 1, None))
        assert_same_fragments(got, oracle.voxelize(tris, s.level))
        counts.append(fl.count)
        capacities.append(fl.capacity)
        lib.svo_fraglist_destroy(ctypes.byref(fl), None)
    assert counts[2] > counts[1] and counts[4] < counts[3]
    assert capacities[4] >= counts[4] and all(c >= n for c, n in zip(capacities, counts))


def test_voxelize_empty(cuda):
    got = gpu_voxelize(np.zeros(0, TRIANGLE_DTYPE), 6)
    assert len(got) == 0


def test_voxelize_golden_vs_reference_shaders(cuda, golden_dir):
    """Reference geometry+fragment shaders (conservative variant, fixture) vs the engine: equal except
    fragments whose pixel-centre depth lies within float rounding of a voxel boundary (one voxel off)."""
    z = np.load(f"{golden_dir}/golden_vox.npz")
    tris = z["tris"].view(TRIANGLE_DTYPE)
    level = int(z["level"])
    got = gpu_voxelize(tris, level)
    assert_same_fragments(got, oracle.voxelize(tris, level))
    a, b = set(got.tolist()), set(z["frags"].tolist())
    assert len(a ^ b) <= 0.002 * len(b)


# ------------------------------------------------------------------------------------------- build
@pytest.mark.parametrize("level", [1, 2, 3, 6, 9])
def test_build_random_fragments(cuda, level):
    g = np.random.default_rng(100 + level)
    R = 1 << level
    n = 20000
    xyz = g.integers(0, R, size=(n, 3))
    if level > 3:  # cluster half of them so leaves merge many fragments (count saturates at 63)
        xyz[: n // 2] = g.integers(0, min(R, 4), size=(n // 2, 3))
    from sparsevoxeloctree_gb300.formats import pack_fragments
    frags = pack_fragments(xyz[:, 0], xyz[:, 1], xyz[:, 2], g.integers(0, 1 << 24, size=n))
    ref = oracle.build_octree(frags, level)
    _, got = gpu_build(frags, level)
    assert np.array_equal(got, ref)


def test_build_plain_256_bit_exact(cuda):
    s = scenes.plain_256()
    frags = oracle.voxelize(s.tris, s.level)
    ref, ref_nodes = oracle.build_octree(frags, s.level, return_level_nodes=True)
    o, got = gpu_build(frags, s.level)
    assert np.array_equal(got, ref)
    assert o.info["level_nodes"] == ref_nodes.tolist()


def test_build_golden_structure(cuda, golden_dir):
    """The reference's own tag/alloc shaders (fixture): same structure; leaf colours agree wherever the
    running mean and the integer mean coincide (one or two fragments per leaf)."""
    z = np.load(f"{golden_dir}/golden_build.npz")
    frags, level, ref_pool = z["frags"], int(z["level"]), z["pool"]
    _, got = gpu_build(frags, level)
    assert len(got) == len(ref_pool)
    assert np.array_equal(got & 0xC0000000, ref_pool & 0xC0000000)
    interior = (ref_pool & 0xC0000000) == 0x80000000
    assert np.array_equal(got[interior], ref_pool[interior])
    leaf = (ref_pool >> 30) == 3
    cnt = (ref_pool >> 24) & 0x3F
    small = leaf & (cnt <= 2)
    assert np.array_equal(got[small], ref_pool[small])
    assert np.array_equal((got[leaf] >> 24) & 0x3F, cnt[leaf])


def test_build_empty(cuda):
    _, got = gpu_build(np.zeros(0, np.uint64), 7)
    assert len(got) == 8 and not got.any()


# ------------------------------------------------------------------------------------------- march
def test_march_golden_vs_reference_shader(cuda, golden_dir):
    zb = np.load(f"{golden_dir}/golden_build.npz")
    zm = np.load(f"{golden_dir}/golden_march.npz")
    level, pool = int(zb["level"]), zb["pool"]
    import torch
    api = _api()
    o = api.Octree()
    o.m_buffer = torch.from_numpy(pool.view(np.int32)).cuda()
    o.m_range, o.m_level = len(pool) * 4, level
    rays = rays_from_arrays(zm["o"], zm["d"])
    h = gpu_trace(o, rays)
    assert np.array_equal(h, oracle.raycast(pool, level, rays))
    hit = (h["flags"] & 1).astype(np.uint32)
    assert np.array_equal(hit, zm["hit"])
    assert np.array_equal(h["iter"], zm["iter"])
    assert np.array_equal(h["pos"], zm["pos"])
    col = np.stack([(h["node"] >> (8 * k)) & 255 for k in range(3)], 1).astype(np.float32) / 255.0
    m = hit == 1
    assert np.array_equal(col[m], zm["color"][m])
    nrm = np.zeros((len(h), 3), np.float32)
    nrm[np.arange(len(h)), (h["flags"] >> 1) & 3] = np.where(h["flags"] & 8, -1.0, 1.0)
    assert np.array_equal(nrm, zm["normal"])


def test_march_camera_and_bounce_plain_256(cuda):
    s = scenes.plain_256()
    frags = oracle.voxelize(s.tris, s.level)
    pool = oracle.build_octree(frags, s.level)
    o, _ = gpu_build(frags, s.level)
    api = _api()
    tracer = api.OctreeTracer.Create(o, s.camera, s.width, s.height)
    h_gpu = api.hits_numpy(tracer.CmdDrawPipeline())
    rays = oracle.camera_rays(s.camera, s.width, s.height)
    h_ref = oracle.raycast(pool, s.level, rays)
    assert_hits_equal(h_gpu, h_ref)
    # one diffuse bounce per hit
    b_gpu = api.OctreeTracer.Bounce(api.to_device(h_gpu), seed=77)
    b_ref = oracle.bounce_rays(h_ref, 77)
    assert np.array_equal(api.from_device(b_gpu, RAY_DTYPE), b_ref)
    h2 = api.hits_numpy(tracer.Trace(b_gpu))
    assert_hits_equal(h2, oracle.raycast(pool, s.level, b_ref))


def test_march_random_rays_many_levels(cuda):
    g = np.random.default_rng(3)
    for level in (1, 3, 7, 10):
        R = 1 << level
        n = 30000
        from sparsevoxeloctree_gb300.formats import pack_fragments
        xyz = g.integers(0, R, size=(n, 3))
        frags = pack_fragments(xyz[:, 0], xyz[:, 1], xyz[:, 2], g.integers(0, 1 << 24, size=n))
        pool = oracle.build_octree(frags, level)
        o, _ = gpu_build(frags, level)
        o1, d1 = scenes.random_rays(g, 20000)
        o2, d2 = scenes.random_rays(g, 20000, inside=True)
        rays = rays_from_arrays(np.concatenate([o1, o2]), np.concatenate([d1, d2]))
        rays["d"][:6] = [[1, 0, 0], [0, 1, 0], [0, 0, -1], [0, 0, 0], [1e-30, 0, 1], [-1, 1e-20, 0]]
        assert_hits_equal(gpu_trace(o, rays), oracle.raycast(pool, level, rays))


def test_march_malformed_pools_are_flagged(cuda):
    """Pools no build produces: child pointers past the range, interior words at the leaf level, a
    cycle back to the root block.  Every read stays inside the range (checked before the load); such rays
    end as misses with the aborted flag, identically to the oracle; rays into valid leaves still hit."""
    import torch

    from sparsevoxeloctree_gb300.formats import HIT_FLAG_ABORTED, HIT_FLAG_HIT
    api = _api()
    leaf = 0xC1000000 | 0x123456
    far = 0x80000000 | 0x0FFF0000
    cases = [
        (3, [far] * 8),                                        # pointers past the range
        (2, [0x80000008] * 8 + [0x80000008] * 8),              # interior word at the leaf level
        (3, [0x80000000] * 8),                                 # cycle to the root block
        (2, [leaf, far, 0, 0x80000008, leaf, 0, far, 0x80000008] + [leaf, 0, 0, 0, 0, 0, 0, 0x80000000]),
    ]
    g = np.random.default_rng(17)
    o1, d1 = scenes.random_rays(g, 4000)
    o2, d2 = scenes.random_rays(g, 4000, inside=True)
    rays = rays_from_arrays(np.concatenate([o1, o2]), np.concatenate([d1, d2]))
    aborted_total = 0
    for level, words in cases:
        pool = np.array(words, np.uint32)
        o = api.Octree()
        o.m_buffer = torch.from_numpy(pool.view(np.int32)).cuda()
        o.m_range = 4 * len(pool)
        o.m_level = level
        got = gpu_trace(o, rays)
        assert_hits_equal(got, oracle.raycast(pool, level, rays))
        ab = (got["flags"] & HIT_FLAG_ABORTED) != 0
        assert not np.any(ab & ((got["flags"] & HIT_FLAG_HIT) != 0))
        aborted_total += int(ab.sum())
    assert aborted_total > 0


def test_camera_golden(cuda, golden_dir):
    """Primary-ray directions: oracle == reference Camera_GenRay (fixture); the GPU march over camera
    rays equals the march over the oracle's explicit rays."""
    z = np.load(f"{golden_dir}/golden_camera.npz")
    from sparsevoxeloctree_gb300.formats import CAMERA_DTYPE
    cam = z["cam"].view(CAMERA_DTYPE)[0]
    w, h = int(z["width"]), int(z["height"])
    rays = oracle.camera_rays(cam, w, h)
    assert np.array_equal(rays["d"], z["dirs"])
    s = scenes.plain_256()
    frags = oracle.voxelize(s.tris, s.level)
    o, pool = gpu_build(frags, s.level)
    api = _api()
    h_cam = api.hits_numpy(api.OctreeTracer.Create(o, cam, w, h).CmdDrawPipeline())
    assert_hits_equal(h_cam, oracle.raycast(pool, s.level, rays))


# ------------------------------------------------------------------------------------------- build edge paths
@pytest.mark.parametrize("level", [10, 11, 12])
def test_build_deep_levels(cuda, level):
    """Levels 11 and 12 go through the sparse tag/alloc path below the dense depth-9 bitmaps."""
    from sparsevoxeloctree_gb300.formats import pack_fragments
    g = np.random.default_rng(300 + level)
    R = 1 << level
    n = 40000
    xyz = g.integers(0, R, size=(n, 3))
    xyz[: n // 4] = (xyz[: n // 4] // 64) * 64 + g.integers(0, 3, size=(n // 4, 3))  # small dense clumps
    frags = pack_fragments(xyz[:, 0], xyz[:, 1], xyz[:, 2], g.integers(0, 1 << 24, size=n))
    ref, nodes = oracle.build_octree(frags, level, return_level_nodes=True)
    o, got = gpu_build(frags, level)
    assert np.array_equal(got, ref)
    assert o.info["level_nodes"] == nodes.tolist()


def _crowded_voxel_fragments(level, n_hot):
    from sparsevoxeloctree_gb300.formats import pack_fragments
    g = np.random.default_rng(7)
    R = 1 << level
    xyz = g.integers(0, R, size=(2000, 3))
    hot = np.tile([[R // 3, R // 2, R // 5]], (n_hot, 1))
    xyz = np.concatenate([xyz, hot])
    return pack_fragments(xyz[:, 0], xyz[:, 1], xyz[:, 2], g.integers(0, 1 << 24, size=len(xyz)))


@pytest.mark.parametrize("n_hot", [257, 258, 5000, 65536, 65576])
def test_build_many_fragments_in_one_voxel(cuda, n_hot):
    """More than 257 fragments in one voxel overflow the packed accumulator: the exact wide pass takes
    over (both through svo_build_ex and through the stream-ordered svo_build_into).  At 65,536 and
    65,576 fragments the voxel's count field wraps to a value below 258, so only the check that the count
    fields add up to the fragment count catches it."""
    import torch
    api = _api()
    level = 6
    frags = _crowded_voxel_fragments(level, n_hot)
    ref = oracle.build_octree(frags, level)
    o, got = gpu_build(frags, level)
    assert np.array_equal(got, ref)
    assert o.info["leaves"] == int(np.count_nonzero((ref & 0xC0000000) == 0xC0000000))
    t = torch.from_numpy(frags.view(np.int64)).cuda()
    b = api.OctreeBuilder.Create(fragments=t, level=level)
    b.GetOctree().fill_(-1)
    b.CmdBuild()
    assert b.GetOctreeRange() == 4 * len(ref)
    assert np.array_equal(b.GetOctree()[: len(ref)].cpu().numpy().view(np.uint32), ref)


def test_build_into_pool_too_small_reports_capacity(cuda):
    import torch
    from sparsevoxeloctree_gb300 import _lib
    api = _api()
    s = scenes.plain_256()
    frags = oracle.voxelize(s.tris, s.level)
    t = torch.from_numpy(frags.view(np.int64)).cuda()
    b = api.OctreeBuilder.Create(fragments=t, level=s.level, capacity=4096)
    b.CmdBuild()
    with pytest.raises(_lib.SvoError) as e:
        b.GetInfo()
    assert e.value.code == _lib.SVO_ERR_CAPACITY
    # the builder is still usable with a large enough pool
    b2 = api.OctreeBuilder.Create(fragments=t, level=s.level)
    b2.CmdBuild()
    b2.Reserve()  # pool shrunk to the exact range
    b2.GetOctree().fill_(-1)  # no stale words from the first build can pass the comparison
    b2.CmdBuild()
    ref = oracle.build_octree(frags, s.level)
    assert b2.GetInfo()["range_words"] == len(ref)  # raises if the build reported an error
    assert np.array_equal(b2.GetOctree()[: len(ref)].cpu().numpy().view(np.uint32), ref)


@pytest.mark.parametrize("short_by", [8, 64])
def test_build_into_pool_short_of_the_leaf_range(cuda, short_by):
    """A pool that holds every interior block but not the whole leaf range: SVO_ERR_CAPACITY through the
    status word and no word written past `capacity` (guard words behind it stay intact)."""
    import ctypes

    import torch
    from sparsevoxeloctree_gb300 import _lib
    lib = _lib.load()
    s = scenes.plain_256()
    frags = oracle.voxelize(s.tris, s.level)
    ref = oracle.build_octree(frags, s.level)
    cap = len(ref) - short_by
    t = torch.from_numpy(frags.view(np.int64)).cuda()
    pool = torch.full((cap + 4096,), 0x5A5A5A5A, dtype=torch.int32, device="cuda")
    ws = torch.empty(lib.svo_build_workspace_size(len(frags), s.level, cap, 0), dtype=torch.uint8, device="cuda")
    res = torch.zeros(64, dtype=torch.int32, device="cuda")
    rc = lib.svo_build_into(ctypes.c_void_p(t.data_ptr()), len(frags), s.level, ctypes.c_void_p(pool.data_ptr()), cap,
                            ctypes.c_void_p(ws.data_ptr()), ws.numel(), ctypes.c_void_p(res.data_ptr()), None)
    assert rc == _lib.SVO_OK
    torch.cuda.synchronize()
    status = int(res.cpu().numpy().view(np.uint32)[ctypes.sizeof(_lib.BuildInfo) // 4])
    assert status & 2  # capacity
    assert bool((pool[cap:] == 0x5A5A5A5A).all())


@pytest.mark.parametrize("size", [(37, 23), (7, 5), (1, 1), (1921, 3), (8, 4)])
def test_camera_image_sizes_not_multiple_of_the_tile(cuda, size):
    """Camera rays are claimed in 8x4 tiles: edge tiles must cover every pixel exactly once."""
    import torch
    api = _api()
    s = scenes.plain_256()
    frags = oracle.voxelize(s.tris, s.level)
    o, pool = gpu_build(frags, s.level)
    w, h = size
    cam = scenes.camera_from_angles((1.5, 1.5, 0.5), 0.05, 0.02, np.pi / 3, w / h)
    n = w * h
    hits = torch.full((n * 32 + 64,), 0xAB, dtype=torch.uint8, device="cuda")  # guard bytes after the image
    api.OctreeTracer.Create(o, cam, w, h).CmdDrawPipeline(hits[: n * 32])
    raw = hits.cpu().numpy()
    assert (raw[n * 32:] == 0xAB).all()  # nothing written past the last pixel
    got = raw[: n * 32].view(np.uint8).view(HIT_DTYPE)
    assert_hits_equal(got, oracle.raycast(pool, s.level, oracle.camera_rays(cam, w, h)))


@pytest.mark.parametrize("bands", [0, 1, 2, 4, 8, 16])
@pytest.mark.parametrize("size", [(37, 23), (1, 1), (64, 3), (300, 97)])
@pytest.mark.parametrize("pinned", [True, False])
def test_camera_download_to_host(cuda, size, bands, pinned):
    """svo_raycast_camera_download: mode 0 stores the hits straight into a mapped (pinned) host buffer;
    band counts trace the image in row bands and copy each band while the next is traced (a pageable host
    buffer always takes the copies).  The host image equals the oracle's and nothing is written past it."""
    import torch

    from sparsevoxeloctree_gb300 import autotune
    if bands not in (0, 2) and not pinned:
        pytest.skip("pageable buffers: one copy mode is enough")
    api = _api()
    s = scenes.plain_256()
    frags = oracle.voxelize(s.tris, s.level)
    o, pool = gpu_build(frags, s.level)
    w, h = size
    n = w * h
    cam = scenes.camera_from_angles((1.5, 1.5, 0.5), 0.05, 0.02, np.pi / 3, w / h)
    autotune.set_value("download_bands", 0, -1, bands)
    try:
        dev = torch.full((n * 32 + 64,), 0xAB, dtype=torch.uint8, device="cuda")
        host = torch.full((n * 32 + 64,), 0xCD, dtype=torch.uint8)
        if pinned:
            host = host.pin_memory()
        api.OctreeTracer.Create(o, cam, w, h).CmdDrawPipelineToHost(host, dev[: n * 32])
        torch.cuda.synchronize()
    finally:
        _lib_reset_tune()
    raw = host.numpy()
    assert (raw[n * 32:] == 0xCD).all() and (dev[n * 32:].cpu().numpy() == 0xAB).all()
    if bands == 0 and pinned:
        assert (dev.cpu().numpy() == 0xAB).all()  # written straight to the host: the staging buffer is untouched
    else:
        assert np.array_equal(raw[: n * 32], dev[: n * 32].cpu().numpy())
    assert_hits_equal(raw[: n * 32].view(HIT_DTYPE), oracle.raycast(pool, s.level, oracle.camera_rays(cam, w, h)))


def _lib_reset_tune():
    from sparsevoxeloctree_gb300 import _lib
    _lib.load().svo_tune_reset()


def test_voxelizer_reemission_needs_exact_unit_scratch(cuda):
    """A mesh that needs more raster units than the default scratch guess (three copies of the room's
    walls at level 10: 36 triangles of 1024 spans x 4 pieces, 147,456 units against a guess of 65,608):
    re-emission (CmdVoxelize) must size its scratch from the first pass's unit count and reproduce every
    fragment, in order."""
    api = _api()
    level = 10
    walls = np.concatenate([scenes.room_shell(level)] * 3, 0)
    tris = scenes._soup(walls, scenes.random_colors(scenes.rng(17), len(walls)))
    v = api.Voxelizer.Create(tris, level)
    first = v.GetVoxelFragmentList().clone()
    assert v.m_units > 2 * len(tris) + 65536  # more than the default guess
    v.GetVoxelFragmentList().fill_(0)
    v.CmdVoxelize()
    v.CheckEmission()
    import torch
    assert torch.equal(v.GetVoxelFragmentList(), first)
    assert_same_fragments(first.cpu().numpy().view(np.uint64), oracle.voxelize(tris, level))


# ------------------------------------------------------------------------------------------- beam / occlusion
def _golden_octree(golden_dir):
    import torch
    api = _api()
    zb = np.load(f"{golden_dir}/golden_build.npz")
    level, pool = int(zb["level"]), zb["pool"]
    o = api.Octree()
    o.m_buffer = torch.from_numpy(pool.view(np.int32)).cuda()
    o.m_range, o.m_level = len(pool) * 4, level
    return o, pool, level


def test_beam_prepass_golden_and_oracle(cuda, golden_dir):
    """The beam image bit for bit against the reference's beam pre-pass and the oracle; the beam march
    (primary rays advanced by it) against the oracle's march of the advanced rays."""
    from sparsevoxeloctree_gb300.formats import CAMERA_DTYPE
    api = _api()
    octree, pool, level = _golden_octree(golden_dir)
    zbeam = np.load(f"{golden_dir}/golden_beam.npz")
    for k in range(2):
        cam = np.frombuffer(zbeam[f"cam{k}"].tobytes(), CAMERA_DTYPE)[0]
        w, h = (int(x) for x in zbeam[f"size{k}"])
        tr = api.OctreeTracer.Create(octree, cam, w, h)
        beam = tr.CmdBeamRenderPass().cpu().numpy()
        assert np.array_equal(beam, zbeam[f"beam{k}"])
        hits = api.hits_numpy(tr.CmdDrawPipelineBeam())
        ref = oracle.raycast(pool, level, oracle.camera_rays_beam(cam, w, h, zbeam[f"beam{k}"]))
        assert_hits_equal(hits, ref)
        again = api.hits_numpy(tr.CmdDrawPipelineBeam(beam=tr.CmdBeamRenderPass()))
        assert np.array_equal(again, hits)


def test_beam_on_built_scene_matches_oracle(cuda):
    api = _api()
    s = scenes.plain_256()
    frags = oracle.voxelize(s.tris, s.level)
    octree, pool = gpu_build(frags, s.level)
    for pos, yaw, pitch, w, h in [((1.5, 1.5, 0.5), 0.0, 0.0, 64, 64), ((1.5, 1.45, 1.5), 0.7, -0.2, 97, 53)]:
        cam = scenes.camera_from_angles(pos, yaw, pitch, aspect=w / h)
        b_ref = oracle.beam(pool, s.level, cam, w, h)
        tr = api.OctreeTracer.Create(octree, cam, w, h)
        assert np.array_equal(tr.CmdBeamRenderPass().cpu().numpy(), b_ref)
        assert_hits_equal(api.hits_numpy(tr.CmdDrawPipelineBeam()),
                          oracle.raycast(pool, s.level, oracle.camera_rays_beam(cam, w, h, b_ref)))


def test_occlusion_golden_and_oracle(cuda, golden_dir):
    api = _api()
    octree, pool, level = _golden_octree(golden_dir)
    zm, zocc = np.load(f"{golden_dir}/golden_march.npz"), np.load(f"{golden_dir}/golden_occlude.npz")
    rays = rays_from_arrays(zm["o"], zm["d"])
    got = api.OctreeTracer.Create(octree).Occlude(api.to_device(rays)).cpu().numpy().view(np.uint32)
    assert np.array_equal(got, zocc["occluded"])
    # a built scene, random rays and null rays (missed bounces)
    s = scenes.plain_256()
    frags = oracle.voxelize(s.tris, s.level)
    oc, pool2 = gpu_build(frags, s.level)
    g = np.random.default_rng(12)
    o, d = scenes.random_rays(g, 5000, inside=True)
    r2 = rays_from_arrays(o, d)
    r2["d"][:50] = 0
    got2 = api.OctreeTracer.Create(oc).Occlude(api.to_device(r2)).cpu().numpy().view(np.uint32)
    assert np.array_equal(got2, oracle.occlude(pool2, s.level, r2))
    assert not got2[:50].any()


# ------------------------------------------------------------------------------------------- files
def test_octree_save_load_and_obj_pipeline(cuda, tmp_path):
    """An OBJ loaded with the reference's normalisation runs the whole path; the octree saved to a file
    and loaded back traces identically."""
    api = _api()
    s = scenes.plain_256()
    lines = ["mtllib m.mtl", "usemtl a"]
    verts = s.tris["v"].reshape(-1, 3)[: 3 * 4000] * 7.0 - 2.0  # any frame: the loader normalises it
    lines += [f"v {x:.7g} {y:.7g} {z:.7g}" for x, y, z in verts]
    lines += [f"f {3 * i + 1} {3 * i + 2} {3 * i + 3}" for i in range(len(verts) // 3)]
    (tmp_path / "m.obj").write_text("\n".join(lines) + "\n")
    (tmp_path / "m.mtl").write_text("newmtl a\nKd 0.5 0.75 1.0\n")
    tris = api.load_obj(str(tmp_path / "m.obj"))
    level = 7
    frags = gpu_voxelize(tris, level)
    ref_frags = oracle.voxelize(tris, level)
    assert_same_fragments(frags, ref_frags)
    octree, words = gpu_build(frags, level)
    assert np.array_equal(words, oracle.build_octree(ref_frags, level))
    path = str(tmp_path / "m.svo")
    api.save_octree(octree, path)
    loaded = api.load_octree(path)
    assert loaded.GetLevel() == level and np.array_equal(loaded.words().cpu().numpy().view(np.uint32), words)
    g = np.random.default_rng(2)
    o, d = scenes.random_rays(g, 3000)
    rays = rays_from_arrays(o, d)
    assert np.array_equal(gpu_trace(loaded, rays), gpu_trace(octree, rays))


# ------------------------------------------------------------------------------------------- launch variants
def test_every_march_variant_matches_oracle(cuda):
    """Every launch variant the autotuner can pick (block size, rays per lane or persistent refill, stack
    in shared or local memory) gives the same hits, bit for bit."""
    import itertools
    from sparsevoxeloctree_gb300 import _lib, autotune
    api = _api()
    s = scenes.plain_256()
    frags = oracle.voxelize(s.tris, s.level)
    octree, pool = gpu_build(frags, s.level)
    cam = scenes.camera_from_angles((1.5, 1.45, 1.4), 0.4, -0.1, aspect=1.3)
    w, h = 83, 64
    ref_cam = oracle.raycast(pool, s.level, oracle.camera_rays(cam, w, h))
    g = np.random.default_rng(8)
    o, d = scenes.random_rays(g, 7000, inside=True)
    rays = rays_from_arrays(o, d)
    rays["d"][:20] = 0  # null rays
    ref_rays = oracle.raycast(pool, s.level, rays)
    rays_dev = api.to_device(rays)
    try:
        for tpb, rpl, shared in itertools.product((64, 128, 256), (0, 1, 2), (0, 1)):
            for name, v in (("march_block", tpb), ("march_rays_per_lane", rpl), ("march_stack_shared", shared),
                            ("march_buffer_rays", rpl)):
                autotune.set_value(name, 0, -1, v)
            tr = api.OctreeTracer.Create(octree, cam, w, h)
            assert_hits_equal(api.hits_numpy(tr.CmdDrawPipeline()), ref_cam)
            assert_hits_equal(api.hits_numpy(tr.Trace(rays_dev)), ref_rays)
    finally:
        _lib.load().svo_tune_reset()


def test_node_fetch_counts_match_oracle(cuda):
    """Launches that report node fetches run their own kernel instantiation (the usual launch carries no
    counter): the count equals the oracle's per-ray fetches summed, and the hits are the same as
    without counting, for camera rays, a ray buffer and the counting server."""
    import torch
    api = _api()
    s = scenes.plain_256()
    frags = oracle.voxelize(s.tris, s.level)
    pool = oracle.build_octree(frags, s.level)
    octree, _ = gpu_build(frags, s.level)
    tr = api.OctreeTracer.Create(octree, s.camera, s.width, s.height)
    ref_hits, ref_f = oracle.raycast(pool, s.level, oracle.camera_rays(s.camera, s.width, s.height),
                                     return_fetches=True)
    plain = api.hits_numpy(tr.CmdDrawPipeline())
    counted = api.hits_numpy(tr.CmdDrawPipeline(count_fetches=True))
    torch.cuda.synchronize()
    assert_hits_equal(plain, ref_hits)
    assert_hits_equal(counted, ref_hits)
    assert int(tr.fetches.item()) == int(ref_f.sum())
    g = np.random.default_rng(23)
    o, d = scenes.random_rays(g, 20000, inside=True)
    rays = rays_from_arrays(o, d)
    ref_hits, ref_f = oracle.raycast(pool, s.level, rays, return_fetches=True)
    t2 = api.OctreeTracer.Create(octree)
    got = api.hits_numpy(t2.Trace(api.to_device(rays), count_fetches=True))
    torch.cuda.synchronize()
    assert_hits_equal(got, ref_hits)
    assert int(t2.fetches.item()) == int(ref_f.sum())
    server = api.Server(lanes=1, count_fetches=True)
    try:
        sid = server.AddOctree(octree)
        rh = torch.from_numpy(rays.view(np.uint8).copy()).pin_memory()
        hh = torch.empty(len(rays) * HIT_DTYPE.itemsize, dtype=torch.uint8).pin_memory()
        assert server.Wait(server.SubmitRays(sid, rh, hh))["status"] == 0
        assert_hits_equal(hh.numpy().view(HIT_DTYPE), ref_hits)
        assert server.stats()["node_fetches"] == int(ref_f.sum())
    finally:
        server.close()


@pytest.mark.parametrize("level,walls", [(11, 6), (12, 2)])
def test_build_with_depth_10_dense_matches_oracle(cuda, level, walls):
    """From 2^24 fragments up, octrees of level >= 11 keep depth 10 as a dense bitmap too: at level 11
    the leaf parents are then dense (windowed leaf stage, 16^3-voxel buckets), at level 12 depth 11 is
    the one sparse depth.  Walls of the room shell give 25.2 M (level 11, six walls) and 33.5 M (level 12,
    two walls) fragments; the octree must be the oracle's word for word."""
    tris = scenes._soup(scenes.room_shell(level)[: 2 * walls], scenes.random_colors(scenes.rng(level), 2 * walls))
    frags = oracle.voxelize(tris, level)
    assert len(frags) >= 1 << 24
    _, got = gpu_build(frags, level)
    assert np.array_equal(got, oracle.build_octree(frags, level))
