"""Pin the oracle against the reference's own shader source compiled for the CPU (oracle/_ref, built by
oracle/build_ref.py from the reference checkout).  Skipped where the checkout is absent (the GPU machine);
the committed fixtures in tests/golden/ carry the same evidence there."""
import numpy as np
import pytest

import oracle
import oracle.reference as ref
from sparsevoxeloctree_gb300 import scenes
from sparsevoxeloctree_gb300.formats import TRIANGLE_DTYPE, pack_fragments, rays_from_arrays

pytestmark = pytest.mark.skipif(not ref.available(), reason="reference checkout not available")


def test_build_matches_reference_shaders_plain_256():
    s = scenes.plain_256()
    frags = oracle.voxelize(s.tris, s.level)
    got = oracle.build_octree(frags, s.level, oracle.COLOR_REF)
    want = ref.build_octree(frags, s.level, oracle.pool_bound(len(frags), s.level))
    assert np.array_equal(got, want)


@pytest.mark.parametrize("level", [1, 2, 5, 9, 12])
def test_build_matches_reference_shaders_random(level):
    g = np.random.default_rng(level)
    n = 5000
    R = 1 << level
    xyz = g.integers(0, R, size=(n, 3))
    xyz[: n // 3] = xyz[0]  # many fragments on one voxel: running mean and count saturation
    frags = pack_fragments(xyz[:, 0], xyz[:, 1], xyz[:, 2], g.integers(0, 1 << 24, size=n))
    got = oracle.build_octree(frags, level, oracle.COLOR_REF)
    want = ref.build_octree(frags, level, oracle.pool_bound(n, level))
    assert np.array_equal(got, want)


def test_march_matches_reference_shader():
    s = scenes.plain_256()
    frags = oracle.voxelize(s.tris, s.level)
    pool = oracle.build_octree(frags, s.level)
    g = np.random.default_rng(1)
    o1, d1 = scenes.random_rays(g, 20000)
    o2, d2 = scenes.random_rays(g, 20000, inside=True)
    cam = oracle.camera_rays(s.camera, s.width, s.height)
    o = np.concatenate([o1, o2, cam["o"]])
    d = np.concatenate([d1, d2, cam["d"]])
    h = oracle.raycast(pool, s.level, rays_from_arrays(o, d))
    r = ref.raycast(pool, o, d, with_iter=True)
    hit = (h["flags"] & 1).astype(np.uint32)
    assert np.array_equal(hit, r["hit"])
    assert np.array_equal(h["iter"], r["iter"])
    assert np.array_equal(h["pos"], r["pos"])
    col = np.stack([(h["node"] >> (8 * k)) & 255 for k in range(3)], 1).astype(np.float32) / 255.0
    assert np.array_equal(col[hit == 1], r["color"][hit == 1])
    # the 5-argument variant differs only in the EPS clamp (>= instead of >) and the colour scaling
    r5 = ref.raycast(pool, o, d, with_iter=False)
    assert np.array_equal(r5["hit"], r["hit"]) and np.array_equal(r5["pos"], r["pos"])
    assert np.abs(r5["color"] - r["color"]).max() <= 1e-7


def test_camera_matches_reference_shader():
    cam = scenes.camera_from_angles((1.2, 1.8, 1.4), 0.7, -0.2, np.pi / 3, 16 / 9)
    assert np.array_equal(oracle.camera_rays(cam, 64, 36)["d"], ref.camera_dirs(cam, 64, 36))


def test_voxelize_matches_reference_shaders():
    """Grid-aligned triangles through the reference's geometry (both variants) and fragment shaders."""
    g = np.random.default_rng(2)
    L = 5
    S = (1 << L) * 256
    total = diff = 0
    for _ in range(200):
        c = g.integers(0, S, size=3)
        sz = int(g.choice([40, 300, 2000, 8000]))
        V = np.clip(c[None, :] + g.integers(-sz, sz + 1, size=(3, 3)), 0, S - 1)
        p = (V / S).astype(np.float32)
        t = np.zeros(1, TRIANGLE_DTYPE)
        t["v"] = p.reshape(1, 9)
        rgb = int(g.integers(0, 1 << 24))
        t["rgb"] = rgb
        mine = set(oracle.voxelize(t, L).tolist())
        for sw in (False, True):
            theirs = set(ref.voxelize_triangle((2 * p - 1).reshape(9), rgb, L, sw).tolist())
            total += len(theirs)
            diff += len(mine ^ theirs)
    assert diff <= 0.002 * total


@pytest.mark.parametrize("cam_args", [((1.5, 1.5, 0.5), 0.0, 0.0, 64, 48), ((1.5, 1.4, 1.45), 1.2, 0.3, 37, 29)])
def test_beam_and_occlusion_match_reference_shaders(cam_args):
    """Octree_RayMarchCoarse + the beam texel arithmetic, and Octree_RayMarchOcclude."""
    s = scenes.plain_256()
    frags = oracle.voxelize(s.tris, s.level)
    pool = oracle.build_octree(frags, s.level)
    pos, yaw, pitch, w, h = cam_args
    cam = scenes.camera_from_angles(pos, yaw, pitch, aspect=w / h)
    assert np.array_equal(oracle.beam(pool, s.level, cam, w, h), ref.beam(pool, cam, w, h, s.level))
    rays = oracle.camera_rays(cam, w, h)
    g = np.random.default_rng(4)
    o, d = scenes.random_rays(g, 2000, inside=True)
    rays = np.concatenate([rays, rays_from_arrays(o, d)])
    rays["d"][:4] = np.float32([[1, 0, 0], [0, 1e-30, 1], [0, 0, -1], [-1, -3.552713678800501e-15, 0]])
    got = oracle.occlude(pool, s.level, rays)
    want = ref.occlude(pool, rays["o"].astype(np.float32), rays["d"].astype(np.float32)).astype(np.uint32)
    assert np.array_equal(got, want)
