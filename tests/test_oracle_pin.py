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


# ---------------------------------------------------------------------------------------------- path tracer
def _pt_scene():
    s = scenes.plain_256()
    pool = oracle.build_octree(oracle.voxelize(s.tris, s.level), s.level)
    return s, pool


def test_sobol_matches_reference_shader():
    """shader/sobol.comp over 300 steps, from the reference's own direction numbers."""
    M = ref.sobol_matrices()
    for dim in (4, 10, 34, 64):
        a = np.zeros(65, np.uint32)
        b = np.zeros(65, np.uint32)
        for _ in range(300):
            oracle.sobol_next(a, M, dim)
            ref.sobol_next(b, dim)
            assert np.array_equal(a, b)


@pytest.mark.parametrize("shape", [(16, 32), (7, 5), (1, 1), (64, 128)])
def test_envmap_tables_match_reference_code(shape):
    """EnvironmentMap::weigh_hdr_image + generate_alias_table compiled from src/EnvironmentMap.cpp."""
    g = np.random.default_rng(shape[0] * 100 + shape[1])
    img = np.zeros(shape + (4,), np.float32)
    img[..., :3] = g.random(shape + (3,), dtype=np.float32) * g.choice([0.01, 1.0, 50.0], size=shape + (1,))
    if img.shape[0] * img.shape[1] > 1:
        img[0, 0, :3] = 0.0  # a black texel
    got, want = oracle.envmap_build(img), ref.envmap_build(img)
    assert np.array_equal(got[0], want[0]) and np.array_equal(got[1], want[1])
    img[..., :3] = 0.0  # no luminance: nothing to sample (the reference would divide by zero)
    assert oracle.envmap_build(img) is None and ref.envmap_build(img) is None


def _pt_compare(light_type, bounce, w, h, samples, env=None, rot=0.0, mult=1.0, engine_trig=False):
    s, pool = _pt_scene()
    g = np.random.default_rng(bounce * 31 + light_type)
    noise = g.integers(0, 256, size=256 * 256 * 2, dtype=np.uint8)
    M = ref.sobol_matrices()
    cam = scenes.camera_from_angles((1.5, 1.45, 1.05), 0.35, -0.2, aspect=w / h)
    st = oracle.PathTraceState(w, h, bounce, M, noise)
    env_o = oracle.envmap_build(env) if env is not None else None
    st.render(pool, s.level, cam, light_type=light_type, env=env_o, samples=samples, rotation=rot, multiplier=mult)
    sob = np.zeros(65, np.uint32)
    col = np.zeros((h, w, 4), np.float32)
    alb = np.zeros((h, w), np.uint32)
    nrm = np.zeros((h, w), np.uint32)
    env_r = ref.envmap_build(env) if env is not None else None
    ref.path_trace(pool, cam, w, h, bounce, sob, noise, col, alb, nrm, light_type=light_type, env=env_r,
                   samples=samples, rotation=rot, multiplier=mult, engine_trig=engine_trig)
    return st, sob, col, alb, nrm


_ENV_RNG = np.random.default_rng(9)
ENV = np.zeros((16, 32, 4), np.float32)
ENV[..., :3] = _ENV_RNG.random((16, 32, 3), dtype=np.float32)
ENV[3, 7, :3] = 40.0  # a sun


@pytest.mark.parametrize("light_type", [0, 1])
@pytest.mark.parametrize("bounce", [1, 2, 4, 8])
def test_path_trace_matches_reference_shader_exactly(light_type, bounce):
    """shader/path_tracer.comp + shader/sobol.comp (ConstColorPathTrace / EnvMapPathTrace with MIS, the
    running means of main()) from the reference source, with GLSL's sin / cos / atan / acos evaluated by
    the engine's restatements: colour, albedo, normal and Sobol state agree bit for bit over 3 samples."""
    st, sob, col, alb, nrm = _pt_compare(light_type, bounce, 40, 30, 3, env=ENV if light_type else None, rot=0.7,
                                         mult=1.3, engine_trig=True)
    assert np.array_equal(sob, st.sobol)
    assert np.array_equal(col, st.color)
    assert np.array_equal(alb, st.albedo) and np.array_equal(nrm, st.normal)


@pytest.mark.parametrize("light_type", [0, 1])
def test_path_trace_with_libm_trig_matches_in_distribution(light_type):
    """With libm's transcendentals in the reference build, first-hit albedo / normal and the Sobol state
    still agree exactly; radiance differs where a direction's last bits change which voxel a bounce or
    shadow ray meets (a ray leaving a face starts on it), so only the image means are compared."""
    st, sob, col, alb, nrm = _pt_compare(light_type, 4, 40, 30, 3, env=ENV if light_type else None, rot=0.7,
                                         mult=1.3)
    assert np.array_equal(sob, st.sobol)
    assert np.array_equal(alb, st.albedo) and np.array_equal(nrm, st.normal)
    assert (col == st.color).all(axis=2).mean() >= (0.8 if light_type == 0 else 0.1)
    assert abs(col[..., :3].mean() - st.color[..., :3].mean()) <= 0.02 * col[..., :3].mean()


# ---------------------------------------------------------------------------------------------- textures
def test_textured_fragment_shader_logic_matches_reference():
    """voxelizer.frag's textured branch (Sample(): alpha < 0.5 discards; packUnorm4x8 colour) with a 1x1
    texture, whose every filtered sample is its one texel: the oracle keeps or drops each triangle's
    fragments as the reference shader does and gives them the same colour word."""
    g = np.random.default_rng(12)
    L = 5
    S = (1 << L) * 256
    lin = [((c / 255.0) / 12.92 if c / 255.0 <= 0.04045 else ((c / 255.0 + 0.055) / 1.055) ** 2.4) for c in range(256)]
    total = diff = 0
    for it in range(120):
        c = g.integers(0, S, size=3)
        sz = int(g.choice([40, 300, 2000]))
        V = np.clip(c[None, :] + g.integers(-sz, sz + 1, size=(3, 3)), 0, S - 1)
        p = (V / S).astype(np.float32)
        t = np.zeros(1, TRIANGLE_DTYPE)
        t["v"] = p.reshape(1, 9)
        img = g.integers(0, 256, size=(1, 1, 4), dtype=np.uint8)
        img[0, 0, 3] = [0, 100, 127, 128, 200, 255][it % 6]
        uv = np.zeros(1, oracle.UV_DTYPE)
        uv["uv"] = g.uniform(-2, 3, size=(1, 6)).astype(np.float32)
        uv["texture"] = 0
        mine = oracle.voxelize_textured(t, uv, L, [img])
        texel = np.array([lin[img[0, 0, 0]], lin[img[0, 0, 1]], lin[img[0, 0, 2]], img[0, 0, 3] / 255.0], np.float32)
        theirs = ref.voxelize_triangle_texel((2 * p - 1).reshape(9), texel, L, True)
        if img[0, 0, 3] < 128:
            assert len(mine) == 0 and len(theirs) == 0
            continue
        assert len(set((mine >> 32).tolist())) <= 1 and set((mine >> 32).tolist()) == set((theirs >> 32).tolist())
        a, b = set(mine.tolist()), set(theirs.tolist())
        total += len(b)
        diff += len(a ^ b)
    assert total > 0 and diff <= 0.002 * total
