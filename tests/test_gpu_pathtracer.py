"""Path tracer on the GPU (the fused per-pixel kernel of shader/path_tracer.comp): bit for bit against the
reference-generated golden image and against the oracle, for both lights, several bounce counts, image
sizes that are not tile multiples, accumulation over samples, resets and edge cases."""
import ctypes
import os
import sys

import numpy as np
import pytest

import oracle
from sparsevoxeloctree_gb300 import scenes
from sparsevoxeloctree_gb300.formats import CAMERA_DTYPE

sys.path.insert(0, os.path.join(os.path.dirname(__file__), "golden"))
from make_golden import pathtrace_inputs  # noqa: E402

pytestmark = pytest.mark.gpu


def _api():
    from sparsevoxeloctree_gb300 import api
    return api


def _octree(pool, level):
    import torch
    api = _api()
    o = api.Octree()
    o.m_buffer = torch.from_numpy(np.ascontiguousarray(pool, np.uint32).view(np.int32)).cuda()
    o.m_range, o.m_level = len(pool) * 4, level
    return o


def _tracer(octree, cam, w, h, bounce, noise, light_type=0, env=None, rot=0.0, mult=1.0, sun=(5.0, 5.0, 5.0)):
    api = _api()
    em = api.EnvironmentMap.Create()
    if env is not None:
        em.Reset(env)
    em.m_rotation, em.m_multiplier = rot, mult
    light = api.Lighting.Create(em)
    light.m_light_type = light_type
    light.m_sun_radiance = list(sun)
    pt = api.PathTracer.Create(octree, cam, light)
    pt.m_width, pt.m_height, pt.m_bounce = w, h, bounce
    pt.Reset()
    pt.SetNoise(noise)
    return pt


def _images(pt):
    im = pt.GetImages()
    return (im["color"].cpu().numpy(), im["albedo"].cpu().numpy().view(np.uint32),
            im["normal"].cpu().numpy().view(np.uint32), im["sobol"].cpu().numpy().view(np.uint32))


def _default_matrices():
    from sparsevoxeloctree_gb300 import _lib
    m = np.zeros(64 * 32, np.uint32)
    _lib.check(_lib.load().svo_sobol_default_matrices(m.ctypes.data_as(ctypes.c_void_p)))
    return m


@pytest.mark.parametrize("light_type", [0, 1])
def test_path_tracer_matches_reference_golden(cuda, golden_dir, light_type):
    """3 samples of a 40x30 image on the golden_build pool equal, word for word, the reference's
    path_tracer.comp + sobol.comp run (with the engine's sin/cos/atan/acos and Sobol numbers)."""
    zb, z = np.load(f"{golden_dir}/golden_build.npz"), np.load(f"{golden_dir}/golden_pathtrace.npz")
    cam, noise, env = pathtrace_inputs()
    pt = _tracer(_octree(zb["pool"], int(zb["level"])), cam, 40, 30, 4, noise, light_type, env if light_type else None,
                 0.7, 1.3)
    pt.CmdRender(samples=3)
    col, alb, nrm, sob = _images(pt)
    assert np.array_equal(sob, z[f"sobol{light_type}"])
    assert np.array_equal(col, z[f"color{light_type}"])
    assert np.array_equal(alb, z[f"albedo{light_type}"])
    assert np.array_equal(nrm, z[f"normal{light_type}"])
    assert pt.GetSPP() == 3 and pt.GetStatus() == 0


CASES = [  # (light, bounce, w, h, samples, camera)
    (0, 1, 37, 29, 2, ((1.5, 1.5, 0.6), 0.0, 0.0)),
    (0, 2, 64, 48, 3, ((1.4, 1.55, 1.5), 2.3, 0.25)),
    (0, 5, 33, 17, 2, ((1.5, 1.45, 1.05), 0.35, -0.2)),
    (1, 1, 40, 31, 2, ((1.5, 1.5, 0.6), 0.2, 0.1)),
    (1, 3, 48, 40, 3, ((1.45, 1.6, 1.3), 2.5, 0.2)),
    (1, 8, 24, 24, 2, ((1.5, 1.45, 1.05), 0.35, -0.2)),
]


@pytest.mark.parametrize("light_type,bounce,w,h,samples,cam_args", CASES)
def test_path_tracer_matches_oracle(cuda, light_type, bounce, w, h, samples, cam_args):
    s = scenes.plain_256()
    pool = oracle.build_octree(oracle.voxelize(s.tris, s.level), s.level)
    g = np.random.default_rng(bounce * 7 + light_type)
    noise = g.integers(0, 256, size=256 * 256 * 2, dtype=np.uint8)
    env = np.zeros((12, 24, 4), np.float32)
    env[..., :3] = g.random((12, 24, 3), dtype=np.float32) * 2
    env[2, 5, :3] = 25.0
    pos, yaw, pitch = cam_args
    cam = scenes.camera_from_angles(pos, yaw, pitch, aspect=w / h)
    pt = _tracer(_octree(pool, s.level), cam, w, h, bounce, noise, light_type, env if light_type else None, -0.4, 0.8,
                 (2.0, 3.0, 4.0))
    pt.CmdRender(samples=samples)
    col, alb, nrm, sob = _images(pt)
    st = oracle.PathTraceState(w, h, bounce, _default_matrices(), noise)
    st.render(pool, s.level, cam, light_type=light_type, const_color=(2.0, 3.0, 4.0), rotation=-0.4, multiplier=0.8,
              env=oracle.envmap_build(env) if light_type else None, samples=samples)
    assert np.array_equal(sob, st.sobol)
    assert np.array_equal(alb, st.albedo) and np.array_equal(nrm, st.normal)
    assert np.array_equal(col, st.color)
    rgb = pt.ExtractColorImage()
    assert np.array_equal(rgb, col[..., :3])
    assert np.allclose(pt.ExtractAlbedoImage(), ((alb[..., None] >> np.array([0, 8, 16])) & 255) / 255.0)


def test_path_tracer_all_miss_and_reset(cuda):
    """A camera looking out of the octree: every sample is the light itself (constant colour, or the
    environment lookup), albedo and normal stay zero; Reset clears targets and Sobol state."""
    s = scenes.plain_256()
    pool = oracle.build_octree(oracle.voxelize(s.tris, s.level), s.level)
    cam = scenes.camera_from_angles((1.5, 1.5, 0.2), np.pi, 0.0, aspect=1.0)  # outside, facing away
    noise = np.zeros(256 * 256 * 2, np.uint8)
    pt = _tracer(_octree(pool, s.level), cam, 16, 16, 4, noise, sun=(1.5, 2.5, 3.5))
    pt.CmdRender(samples=4)
    col, alb, nrm, sob = _images(pt)
    assert np.all(col[..., :3] == np.float32([1.5, 2.5, 3.5])) and np.all(col[..., 3] == 1.0)
    assert np.all(alb == 0xFF000000) and np.all(nrm == 0x7F000000)
    assert sob[10] == 4
    pt.Reset()
    col, alb, nrm, sob = _images(pt)
    assert not col.any() and not alb.any() and not nrm.any() and not sob.any() and pt.GetSPP() == 0
    # an environment-map request without a map renders with the constant colour (GetFinalLightType)
    api = _api()
    pt.m_lighting.m_light_type = api.Lighting.kEnvironmentMap
    assert pt.m_lighting.GetFinalLightType() == api.Lighting.kConstantColor
    pt.CmdRender()
    assert np.all(_images(pt)[0][..., :3] == np.float32([1.5, 2.5, 3.5]))


def test_envmap_tables_of_the_engine_match_the_oracle(cuda):
    """svo_envmap_create's tables (weights + alias, built on the host) equal the oracle's restatement."""
    api = _api()
    g = np.random.default_rng(2)
    img = np.zeros((9, 20, 4), np.float32)
    img[..., :3] = g.random((9, 20, 3), dtype=np.float32) * 10
    em = api.EnvironmentMap.Create()
    em.Reset(img)
    tex, alias = em.GetTables()
    want = oracle.envmap_build(img)
    assert np.array_equal(tex, want[0]) and np.array_equal(alias, want[1])
    em.Reset()
    assert em.Empty()
