"""Texture-sampled fragment colour on the GPU (shader/voxelizer.frag:27-36): the engine's mip chains and
textured voxelization bit for bit against the oracle, and the untextured case against svo_voxelize."""
import numpy as np
import pytest

import oracle
from sparsevoxeloctree_gb300 import scenes
from sparsevoxeloctree_gb300.formats import TRIANGLE_DTYPE

pytestmark = pytest.mark.gpu


def _api():
    from sparsevoxeloctree_gb300 import api
    return api


def _textures(g):
    imgs = [g.integers(0, 256, size=(16, 16, 4), dtype=np.uint8),
            g.integers(0, 256, size=(7, 33, 4), dtype=np.uint8),
            g.integers(0, 256, size=(64, 64, 4), dtype=np.uint8),
            g.integers(0, 256, size=(1, 1, 4), dtype=np.uint8)]
    imgs[2][..., 3] = np.where((np.arange(64)[:, None] // 8 + np.arange(64)[None, :] // 8) % 2, 255, 0)  # cut-out
    imgs[3][..., 3] = 255
    return imgs


def test_mip_chains_match_oracle(cuda):
    g = np.random.default_rng(4)
    imgs = _textures(g) + [g.integers(0, 256, size=(5, 1, 4), dtype=np.uint8)]
    ts = _api().TextureSet(imgs)
    for t, img in enumerate(imgs):
        want = oracle.texture_mips(img)
        for lv, w in enumerate(want):
            assert np.array_equal(ts.GetLevel(t, lv), w), (t, lv)


@pytest.mark.parametrize("uv_scale", [0.05, 1.0, 40.0])
def test_textured_voxelize_matches_oracle(cuda, uv_scale):
    """Random texture coordinates (magnified, near 1:1 and strongly minified, so every level and both
    filters are used), textures with and without cut-outs, untextured and out-of-range ids."""
    api = _api()
    s = scenes.plain_256()
    g = np.random.default_rng(int(uv_scale * 100))
    imgs = _textures(g)
    uv = np.zeros(len(s.tris), api.UV_DTYPE)
    uv["uv"] = (g.uniform(-1, 1, size=(len(s.tris), 6)) * uv_scale).astype(np.float32)
    uv["texture"] = g.integers(0, 5, size=len(s.tris)).astype(np.uint32)  # 4 = beyond the set: untextured
    uv["texture"][::7] = 0xFFFFFFFF
    got = api.voxelize_textured(s.tris, uv, s.level, api.TextureSet(imgs)).cpu().numpy().view(np.uint64)
    want = oracle.voxelize_textured(s.tris, uv, s.level, imgs)
    assert len(got) == len(want) and 0 < len(got) < len(oracle.voxelize(s.tris, s.level))
    assert np.array_equal(np.sort(got), np.sort(want))


def test_untextured_equals_plain_voxelize(cuda):
    api = _api()
    s = scenes.plain_256()
    uv = np.zeros(len(s.tris), api.UV_DTYPE)
    uv["texture"] = 0xFFFFFFFF
    got = api.voxelize_textured(s.tris, uv, s.level, None).cpu().numpy()
    plain = api.voxelize(s.tris, s.level).cpu().numpy()
    assert np.array_equal(got, plain)  # same fragments in the same order


def test_textured_voxelize_empty_and_all_discarded(cuda):
    api = _api()
    empty = api.voxelize_textured(np.zeros(0, TRIANGLE_DTYPE), np.zeros(0, api.UV_DTYPE), 6, None)
    assert empty.numel() == 0
    s = scenes.plain_256()
    img = np.zeros((4, 4, 4), np.uint8)  # alpha 0 everywhere
    uv = np.zeros(len(s.tris), api.UV_DTYPE)
    got = api.voxelize_textured(s.tris, uv, s.level, api.TextureSet([img]))
    assert got.numel() == 0
