"""OBJ loading with the reference's normalisation and the octree file format (host-side, no GPU)."""
import os

import numpy as np
import pytest

import oracle
from sparsevoxeloctree_gb300 import _lib, scenes
from sparsevoxeloctree_gb300.formats import TRIANGLE_DTYPE


def _api():
    from sparsevoxeloctree_gb300 import api
    return api


OBJ = """# quad (fan), triangle with negative indices, v/t/n forms
mtllib scene.mtl
v 0 0 0
v 4 0 0
v 4 2 0
v 0 2 0
vt 0 0
vn 0 0 1
v 1 1 3
v 3 1 3
v 2 -1 3
usemtl red
f 1/1/1 2/1/1 3/1/1 4/1/1
usemtl blue
f -3//1 -2//1 -1//1
usemtl nosuch
f 1 2 5
"""
MTL = """newmtl red
Kd 1.0 0.25 0.0
newmtl blue
Kd 0.1 0.2 0.9
"""


def _write(tmp_path, obj=OBJ, mtl=MTL):
    (tmp_path / "scene.obj").write_text(obj)
    if mtl is not None:
        (tmp_path / "scene.mtl").write_text(mtl)
    return str(tmp_path / "scene.obj")


def test_obj_normalisation_and_materials(tmp_path):
    tris = _api().load_obj(_write(tmp_path))
    assert len(tris) == 4  # quad -> 2 fan triangles, 1 triangle, 1 with an undefined material
    v = np.float32([[0, 0, 0], [4, 0, 0], [4, 2, 0], [0, 2, 0], [1, 1, 3], [3, 1, 3], [2, -1, 3]])
    faces = [(0, 1, 2), (0, 2, 3), (4, 5, 6), (0, 1, 4)]
    used = v[sorted({i for f in faces for i in f})]
    pmin, pmax = used.min(0), used.max(0)
    extent = np.float32((pmax - pmin).max() * np.float32(0.5))
    inv = np.float32(1.0) / extent
    center = (pmax + pmin) * np.float32(0.5)
    for t, f in zip(tris, faces):
        p = ((v[list(f)] - center) * inv + np.float32(1.0)) * np.float32(0.5)
        assert np.array_equal(t["v"].reshape(3, 3), np.clip(p, 0, 1).astype(np.float32))
    red = 255 | (64 << 8) | (0 << 16)       # round(0.25 * 255) = 64
    blue = 26 | (51 << 8) | (230 << 16)     # round(0.1/0.2/0.9 * 255)
    assert list(tris["rgb"][:, 0]) == [red, red, blue, red]  # undefined material -> first material
    assert (tris["rgb"] == tris["rgb"][:, :1]).all()
    frags = oracle.voxelize(tris, 5)
    assert len(frags) > 0


def test_obj_errors(tmp_path):
    api = _api()
    with pytest.raises(_lib.SvoError):
        api.load_obj(str(tmp_path / "missing.obj"))
    with pytest.raises(_lib.SvoError, match="no material"):
        api.load_obj(_write(tmp_path, mtl=None))
    with pytest.raises(_lib.SvoError, match="bad face index"):
        api.load_obj(_write(tmp_path, obj=OBJ + "f 1 2 99\n"))
    with pytest.raises(_lib.SvoError, match="fewer than 3"):
        api.load_obj(_write(tmp_path, obj=OBJ + "f 1 2\n"))


def test_octree_file_round_trip_and_rejection(tmp_path):
    api = _api()
    s = scenes.plain_256()
    pool = oracle.build_octree(oracle.voxelize(s.tris, s.level), s.level)
    path = str(tmp_path / "o.svo")
    api.write_octree_file(pool, s.level, path)
    assert os.path.getsize(path) == 32 + 4 * len(pool)
    words, level = api.read_octree_file(path)
    assert level == s.level and np.array_equal(words, pool)
    raw = bytearray(open(path, "rb").read())
    bad = [bytes(raw[:-4]), bytes(raw) + b"\0\0\0\0", b"XXXXXXXX" + bytes(raw[8:])]
    interior = next(i for i, w in enumerate(pool) if (w >> 30) == 2)  # an interior word
    b = bytearray(raw)
    b[32 + 4 * interior: 32 + 4 * interior + 4] = np.uint32(0x80000000 | (len(pool) + 8)).tobytes()
    bad.append(bytes(b))
    for k, data in enumerate(bad):
        p = str(tmp_path / f"bad{k}.svo")
        open(p, "wb").write(data)
        with pytest.raises(_lib.SvoError):
            api.read_octree_file(p)
    with pytest.raises(_lib.SvoError):
        api.write_octree_file(pool[:12], s.level, str(tmp_path / "x.svo"))  # range not a multiple of 8
