"""The C++ host classes (include/svo.hpp) over the C ABI: they compile and link here; on a GPU the
reference-shaped pipeline (Scene -> Voxelizer -> OctreeBuilder -> Octree -> OctreeTracer) reproduces the
oracle's fragments, octree and hits."""
import os
import subprocess

import numpy as np
import pytest

import oracle
from sparsevoxeloctree_gb300 import build as engine_build
from sparsevoxeloctree_gb300 import scenes
from sparsevoxeloctree_gb300.formats import HIT_DTYPE

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "wrapper_pipeline.cpp")


def compile_wrapper(tmp_path) -> str:
    engine_build.build()
    exe = str(tmp_path / "wrapper_pipeline")
    libdir = os.path.dirname(engine_build.LIB)
    cmd = ["g++", "-std=c++17", "-O2", "-Wall", "-Wextra", "-I", os.path.join(ROOT, "include"), SRC, "-o", exe,
           "-L", libdir, "-lsvo", f"-Wl,-rpath,{libdir}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_cpp_wrappers_compile_and_link(tmp_path):
    assert os.path.exists(compile_wrapper(tmp_path))


@pytest.mark.gpu
def test_cpp_wrapper_pipeline_matches_oracle(tmp_path, cuda):
    exe = compile_wrapper(tmp_path)
    s = scenes.plain_256()
    (tmp_path / "tris.bin").write_bytes(np.ascontiguousarray(s.tris).tobytes())
    (tmp_path / "cam.bin").write_bytes(np.ascontiguousarray(s.camera).tobytes())
    out = str(tmp_path / "out")
    r = subprocess.run([exe, str(tmp_path / "tris.bin"), str(s.level), str(tmp_path / "cam.bin"), str(s.width),
                        str(s.height), out], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    frags = np.fromfile(out + ".frags", np.uint64)
    pool = np.fromfile(out + ".pool", np.uint32)
    hits = np.fromfile(out + ".hits", HIT_DTYPE)
    ref_frags = oracle.voxelize(s.tris, s.level)
    assert np.array_equal(np.sort(frags), np.sort(ref_frags))
    ref_pool = oracle.build_octree(ref_frags, s.level)
    assert np.array_equal(pool, ref_pool)
    assert np.array_equal(hits, oracle.raycast(ref_pool, s.level, oracle.camera_rays(s.camera, s.width, s.height)))
    beam = np.fromfile(out + ".beam", np.float32)
    assert np.array_equal(beam, oracle.beam(ref_pool, s.level, s.camera, s.width, s.height).reshape(-1))
    # PathTracer: 2 samples, constant light (1, 2, 3), 3 path vertices, noise byte i = 37 i
    import ctypes

    from sparsevoxeloctree_gb300 import _lib
    m = np.zeros(64 * 32, np.uint32)
    _lib.check(_lib.load().svo_sobol_default_matrices(m.ctypes.data_as(ctypes.c_void_p)))
    noise = (np.arange(256 * 256 * 2, dtype=np.uint64) * 37 % 256).astype(np.uint8)
    st = oracle.PathTraceState(s.width, s.height, 3, m, noise)
    st.render(ref_pool, s.level, s.camera, const_color=(1.0, 2.0, 3.0), samples=2)
    pt = np.fromfile(out + ".pt", np.float32).reshape(s.height, s.width, 3)
    assert np.array_equal(pt, st.color[..., :3])
