#!/usr/bin/env python3
"""Generate tests/golden/*.npz from the reference's own shader code (oracle/_ref, see oracle/build_ref.py).

Run from the repository root, where the reference checkout is available:
    python tests/golden/make_golden.py
The fixtures are small (well under 1 MB together) and travel with the tests; nothing at test time needs
the reference checkout.

  golden_build.npz   fragments of a small scene (icosphere + boxes at level 6, voxelized by the oracle)
                     and the octree the reference's init/tag/alloc/modify-arg shaders build from them
                     (CAS colour merge in list order, blocks in word order);
  golden_march.npz   rays (random, inside and outside the cube, plus a 32x32 camera) and the outputs of
                     the reference's Octree_RayMarchLeaf (iteration variant) over that octree;
  golden_camera.npz  a camera and the directions Camera_GenRay produces for a 48x32 image;
  golden_vox.npz     grid-aligned triangles and the fragments the reference's conservative geometry
                     shader + fragment shader produce for them (pixel-centre raster in double);
  golden_diffuse.npz normals, sample pairs and the reference's Diffuse_Sample directions;
  golden_beam.npz    two cameras and the beam image of the reference's beam pre-pass (Octree_RayMarchCoarse
                     from the shader source, texel arithmetic of shader/octree_tracer_beam.frag) on the
                     golden_build pool;
  golden_occlude.npz Octree_RayMarchOcclude of the golden_march rays on that pool;
  golden_pathtrace.npz the reference's path tracer (shader/path_tracer.comp + shader/sobol.comp, built with
                     GLSL's sin / cos / atan / acos evaluated by the engine's restatements) on the
                     golden_build pool: constant-colour and environment-map light, 4 path vertices,
                     3 samples of a 40x30 image, with the engine's default Sobol numbers, a seeded noise
                     texture and a small environment map.
"""
from __future__ import annotations

import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
import oracle.reference as ref  # noqa: E402
from sparsevoxeloctree_gb300 import scenes  # noqa: E402
from sparsevoxeloctree_gb300.formats import TRIANGLE_DTYPE  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))
SEED = 20260101


def small_scene(level: int = 6):
    g = scenes.rng(SEED, 0)
    sphere = scenes.icosphere(2, 0.3, (0.5, 0.5, 0.5))
    bx = scenes.boxes(scenes.rng(SEED, 1), 8)
    verts = np.concatenate([sphere, bx], 0)
    tris = np.zeros(len(verts), TRIANGLE_DTYPE)
    tris["v"] = verts.astype(np.float32).reshape(-1, 9)
    tris["rgb"] = scenes.random_colors(g, len(verts))
    return tris, level


def pathtrace_inputs():
    """Seeded inputs of golden_pathtrace (rebuilt the same way by the tests): camera, noise, env image."""
    g = scenes.rng(SEED, 5)
    noise = g.integers(0, 256, size=256 * 256 * 2, dtype=np.uint8)
    env = np.zeros((16, 32, 4), np.float32)
    env[..., :3] = g.random((16, 32, 3), dtype=np.float32)
    env[3, 7, :3] = 40.0
    cam = scenes.camera_from_angles((1.5, 1.45, 1.05), 0.35, -0.2, np.pi / 3, 40 / 30)
    return cam, noise, env


def pathtrace_golden(pool, level):
    import ctypes

    from sparsevoxeloctree_gb300 import _lib
    matrices = np.zeros(64 * 32, np.uint32)
    _lib.check(_lib.load().svo_sobol_default_matrices(matrices.ctypes.data_as(ctypes.c_void_p)))
    cam, noise, env = pathtrace_inputs()
    out = {"matrices": matrices, "env": env, "cam": np.frombuffer(cam.tobytes(), np.float32)}
    env_r = ref.envmap_build(env)
    for lt in (0, 1):
        sob = np.zeros(65, np.uint32)
        col = np.zeros((30, 40, 4), np.float32)
        alb = np.zeros((30, 40), np.uint32)
        nrm = np.zeros((30, 40), np.uint32)
        # the engine's default direction numbers replace the reference's kMatrices for this fixture
        ref.path_trace(pool, cam, 40, 30, 4, sob, noise, col, alb, nrm, light_type=lt, env=env_r if lt else None,
                       rotation=0.7, multiplier=1.3, samples=3, engine_trig=True, matrices=matrices)
        out[f"color{lt}"], out[f"albedo{lt}"], out[f"normal{lt}"], out[f"sobol{lt}"] = col, alb, nrm, sob
    np.savez_compressed(os.path.join(OUT, "golden_pathtrace.npz"), **out)


def main() -> int:
    if not ref.available():
        print("reference library not available (run oracle/build_ref.py with the reference checkout)")
        return 2
    tris, level = small_scene()
    frags = oracle.voxelize(tris, level)
    pool = ref.build_octree(frags, level, oracle.pool_bound(len(frags), level))
    np.savez_compressed(os.path.join(OUT, "golden_build.npz"), tris=tris.view(np.uint8), level=level, frags=frags,
                        pool=pool)

    g = scenes.rng(SEED, 2)
    o1, d1 = scenes.random_rays(g, 3000)
    o2, d2 = scenes.random_rays(g, 1000, inside=True)
    cam = scenes.camera_from_angles((1.5, 1.5, 0.5), 0.1, -0.05, np.pi / 3, 1.0)
    cd = ref.camera_dirs(cam, 32, 32)
    o = np.concatenate([o1, o2, np.tile(cam["pos"][:3], (len(cd), 1))]).astype(np.float32)
    d = np.concatenate([d1, d2, cd]).astype(np.float32)
    # a few axis-parallel and tiny-component directions exercise the EPS clamp
    d[:8] = np.array([[1, 0, 0], [0, -1, 0], [0, 0, 1], [1e-20, 1, 0], [-1, 0, 1e-30], [0.6, 0.8, 0],
                      [0, 0, -1], [-1, -1e-16, 0]], np.float32)
    d[:8] /= np.linalg.norm(d[:8], axis=1, keepdims=True)
    r = ref.raycast(pool, o, d, with_iter=True)
    np.savez_compressed(os.path.join(OUT, "golden_march.npz"), o=o, d=d, **{k: v for k, v in r.items()})

    cam2 = scenes.camera_from_angles((1.3, 1.7, 1.2), 2.1, 0.25, np.pi / 3, 1.5)
    np.savez_compressed(os.path.join(OUT, "golden_camera.npz"), cam=np.frombuffer(cam2.tobytes(), np.float32),
                        width=48, height=32, dirs=ref.camera_dirs(cam2, 48, 32))

    g = scenes.rng(SEED, 3)
    vl = 6
    S = (1 << vl) * 256
    vtris, vfrag, vcount = [], [], []
    for _ in range(300):
        c = g.integers(0, S, size=3)
        sz = int(g.choice([32, 128, 512, 2048, 6000]))
        V = np.clip(c[None, :] + g.integers(-sz, sz + 1, size=(3, 3)), 0, S - 1)
        p = (V / S).astype(np.float32)
        rgb = int(g.integers(0, 1 << 24))
        t = np.zeros(1, TRIANGLE_DTYPE)
        t["v"] = p.reshape(1, 9)
        t["rgb"] = rgb
        f = ref.voxelize_triangle((2 * p - 1).reshape(9).astype(np.float32), rgb, vl, True)
        vtris.append(t)
        vfrag.append(f)
        vcount.append(len(f))
    np.savez_compressed(os.path.join(OUT, "golden_vox.npz"), tris=np.concatenate(vtris).view(np.uint8), level=vl,
                        frags=np.concatenate(vfrag), counts=np.array(vcount, np.uint32))

    # beam pre-pass (Octree_RayMarchCoarse + shader/octree_tracer_beam.frag) for an outside and an inside
    # camera, and Octree_RayMarchOcclude for the march rays
    beams = {}
    for k, (pos, yaw, pitch, w, h) in enumerate([((1.5, 1.5, 0.5), 0.1, -0.05, 61, 45), ((1.45, 1.55, 1.3), 2.5, 0.2, 40, 33)]):
        camk = scenes.camera_from_angles(pos, yaw, pitch, np.pi / 3, w / h)
        beams[f"cam{k}"] = np.frombuffer(camk.tobytes(), np.float32)
        beams[f"size{k}"] = np.array([w, h])
        beams[f"beam{k}"] = ref.beam(pool, camk, w, h, level)
    np.savez_compressed(os.path.join(OUT, "golden_beam.npz"), **beams)
    np.savez_compressed(os.path.join(OUT, "golden_occlude.npz"), occluded=ref.occlude(pool, o, d).astype(np.uint32))

    pathtrace_golden(pool, level)

    g = scenes.rng(SEED, 4)
    normals = np.zeros((60, 3), np.float32)
    normals[np.arange(60), np.arange(60) % 3] = np.where(np.arange(60) % 2, -1.0, 1.0)
    u = g.uniform(0, 1, size=(60, 2)).astype(np.float32)
    dirs = np.stack([ref.diffuse_sample(normals[i], float(u[i, 0]), float(u[i, 1])) for i in range(60)])
    np.savez_compressed(os.path.join(OUT, "golden_diffuse.npz"), normals=normals, u=u, dirs=dirs)
    for f in sorted(os.listdir(OUT)):
        if f.endswith(".npz"):
            print(f, os.path.getsize(os.path.join(OUT, f)))
    return 0


if __name__ == "__main__":
    sys.exit(main())
