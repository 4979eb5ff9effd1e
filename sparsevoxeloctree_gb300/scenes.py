"""Seeded synthetic scenes standing in for the reference's OBJ scenes (which are not available here).

Five workloads, with the shapes, sizes and value distributions of the engine's benchmark configurations:

* ``plain_256``   — level 8: subdivision-5 icosphere (20,480 tris, r=0.3, centre 0.5) + 64 boxes,
                    64x64 primary rays from a pinhole at (0.5, 0.5, -0.5) looking +z, fov 60 deg;
* ``room_1024``   — level 10: room shell (12 tris), 200 64-segment cylinders on a jittered grid,
                    210,932 clutter tris (edge lognormal(ln 0.004, 0.7)), 1920x1080 rays from a seeded
                    interior camera;
* ``batch_64``    — 64 clutter meshes, T log-uniform in [1e3, 5e5], level in {7,8,9,10};
* ``clusters_4096`` — level 12: ~10M tris in 4 Gaussian clusters (sigma 0.1, edge lognormal(ln 0.001, 0.8)),
                    3840x2160 primary rays plus one diffuse bounce per hit;
* ``clusters_4096_groups`` — the clusters_4096 triangles as 4 meshes, one per group (batched build).
* ``serving``     — 16 resident scenes (levels 9..11, sphere+boxes+clutter, T log-uniform [5e4, 2e6]).

Meshes are triangle soups in the unit cube (TRIANGLE_DTYPE) with uniform random RGB8 per vertex.  Rays are
in octree space ([1,2]^3, the reference's march convention): unit-cube point p is octree point p + 1.
Every stream is a numpy PCG64 seeded by (seed, item), so each piece is reproducible on its own.
"""
from __future__ import annotations

import math

import numpy as np

from .formats import CAMERA_DTYPE, TRIANGLE_DTYPE


def rng(seed: int, *item: int) -> np.random.Generator:
    return np.random.Generator(np.random.PCG64(np.random.SeedSequence([seed, *item])))


# ---------------------------------------------------------------------------------------------- meshes

def _soup(verts: np.ndarray, colors: np.ndarray) -> np.ndarray:
    """verts (T,3,3) float, colors (T,3) uint32 -> TRIANGLE_DTYPE array."""
    t = np.zeros(len(verts), TRIANGLE_DTYPE)
    t["v"] = np.asarray(verts, np.float32).reshape(-1, 9)
    t["rgb"] = colors
    return t


def random_colors(g: np.random.Generator, n: int) -> np.ndarray:
    return g.integers(0, 1 << 24, size=(n, 3), dtype=np.uint32)


def icosphere(subdiv: int, radius: float, centre) -> np.ndarray:
    """(20*4^subdiv, 3, 3) float64 triangles of a subdivided icosahedron projected to the sphere."""
    p = (1.0 + math.sqrt(5.0)) / 2.0
    v = np.array([[-1, p, 0], [1, p, 0], [-1, -p, 0], [1, -p, 0], [0, -1, p], [0, 1, p], [0, -1, -p],
                  [0, 1, -p], [p, 0, -1], [p, 0, 1], [-p, 0, -1], [-p, 0, 1]], np.float64)
    f = np.array([[0, 11, 5], [0, 5, 1], [0, 1, 7], [0, 7, 10], [0, 10, 11], [1, 5, 9], [5, 11, 4],
                  [11, 10, 2], [10, 7, 6], [7, 1, 8], [3, 9, 4], [3, 4, 2], [3, 2, 6], [3, 6, 8],
                  [3, 8, 9], [4, 9, 5], [2, 4, 11], [6, 2, 10], [8, 6, 7], [9, 8, 1]])
    tris = v[f]
    tris /= np.linalg.norm(tris, axis=2, keepdims=True)
    for _ in range(subdiv):
        a, b, c = tris[:, 0], tris[:, 1], tris[:, 2]
        ab, bc, ca = a + b, b + c, c + a
        ab /= np.linalg.norm(ab, axis=1, keepdims=True)
        bc /= np.linalg.norm(bc, axis=1, keepdims=True)
        ca /= np.linalg.norm(ca, axis=1, keepdims=True)
        tris = np.stack([np.stack([a, ab, ca], 1), np.stack([ab, b, bc], 1), np.stack([ca, bc, c], 1),
                         np.stack([ab, bc, ca], 1)], 1).reshape(-1, 3, 3)
    return tris * radius + np.asarray(centre, np.float64)


def boxes(g: np.random.Generator, n: int, centre_lo=0.1, centre_hi=0.9, half_lo=0.01, half_hi=0.08) -> np.ndarray:
    """(12n, 3, 3) axis-aligned boxes."""
    c = g.uniform(centre_lo, centre_hi, size=(n, 3))
    h = g.uniform(half_lo, half_hi, size=(n, 3))
    corner = np.array([[(i >> 0) & 1, (i >> 1) & 1, (i >> 2) & 1] for i in range(8)], np.float64) * 2 - 1
    faces = [(0, 2, 3, 1), (4, 5, 7, 6), (0, 1, 5, 4), (2, 6, 7, 3), (0, 4, 6, 2), (1, 3, 7, 5)]
    quad = []
    for a, b, cc, d in faces:
        quad += [(a, b, cc), (a, cc, d)]
    quad = np.array(quad)
    pts = c[:, None, :] + h[:, None, :] * corner[None]  # (n, 8, 3)
    return pts[:, quad].reshape(-1, 3, 3)


def clutter(g: np.random.Generator, n: int, mu: float, sigma: float, centres: np.ndarray | None = None) -> np.ndarray:
    """(n,3,3) small random triangles: vertex = centre + random direction * lognormal(mu, sigma), clamped."""
    if centres is None:
        centres = g.uniform(0.0, 1.0, size=(n, 3))
    d = g.normal(size=(n, 3, 3))
    d /= np.maximum(np.linalg.norm(d, axis=2, keepdims=True), 1e-12)
    length = g.lognormal(mu, sigma, size=(n, 3, 1))
    return np.clip(centres[:, None, :] + d * length, 0.0, np.nextafter(1.0, 0.0))


def cylinders(g: np.random.Generator, n: int, segments: int = 64) -> np.ndarray:
    """n vertical cylinders (y up) on a jittered grid resting on the floor: 4*segments tris each."""
    nx, nz = 15, 14
    cells = g.permutation(nx * nz)[:n]
    cx = (cells % nx + g.uniform(0.2, 0.8, size=n)) / nx
    cz = (cells // nx + g.uniform(0.2, 0.8, size=n)) / nz
    r = g.uniform(0.005, 0.02, size=n)
    h = g.uniform(0.3, 0.9, size=n)
    ang = np.linspace(0.0, 2.0 * np.pi, segments + 1)
    out = []
    y0 = np.full(n, 0.5 / 1024.0)
    y1 = y0 + h
    for s in range(segments):
        ax0, az0 = np.cos(ang[s]), np.sin(ang[s])
        ax1, az1 = np.cos(ang[s + 1]), np.sin(ang[s + 1])
        p00 = np.stack([cx + r * ax0, y0, cz + r * az0], 1)
        p01 = np.stack([cx + r * ax1, y0, cz + r * az1], 1)
        p10 = np.stack([cx + r * ax0, y1, cz + r * az0], 1)
        p11 = np.stack([cx + r * ax1, y1, cz + r * az1], 1)
        cb = np.stack([cx, y0, cz], 1)
        ct = np.stack([cx, y1, cz], 1)
        out += [np.stack([p00, p01, p11], 1), np.stack([p00, p11, p10], 1), np.stack([cb, p01, p00], 1),
                np.stack([ct, p10, p11], 1)]
    return np.clip(np.concatenate(out, 0), 0.0, np.nextafter(1.0, 0.0))


def room_shell(level: int) -> np.ndarray:
    """6 walls x 2 tris at the unit cube boundary, inset by half a voxel."""
    e = 0.5 / (1 << level)
    lo, hi = e, 1.0 - e
    c = np.array([[x, y, z] for z in (lo, hi) for y in (lo, hi) for x in (lo, hi)])  # index = x|y<<1|z<<2
    faces = [(0, 2, 6, 4), (1, 5, 7, 3), (0, 4, 5, 1), (2, 3, 7, 6), (0, 1, 3, 2), (4, 6, 7, 5)]
    tris = []
    for a, b, cc, d in faces:
        tris += [(c[a], c[b], c[cc]), (c[a], c[cc], c[d])]
    return np.array(tris, np.float64)


# ---------------------------------------------------------------------------------------------- camera

def camera_from_angles(pos, yaw: float, pitch: float, fov: float = math.pi / 3, aspect: float = 1.0) -> np.ndarray:
    """Camera::fetch_uniform_data (src/Camera.cpp:77-95): look/side/up from yaw about +y then pitch about -x."""
    cy, sy, cp, sp = math.cos(yaw), math.sin(yaw), math.cos(pitch), math.sin(pitch)
    tg = math.tan(fov * 0.5)
    look = np.array([sy * cp, sp, cy * cp])
    look /= np.linalg.norm(look)
    side = np.array([cy, 0.0, -sy])
    side = side / np.linalg.norm(side) * tg * aspect
    up = np.cross(look, side)
    up = up / np.linalg.norm(up) * tg
    cam = np.zeros(1, CAMERA_DTYPE)
    cam["pos"][0, :3] = pos
    cam["look"][0, :3] = look
    cam["side"][0, :3] = side
    cam["up"][0, :3] = up
    cam["pos"][0, 3] = cam["look"][0, 3] = cam["side"][0, 3] = cam["up"][0, 3] = 1.0
    return cam[0]


# ---------------------------------------------------------------------------------------------- workloads

class Scene:
    """One mesh + level + primary camera (octree space) for a plain build+march."""

    def __init__(self, name: str, tris: np.ndarray, level: int, camera: np.ndarray, width: int, height: int,
                 bounce: bool = False, seed: int = 0):
        self.name, self.tris, self.level = name, tris, level
        self.camera, self.width, self.height = camera, width, height
        self.bounce, self.seed = bounce, seed

    @property
    def n_rays(self) -> int:
        return self.width * self.height


def plain_256(seed: int = 1) -> Scene:
    g = rng(seed, 0)
    sphere = icosphere(5, 0.3, (0.5, 0.5, 0.5))
    bx = boxes(rng(seed, 1), 64)
    verts = np.concatenate([sphere, bx], 0)
    tris = _soup(verts, random_colors(g, len(verts)))
    cam = camera_from_angles((1.5, 1.5, 0.5), 0.0, 0.0, math.pi / 3, 1.0)
    return Scene("plain_256", tris, 8, cam, 64, 64, seed=seed)


def interior_camera(g: np.random.Generator, aspect: float) -> np.ndarray:
    pos = g.uniform(0.2, 0.8, size=3) + 1.0
    return camera_from_angles(pos, g.uniform(0.0, 2.0 * math.pi), g.uniform(-0.3, 0.3), math.pi / 3, aspect)


def room_1024(seed: int = 2, clutter_tris: int = 210_932, width: int = 1920, height: int = 1080) -> Scene:
    level = 10
    shell = room_shell(level)
    cyl = cylinders(rng(seed, 1), 200)
    cl = clutter(rng(seed, 2), clutter_tris, math.log(0.004), 0.7)
    verts = np.concatenate([shell, cyl, cl], 0)
    tris = _soup(verts, random_colors(rng(seed, 3), len(verts)))
    cam = interior_camera(rng(seed, 4), width / height)
    return Scene("room_1024", tris, level, cam, width, height, seed=seed)


def _clusters(seed: int, n_tris: int):
    """Triangles of the 4-cluster distribution and each triangle's cluster."""
    g = rng(seed, 0)
    centres_c = g.uniform(0.25, 0.75, size=(4, 3))
    which = g.integers(0, 4, size=n_tris)
    centres = np.clip(centres_c[which] + g.normal(0.0, 0.1, size=(n_tris, 3)), 0.0, np.nextafter(1.0, 0.0))
    verts = clutter(rng(seed, 1), n_tris, math.log(0.001), 0.8, centres=centres)
    return _soup(verts, random_colors(rng(seed, 2), n_tris)), which


def clusters_4096(seed: int = 4, n_tris: int = 10_000_000, width: int = 3840, height: int = 2160,
                  level: int = 12) -> Scene:
    tris, _ = _clusters(seed, n_tris)
    cam = interior_camera(rng(seed, 3), width / height)
    return Scene("clusters_4096", tris, level, cam, width, height, bounce=True, seed=seed)


def clusters_4096_groups(seed: int = 4, n_tris: int = 10_000_000, level: int = 12):
    """The same triangles as clusters_4096 split into its 4 clustered groups: a list of 4 (tris, level)
    meshes for the batched build.  Each group's octree (about a quarter of the whole scene's 1.95 G node
    words at 10 M triangles) fits the 30-bit child-pointer format that the single octree exceeds."""
    tris, which = _clusters(seed, n_tris)
    return [(np.ascontiguousarray(tris[which == k]), level) for k in range(4)]


def batch_64(seed: int = 3, n_meshes: int = 64, t_lo: float = 1e3, t_hi: float = 5e5):
    """List of (tris, level) clutter meshes with log-uniform sizes and levels 7..10."""
    g = rng(seed, 0)
    sizes = np.round(np.exp(g.uniform(math.log(t_lo), math.log(t_hi), size=n_meshes))).astype(np.int64)
    levels = g.integers(7, 11, size=n_meshes)
    out = []
    for i in range(n_meshes):
        verts = clutter(rng(seed, 1, i), int(sizes[i]), math.log(0.004), 0.7)
        out.append((_soup(verts, random_colors(rng(seed, 2, i), len(verts))), int(levels[i])))
    return out


def serving_scenes(seed: int = 5, n_scenes: int = 16, t_lo: float = 5e4, t_hi: float = 2e6, scale: float = 1.0):
    """16 resident scenes: icosphere + boxes + clutter with T log-uniform in [t_lo, t_hi], levels 9..11."""
    g = rng(seed, 0)
    sizes = np.exp(g.uniform(math.log(t_lo), math.log(t_hi), size=n_scenes)) * scale
    levels = g.integers(9, 12, size=n_scenes)
    out = []
    sphere = icosphere(5, 0.3, (0.5, 0.5, 0.5))
    for i in range(n_scenes):
        bx = boxes(rng(seed, 1, i), 64)
        n_cl = max(int(sizes[i]) - len(sphere) - len(bx), 0)
        cl = clutter(rng(seed, 2, i), n_cl, math.log(0.004), 0.7)
        verts = np.concatenate([sphere, bx, cl], 0)
        out.append((_soup(verts, random_colors(rng(seed, 3, i), len(verts))), int(levels[i])))
    return out


def random_rays(g: np.random.Generator, n: int, inside: bool = False) -> tuple[np.ndarray, np.ndarray]:
    """Random rays in octree space: origins outside the cube aimed at it, or inside it."""
    if inside:
        o = g.uniform(1.0, 2.0, size=(n, 3))
        d = g.normal(size=(n, 3))
    else:
        o = g.uniform(-0.5, 3.5, size=(n, 3))
        tgt = g.uniform(1.1, 1.9, size=(n, 3))
        d = tgt - o
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    return o.astype(np.float32), d.astype(np.float32)
