"""Path tracer on the CPU: the oracle against the reference-generated golden image, the engine's default
Sobol numbers, its transcendental restatements and the host-side environment-map tables (no GPU)."""
import ctypes
import os
import sys

import numpy as np
import pytest

import oracle
from sparsevoxeloctree_gb300 import _lib

sys.path.insert(0, os.path.join(os.path.dirname(__file__), "golden"))
from make_golden import pathtrace_inputs  # noqa: E402


def default_matrices() -> np.ndarray:
    m = np.zeros(64 * 32, np.uint32)
    _lib.check(_lib.load().svo_sobol_default_matrices(m.ctypes.data_as(ctypes.c_void_p)))
    return m.reshape(64, 32)


@pytest.mark.parametrize("light_type", [0, 1])
def test_oracle_matches_reference_path_trace_golden(golden_dir, light_type):
    """golden_pathtrace: the reference's path_tracer.comp + sobol.comp (engine sin/cos/atan/acos, engine
    Sobol numbers) on the golden_build pool; the oracle reproduces every word."""
    zb, z = np.load(f"{golden_dir}/golden_build.npz"), np.load(f"{golden_dir}/golden_pathtrace.npz")
    assert np.array_equal(z["matrices"], default_matrices().reshape(-1))
    cam, noise, env = pathtrace_inputs()
    st = oracle.PathTraceState(40, 30, 4, z["matrices"], noise)
    st.render(zb["pool"], int(zb["level"]), cam, light_type=light_type,
              env=oracle.envmap_build(env) if light_type else None, rotation=0.7, multiplier=1.3, samples=3)
    assert np.array_equal(st.sobol, z[f"sobol{light_type}"])
    assert np.array_equal(st.color, z[f"color{light_type}"])
    assert np.array_equal(st.albedo, z[f"albedo{light_type}"])
    assert np.array_equal(st.normal, z[f"normal{light_type}"])


def test_default_sobol_numbers_are_sobol_sequences():
    """Every dimension's direction numbers form a nonsingular triangular generator (m_k odd: the lowest
    set bit of v_k is 2^-k), so each 1-D projection is a (0,1)-sequence: the first 2^k points fall one
    into each interval of width 2^-k.  Dimensions 0 and 1 also stratify the unit square (t = 0)."""
    M = default_matrices().astype(np.uint64)
    for d in range(64):
        for k in range(32):
            assert (M[d, k] >> np.uint64(31 - k)) & np.uint64(1) == 1, (d, k)
            assert M[d, k] & np.uint64((1 << (31 - k)) - 1) == 0, (d, k)
    M = M.astype(np.uint32)
    assert np.array_equal(M[0], (np.uint64(1) << (31 - np.arange(32, dtype=np.uint64))).astype(np.uint32))
    assert len({tuple(r) for r in M}) == 64  # distinct dimensions
    state = np.zeros(65, np.uint32)
    pts = []
    for _ in range(1024):
        pts.append(state[:64].copy())
        oracle.sobol_next(state, M, 64)
    P = np.array(pts, np.uint64)
    for k in (1, 4, 10):
        cells = P[: 1 << k] >> np.uint64(32 - k)
        for d in range(64):
            assert len(np.unique(cells[:, d])) == 1 << k
    for a in range(0, 11):  # 2^a x 2^(10-a) boxes of dimensions 0 and 1 hold one point each
        x, y = P[:, 0] >> np.uint64(32 - a), P[:, 1] >> np.uint64(32 - (10 - a))
        assert len(np.unique(x * np.uint64(1 << (10 - a)) + y)) == 1024


def test_trig_restatements_are_accurate():
    """The engine's sin/cos/atan2/acos stay within a few float ulps of the exact values."""
    g = np.random.default_rng(5)
    xs = np.concatenate([g.uniform(-7, 14, 3000), [0.0, np.pi / 2, np.pi, 2 * np.pi, -np.pi]]).astype(np.float32)
    for x in xs:
        s, c, _, _ = oracle.trig(float(x), 1.0)
        assert abs(s - np.sin(np.float64(x))) < 6e-7 * max(1.0, abs(float(x)))
        assert abs(c - np.cos(np.float64(x))) < 6e-7 * max(1.0, abs(float(x)))
    for y, x in g.uniform(-3, 3, size=(3000, 2)).astype(np.float32):
        a = oracle.trig(float(x), float(y))[2]
        assert abs(a - np.arctan2(np.float64(y), np.float64(x))) < 1e-6
    for x in np.concatenate([g.uniform(-1, 1, 3000), [-1.0, 1.0, 0.0, 0.999999, -0.999999]]).astype(np.float32):
        assert abs(oracle.trig(float(x), 0.0)[3] - np.arccos(np.float64(x))) < 1e-6
    assert oracle.trig(0.0, 0.0)[2] == 0.0


def test_envmap_create_refuses_a_black_map():
    lib = _lib.load()
    img = np.zeros((4, 4, 4), np.float32)
    h = ctypes.c_void_p(0)
    assert lib.svo_envmap_create(img.ctypes.data_as(ctypes.c_void_p), 4, 4, ctypes.byref(h)) == _lib.SVO_ERR_INVALID
    assert not h.value


def test_path_tracer_arguments_are_checked():
    lib = _lib.load()
    h = ctypes.c_void_p(0)
    assert lib.svo_path_tracer_create(0, 10, 4, ctypes.byref(h)) == _lib.SVO_ERR_INVALID
    assert lib.svo_path_tracer_create(10, 10, 0, ctypes.byref(h)) == _lib.SVO_ERR_INVALID
    assert lib.svo_path_tracer_create(10, 10, 32, ctypes.byref(h)) == _lib.SVO_ERR_INVALID
    assert not h.value
