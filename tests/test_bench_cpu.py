"""bench.py's host-side helpers (no GPU): the compact summary it prints as the line's last key, the CPU
description of the baseline, and the algorithmic byte counts behind the roofline."""
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402


def test_cpu_model_names_the_host():
    name = bench.cpu_model()
    assert isinstance(name, str) and name


def test_algorithmic_bytes_of_the_roofline_kernels():
    w = {"fragments": 100, "triangles": 10, "level": 10, "rays": 4, "fetches_per_ray": 5.0, "range_words": 800,
         "leaf_words": 160}
    assert bench.algorithmic_bytes("march_camera", w) == 4 * (32.0 + 4.0 * 5.0)
    assert bench.algorithmic_bytes("dense_mark", w) == 800.0
    assert bench.algorithmic_bytes("build_leaf_windows", w) == 8.0 * 100 + 4.0 * 160
    assert bench.algorithmic_bytes("vox_emit", w) is None  # overlapped on two streams: no roofline basis


def test_summary_block_carries_the_headline_figures():
    line = {
        "value": 1.3214, "roofline": {"frac": 0.178},
        "e2e": {"value": 1.56, "host_link": {"floor_ms": 0.526}},
        "parity": {"fragments": True, "octree": True, "hits_equal_frac": 1.0},
        "batched": {"speedup_vs_sequential": 3.33, "roofline": {"frac": 0.135}, "batched_ms": 3.98},
        "served": {"same_150_requests": {"speedup_vs_plain_abi": 3.97, "speedup_vs_unbatched_server": 3.6},
                   "saturated_400": {"grays_per_s": 3.0},
                   "roofline": {"frac": 0.09, "launch_ms": 0.69, "host_link": {"frac": 0.67}},
                   "poisson": {"100": {"p50_ms": 0.28, "p99_ms": 1.1}}},
        "large": {"summary": {"step_ms": 9.26}},
    }
    out = bench.summary_block(line)
    assert out["step_ms"] == 1.3214 and out["e2e_ms"] == 1.56 and out["e2e_copy_floor_ms"] == 0.526
    assert out["parity"] == {"fragments": True, "octree": True, "hits_equal_frac": 1.0}
    assert out["served_host_link_frac"] == 0.67
    assert out["batched_speedup"] == 3.33 and out["batched_ms"] == 3.98
    assert out["served_p50_p99_ms"] == {"100": [0.28, 1.1]}
    assert out["large"] == {"step_ms": 9.26}


def test_summary_block_without_the_optional_legs():
    out = bench.summary_block({"value": 2.0, "roofline": {"frac": 0.1}})
    assert out["step_ms"] == 2.0 and out["e2e_ms"] is None and out["e2e_copy_floor_ms"] is None


def test_issue_roofline_of_the_march_from_its_committed_capture():
    out = bench.issue_roofline("march_camera", "room_1024", launch_ms=0.4169, sms=152, sm_mhz=2050.6)
    assert out is not None and out["warp_instructions_per_launch"] == 350298511
    assert abs(out["peak"] - 152 * 4 * 2.0506) < 1e-6
    assert 0.6 < out["frac"] < 0.75 and out["source"].endswith("march_kernel_room_1024.md")
    assert bench.issue_roofline("march_camera", "no_such_workload", 0.4, 152, 2000.0) is None
    assert bench.issue_roofline("dense_mark", "room_1024", 0.1, 152, 2000.0) is None


def test_summary_block_carries_the_issue_fraction():
    out = bench.summary_block({"value": 1.27, "roofline": {"frac": 0.18, "issue": {"frac": 0.674}}})
    assert out["march_issue_frac"] == 0.674
