"""Autotuner of the engine's launch parameters.

The library keeps one value per (parameter, octree level, size class of the launch's work items) and
every launch reads it (svo_tune_set / svo_tune_get, include/svo.h).  This module measures the candidate
values on a real workload with CUDA events and sets the fastest:

  march   threads per block (64 / 128 / 256) x rays per lane per ticket (1 / 2, or persistent refill) x
          stack in shared or local memory, exhaustively (18 variants), on the workload's camera launch
          (and the rays-per-lane choice of ray-buffer launches when the workload traces bounce rays);
  build   blocks per SM of the fragment sweeps x blocks per SM of the leaf stage x one or two streams
          for the bucket / dense stages, on a build;
  emit    blocks per SM of the voxelizer's emission, on a voxelize pass.

The resulting table (parameter -> {"level:size_class": value}) is what `save` writes and `load` applies,
so a tuned table can be reused by later processes.  Results never depend on the parameters, only the
speed does.
"""
from __future__ import annotations

import itertools
import json
import statistics

import torch

from . import _lib

PARAMS = {  # name -> (parameter id, candidate values)
    "march_block": (0, (64, 128, 256)),
    "march_rays_per_lane": (1, (1, 2, 0)),  # 0: persistent refill
    "march_stack_shared": (2, (1, 0)),
    "sweep_blocks": (3, (8, 16, 32)),
    "leaf_blocks": (4, (4, 6, 8)),
    "emit_blocks": (5, (8, 16, 32)),
    "build_streams": (6, (2, 1)),
    "march_buffer_rays": (7, (0, 1, 2)),  # rays per lane for ray-buffer marches (0: persistent refill)
    "download_bands": (8, (0, 1, 2, 4)),  # camera-to-host: 0 = store into mapped host memory, else row bands
}


def size_class(items: int) -> int:
    return int(_lib.load().svo_tune_size_class(int(items)))


def get(name: str, level: int, items: int) -> int:
    return int(_lib.load().svo_tune_get(PARAMS[name][0], level, int(items)))


def set_value(name: str, level: int, cls: int, value: int) -> None:
    _lib.check(_lib.load().svo_tune_set(PARAMS[name][0], level, cls, int(value)))


def _time_ms(fn, reps: int = 3, warmup: int = 1) -> float:
    for _ in range(warmup):
        fn()
    out = []
    for _ in range(reps):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        fn()
        b.record()
        b.synchronize()
        out.append(a.elapsed_time(b))
    return statistics.median(out)


def _sweep(names, level: int, items: int, fn, reps: int = 3) -> dict:
    """Times fn under every combination of the named parameters at (level, class(items)); sets and
    returns the fastest combination with its time."""
    cls = size_class(items)
    best = None
    trials = []
    for combo in itertools.product(*(PARAMS[n][1] for n in names)):
        for n, v in zip(names, combo):
            set_value(n, level, cls, v)
        ms = _time_ms(fn, reps)
        trials.append((dict(zip(names, combo)), ms))
        if best is None or ms < best[1]:
            best = (dict(zip(names, combo)), ms)
    for n, v in best[0].items():
        set_value(n, level, cls, v)
    return {"level": level, "size_class": cls, "best": best[0], "best_ms": best[1],
            "trials": [{"params": p, "ms": m} for p, m in trials]}


def tune_march(tracer, hits=None, reps: int = 3) -> dict:
    """tracer: api.OctreeTracer with a camera; tunes the camera-ray launch of its image."""
    n = tracer.m_width * tracer.m_height
    hits = hits if hits is not None else tracer.CmdDrawPipeline()
    return _sweep(["march_block", "march_rays_per_lane", "march_stack_shared"], tracer.m_octree.GetLevel(), n,
                  lambda: tracer.CmdDrawPipeline(hits), reps)


def tune_build(builder, reps: int = 3) -> dict:
    """builder: api.OctreeBuilder; tunes the fragment sweeps and the leaf stage of its build."""
    return _sweep(["sweep_blocks", "leaf_blocks", "build_streams"], builder.GetLevel(), builder.m_count,
                  builder.CmdBuild, reps)


def tune_voxelize(voxelizer, reps: int = 3) -> dict:
    """voxelizer: api.Voxelizer; tunes the emission of its re-recorded pass."""
    return _sweep(["emit_blocks"], voxelizer.GetLevel(), voxelizer.m_n_tris, voxelizer.CmdVoxelize, reps)


def tune_batch(batcher, meshes, fragments: int, triangles: int, reps: int = 2) -> dict:
    """batcher: api.BatchBuilder with `meshes` built once; tunes sweeps, leaf stage and emission at the
    batch's deepest level (the level its launches select their parameters by)."""
    level = max(lv for _, lv in meshes)
    out = {"build": _sweep(["sweep_blocks", "leaf_blocks", "build_streams"], level, fragments,
                           lambda: batcher.Build(meshes), reps)}
    out["emit"] = _sweep(["emit_blocks"], level, triangles, lambda: batcher.Build(meshes), reps)
    return out


def table(levels=range(1, 13), classes=range(8)) -> dict:
    """The library's current table: {param: {"level:class": value}} for every entry off its default."""
    lib = _lib.load()
    lib.svo_tune_get  # noqa: B018 - loaded
    out = {}
    for name, (pid, cands) in PARAMS.items():
        default = None
        entries = {}
        for lv in levels:
            for c in classes:
                items = 0 if c == 0 else (1 << (16 + 2 * (c - 1)))
                entries[f"{lv}:{c}"] = int(lib.svo_tune_get(pid, lv, items))
        default = statistics.mode(entries.values())
        out[name] = {"default": default, **{k: v for k, v in entries.items() if v != default}}
    return out


def save(path: str) -> None:
    with open(path, "w") as f:
        json.dump(table(), f, indent=1, sort_keys=True)


def load(path: str) -> None:
    with open(path) as f:
        tab = json.load(f)
    for name, entries in tab.items():
        if name not in PARAMS:
            continue
        if "default" in entries:
            set_value(name, 0, -1, entries["default"])
        for key, v in entries.items():
            if key == "default":
                continue
            lv, c = (int(x) for x in key.split(":"))
            set_value(name, lv, c, v)
