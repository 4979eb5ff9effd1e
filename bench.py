#!/usr/bin/env python3
"""Benchmark: the plain sparse-voxel-octree hot path (voxelize -> build -> primary-ray march) on GB300.

One step = one pass of the whole path over the 2^10 room workload (262,144 triangles, 1920x1080 primary
rays; a seeded synthetic scene standing in for the reference's OBJ scenes): count + emit the fragment
list, build the octree level by level, march every pixel's primary ray.  `value` is the device time of a
step with inputs already in HBM (lower is better), the step's launches recorded once as a CUDA graph and
replayed; `e2e` is the same step through the C ABI with host buffers (triangle upload, the ABI's own
count/range readbacks, hit download), launched call by call.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl engine|reference] [--workload NAME]

--impl reference times the CPU implementation of the same path (the oracle: a restatement pinned
bit-exact to the reference's own shader code) on the host cores, full workload per step.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

from sparsevoxeloctree_gb300 import replicas  # noqa: E402

METRIC = "SVO build ms & Grays/s ray march; batched/served vs plain; served p50/p99 ms"
L2_FLUSH_BYTES = 512 << 20

WORKLOADS = {
    "room_1024": "plain voxelize+build+march at 2^10: room shell, 200 cylinders, 210,932 clutter tris "
                 "(262,144 tris), 1920x1080 primary rays from a seeded interior camera",
    "plain_256": "plain voxelize+build+march at 2^8: icosphere (20,480 tris) + 64 boxes, 64x64 primary rays",
    "clusters_4096": "plain voxelize+build+march at 2^12: ~10M tris in 4 clusters, 3840x2160 primary rays plus one "
                     "diffuse bounce per hit (its octree needs 1.95G node words: beyond the 30-bit pointer format, "
                     "reported as SVO_ERR_CAPACITY)",
    "clusters_4096_4m": "plain voxelize+build+march at 2^12: the 4-cluster distribution with 4M tris (the largest "
                        "that fits the 30-bit pointer format), 3840x2160 primary rays plus one diffuse bounce per hit",
}


def make_scene(name: str):
    from sparsevoxeloctree_gb300 import scenes
    if name == "clusters_4096_4m":
        return scenes.clusters_4096(n_tris=4_000_000)
    return {"room_1024": scenes.room_1024, "plain_256": scenes.plain_256, "clusters_4096": scenes.clusters_4096}[name]()


def load_peaks() -> dict:
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return {"hbm_gbs": float(p["hbm_gbs"]), "source": "measured"}
    except (OSError, KeyError, ValueError):
        return {"hbm_gbs": 6800.0, "source": "fallback"}


# ------------------------------------------------------------------------------------------ clocks
class ClockSampler:
    """nvidia-smi samples (200 ms) of SM clock and throttle reasons while the timed region runs."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.lines: list[str] = []
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                                          "-lms", "100", "-i", str(self.gpu)], stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        if self.thread:
            self.thread.join(timeout=2)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, val in zip(names, parts[5:9]):
                if val.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# ------------------------------------------------------------------------------------------ engine arm
def algorithmic_bytes(kernel: str, w: dict) -> float | None:
    """Algorithmic bytes of one launch: units the launch processes x bytes per unit (design notes)."""
    F, T, L, n, k = w["fragments"], w["triangles"], w["level"], w["rays"], w["fetches_per_ray"]
    leaf_words = w["leaf_words"]
    table = {
        "vox_classify_scan": 48.0 * T + 12.0 * T,     # triangles in, offsets out
        "dense_mark": 8.0 * F,                        # the fragment list, read once
        "build_tag": 8.0 * F,                         # one sparse level: the fragment list
        "build_leaf": 8.0 * F + 4.0 * leaf_words,     # items in, leaf words out (sparse-parent octrees)
        "build_leaf_windows": 8.0 * F + 4.0 * leaf_words,  # items in, leaf words out
        "bucket_scatter": 16.0 * F,                   # fragment in, bucketed item out
        "build_finalize": 12.0 * leaf_words,          # 8 B accumulator in, 4 B leaf word out
        "dense_write": 4.0 * (w["range_words"] - leaf_words),  # interior words out
        "march_camera": n * (32.0 + 4.0 * k),         # hit out + node words fetched (rays made in-kernel)
        "march_rays": n * (24.0 + 32.0 + 4.0 * k),
    }
    return table.get(kernel)


# ncu kernel names of the profile labels whose captures are committed under profiles/
PROFILE_FILES = {"build_leaf_windows": "build_leaf_windows", "bucket_scatter": "bucket_scatter",
                 "march_camera": "march_kernel", "vox_emit_units": "vox_emit_units"}


def profiled_value(label: str, workload: str, key: str):
    """(value, path) of a `key: value` line of the kernel's committed ncu capture on this workload
    (profiles/<kernel>_<workload>.md), or (None, None) without one."""
    name = PROFILE_FILES.get(label)
    if name is None:
        return None, None
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "profiles", f"{name}_{workload}.md")
    if not os.path.exists(path):
        return None, None
    with open(path) as f:
        for line in f:
            if line.startswith(key + ":"):
                return int(line.split(":", 1)[1]), os.path.relpath(path)
    return None, None


def profiled_traffic(label: str, workload: str) -> dict:
    """DRAM bytes per launch (dram__bytes_read.sum + dram__bytes_write.sum) of the kernel, from its
    committed ncu capture on this workload, or null without one."""
    traffic, path = profiled_value(label, workload, "dram_bytes_per_launch")
    return {"traffic": traffic, "traffic_source": path} if traffic is not None else {"traffic": None}


def issue_roofline(label: str, workload: str, launch_ms: float, sms: int, sm_mhz) -> dict | None:
    """The kernel's instruction-issue rate against what the SMs can issue (4 schedulers per SM, one warp
    instruction each per clock, at the SM clock sampled during the timed region): the warp instructions
    of one launch from its committed ncu capture on this workload, divided by the live launch time."""
    wi, path = profiled_value(label, workload, "warp_instructions_per_launch")
    if wi is None or not sm_mhz or not launch_ms:
        return None
    achieved = wi / (launch_ms * 1e-3) / 1e9
    peak = sms * 4 * sm_mhz * 1e6 / 1e9
    return {"unit": "G warp instructions/s", "achieved": achieved, "peak": peak, "frac": achieved / peak,
            "warp_instructions_per_launch": wi, "source": path,
            "peak_basis": f"{sms} SMs x 4 schedulers x 1 warp instruction per clock at {sm_mhz:.0f} MHz"}


def engine_arm(args, env, device, workload: str | None = None, light: bool = False) -> dict:
    """The plain step on `workload` (default: the headline workload).  light: the step, its kernel
    breakdown, roofline and oracle parity only (no beam, path-trace or end-to-end legs)."""
    import numpy as np
    import torch

    from sparsevoxeloctree_gb300 import _lib, api
    from sparsevoxeloctree_gb300.formats import HIT_DTYPE

    lib = _lib.load()
    workload = workload or args.workload
    scene = make_scene(workload)
    T = len(scene.tris)
    n_rays = scene.n_rays
    tris_host = torch.from_numpy(np.ascontiguousarray(scene.tris).view(np.uint8).reshape(-1)).pin_memory()
    tris_dev = tris_host.to(device)
    stream = torch.cuda.current_stream()

    vox = api.Voxelizer.Create(tris_dev, scene.level)
    F = vox.GetVoxelFragmentCount()
    builder = api.OctreeBuilder.Create(vox)
    builder.CmdBuild()
    builder.Reserve()  # pool sized to this scene's exact range
    builder.CmdBuild()
    octree = api.Octree.Create()
    octree.Update(builder)
    tracer = api.OctreeTracer.Create(octree, scene.camera, scene.width, scene.height)
    hits = tracer.CmdDrawPipeline(count_fetches=True)
    torch.cuda.synchronize()
    fetches = int(tracer.fetches.item())
    info = builder.GetInfo()
    hit_np = api.hits_numpy(hits)

    bounce_rays = bounce_hits = None
    if scene.bounce:  # one cosine-weighted diffuse bounce per primary hit, traced in the same step
        bounce_rays = api.OctreeTracer.Bounce(hits, scene.seed)
        bounce_hits = tracer.Trace(bounce_rays)
        torch.cuda.synchronize()

    def step():
        vox.CmdVoxelize()
        builder.CmdBuild()
        tracer.CmdDrawPipeline(hits)
        if scene.bounce:
            api.OctreeTracer.Bounce(hits, scene.seed, bounce_rays)
            tracer.Trace(bounce_rays, bounce_hits)

    tuning = None
    if not args.no_autotune:  # launch parameters measured on this workload before timing
        from sparsevoxeloctree_gb300 import autotune
        t_tune = time.perf_counter()
        tuning = {"emit": autotune.tune_voxelize(vox), "build": autotune.tune_build(builder)}
        if scene.bounce:  # primary and bounce launches share a table entry (same level and ray count): tuned together
            tuning["march"] = autotune._sweep(
                ["march_block", "march_rays_per_lane", "march_stack_shared", "march_buffer_rays"], scene.level,
                n_rays, lambda: (tracer.CmdDrawPipeline(hits), tracer.Trace(bounce_rays, bounce_hits)))
        else:
            tuning["march"] = autotune.tune_march(tracer, hits)
        tuning = {k: {"best": v["best"], "best_ms": v["best_ms"], "level": v["level"], "size_class": v["size_class"],
                      "trials": [[t["params"], round(t["ms"], 4)] for t in v["trials"]]} for k, v in tuning.items()}
        tuning["seconds"] = time.perf_counter() - t_tune

    flush_buf = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device=device)
    for _ in range(args.warmup):
        flush_buf.zero_()
        step()
    torch.cuda.synchronize()
    vox.CheckEmission()  # the re-recorded voxelize pass produced every fragment
    if builder.GetInfo()["range_words"] != info["range_words"]:
        raise RuntimeError("re-recorded build differs from the first build")

    def barrier():
        torch.cuda.synchronize()
        replicas.barrier(env)

    # the step recorded once as a CUDA graph and replayed: the same kernels on the same buffers, without
    # the host launch gaps between the step's ~26 launches (stream capture; the library's per-launch
    # events are off while capturing)
    graph, graph_note = None, None
    try:
        side = torch.cuda.Stream()
        side.wait_stream(stream)
        with torch.cuda.stream(side):
            step()
        stream.wait_stream(side)
        torch.cuda.synchronize()
        graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(graph):
            step()
        torch.cuda.synchronize()
        for _ in range(args.warmup):
            flush_buf.zero_()
            graph.replay()
        torch.cuda.synchronize()
        vox.CheckEmission()
    except Exception as e:  # capture not possible: the eager step is the measurement
        graph, graph_note = None, f"graph capture failed ({type(e).__name__}: {e}); eager step timed"
        torch.cuda.synchronize()

    sampler = ClockSampler(device.index if device.index is not None else 0)
    barrier()
    sampler.start()
    graph_ms = None
    if graph is not None:
        gev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
        for a, b in gev:
            flush_buf.zero_()
            a.record(stream)
            graph.replay()
            b.record(stream)
        barrier()
        graph_ms = [a.elapsed_time(b) for a, b in gev]
    # eager steps with the library's per-kernel events: the stage and kernel breakdown
    events = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    launches0 = lib.svo_kernel_launches()
    lib.svo_profile_enable(1)
    for a, b in events:
        flush_buf.zero_()
        a.record(stream)
        step()
        b.record(stream)
    barrier()
    launches = lib.svo_kernel_launches() - launches0
    profile = _lib.profile_summary()
    lib.svo_profile_enable(0)
    clocks = sampler.stop()
    eager_ms = [a.elapsed_time(b) for a, b in events]
    step_ms = graph_ms if graph_ms is not None else eager_ms
    ms = replicas.max_over_ranks(env, float(np.mean(step_ms)), device)

    # per-stage device time from the per-kernel events
    # stage times: each stage's calls timed alone with CUDA events on the stream (the per-kernel events
    # over-count where a stage's kernels overlap on two streams: the emissions, the bucket scan and
    # interior words beside the dense scans and the bucketed copy)
    def stage_time(fn, reps=10):
        fn()
        ts = []
        for _ in range(reps):
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            flush_buf.zero_()
            a.record(stream)
            fn()
            b.record(stream)
            torch.cuda.synchronize()
            ts.append(a.elapsed_time(b))
        return float(np.median(ts))

    def march_stage():
        tracer.CmdDrawPipeline(hits)
        if scene.bounce:
            api.OctreeTracer.Bounce(hits, scene.seed, bounce_rays)
            tracer.Trace(bounce_rays, bounce_hits)

    vox_ms = stage_time(vox.CmdVoxelize)
    build_ms = stage_time(builder.CmdBuild)
    march_ms = stage_time(march_stage)
    n_traced = n_rays * (2 if scene.bounce else 1)
    leaf_words = 8 if scene.level == 1 else 8 * info["level_nodes"][scene.level - 2]
    wl = {"fragments": F, "triangles": T, "level": scene.level, "rays": n_rays, "fetches_per_ray": fetches / n_rays,
          "range_words": info["range_words"], "leaf_words": leaf_words}
    peaks = load_peaks()
    # the dominant kernel among those with an algorithmic-byte count (the emissions overlap each other on
    # two streams, so their event intervals span each other's work and are no roofline basis)
    dom = max(((k, v) for k, v in profile.items() if algorithmic_bytes(k, wl) is not None), key=lambda kv: kv[1]["ms"])
    dom_name, dom_stats = dom[0], dom[1]
    dom_launch_ms = dom_stats["ms"] / dom_stats["launches"]
    alg = algorithmic_bytes(dom_name, wl)
    roofline = {"kernel": dom_name, "bound": "hbm", "unit": "GB/s", "peak": peaks["hbm_gbs"],
                "peak_source": peaks["source"], "launch_ms": dom_launch_ms,
                "share_of_step": dom_stats["ms"] / args.steps / ms}
    if alg is not None:
        ach = alg / (dom_launch_ms * 1e-3) / 1e9
        roofline.update({"achieved": ach, "frac": ach / peaks["hbm_gbs"], "algorithmic_bytes_per_launch": alg})
    roofline.update(profiled_traffic(dom_name, workload))
    mk = profile.get("march_camera")  # the primary march's own fraction, whichever kernel dominates
    march_frac = (algorithmic_bytes("march_camera", wl) / (mk["ms"] / mk["launches"] * 1e-3) / 1e9 / peaks["hbm_gbs"]
                  if mk and mk["ms"] > 0 else None)
    if dom_name.startswith("march"):
        roofline["limiter"] = ("instruction issue: node words stay in L1/L2, DRAM idle (ncu, "
                               "profiles/march_kernel_room_1024.md); the HBM fraction is low by construction")
        issue = issue_roofline(dom_name, workload, dom_launch_ms,
                               torch.cuda.get_device_properties(device).multi_processor_count,
                               clocks.get("sm_mhz") or clocks.get("sm_max_mhz"))
        if issue:
            roofline["issue"] = issue

    stages = {
        "voxelize_ms": vox_ms, "build_ms": build_ms, "march_ms": march_ms,
        "svo_build_ms": vox_ms + build_ms, "march_frac": march_frac,
        "mfragments_per_s": F / (vox_ms * 1e-3) / 1e6 if vox_ms else None,
        "grays_per_s": n_traced / (march_ms * 1e-3) / 1e9 if march_ms else None,
        "rays_traced_per_step": n_traced,
        "voxelize_gbs": (48.0 * T + 8.0 * F) / (vox_ms * 1e-3) / 1e9 if vox_ms else None,
        # the build's minimum traffic (each fragment read once, each node word written once) over its time
        "build_min_bytes_gbs": (8.0 * F + 4.0 * info["range_words"]) / (build_ms * 1e-3) / 1e9 if build_ms else None,
        "march_gbs": n_rays * (24.0 + 32.0 + 4.0 * fetches / n_rays) / (march_ms * 1e-3) / 1e9 if march_ms else None,
        "hit_fraction": float((hit_np["flags"] & 1).mean()), "mean_iterations": float(hit_np["iter"].mean()),
        "node_fetches_per_ray": fetches / n_rays, "octree_words": info["range_words"], "leaves": info["leaves"],
        "kernels": profile,
        "step_timing": "CUDA graph replay of the step" if graph_ms is not None else "eager launches",
        "eager_step_ms": float(np.mean(eager_ms)),
        "graph_step_ms": float(np.mean(graph_ms)) if graph_ms is not None else None,
        "graph_note": graph_note,
    }

    if light:
        return light_result(args, env, scene, F, T, n_rays, ms, stages, roofline, clocks, launches, vox, octree,
                            hits, bounce_hits, device)

    # the tracer's beam optimisation on the same frame: pre-pass + advanced primary march
    beam_img = tracer.CmdBeamRenderPass()
    hits_beam = tracer.CmdDrawPipelineBeam(beam_img)
    bev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True),
            torch.cuda.Event(enable_timing=True)) for _ in range(5)]
    for e0, e1, e2 in bev:
        flush_buf.zero_()
        e0.record(stream)
        tracer.CmdBeamRenderPass(beam_img)
        e1.record(stream)
        tracer.CmdDrawPipelineBeam(beam_img, hits_beam)
        e2.record(stream)
    torch.cuda.synchronize()
    hb = api.hits_numpy(hits_beam)
    beam = {"prepass_ms": float(np.median([a.elapsed_time(b) for a, b, _ in bev])),
            "march_ms": float(np.median([b.elapsed_time(c) for _, b, c in bev])),
            "mean_iterations": float(hb["iter"].mean()),
            "voxel_agreement_with_plain_march": float((hb["voxel"] == hit_np["voxel"]).all(axis=1).mean()),
            "texels": int(beam_img.numel())}
    beam["grays_per_s"] = n_rays / ((beam["prepass_ms"] + beam["march_ms"]) * 1e-3) / 1e9
    # the pre-pass and the march in one launch (the tracer's beam path when no beam image is given)
    hits_fused = tracer.CmdDrawPipelineBeam(None)
    fev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(5)]
    for e0, e1 in fev:
        flush_buf.zero_()
        e0.record(stream)
        tracer.CmdDrawPipelineBeam(None, hits_fused)
        e1.record(stream)
    torch.cuda.synchronize()
    beam["fused_ms"] = float(np.median([a.elapsed_time(b) for a, b in fev]))
    beam["fused_hits_equal_two_launch"] = bool(np.array_equal(api.hits_numpy(hits_fused), hb))
    stages["beam"] = beam
    if not args.no_path_trace:
        stages["path_trace"] = path_trace_stats(api, octree, scene, stream)

    e2e = None if args.no_e2e else e2e_arm(args, scene, tris_host, device, env)
    if e2e is not None:  # the host link bounds the copies of the end-to-end step
        link = host_link_probe(device)
        e2e["host_link"] = {**{k: link[k] for k in ("hit_store_gbs", "dma_d2h_gbs", "dma_h2d_gbs")},
                            "floor_ms": e2e["h2d_bytes_per_step"] / link["dma_h2d_gbs"] / 1e6 +
                                        e2e["d2h_bytes_per_step"] / link["hit_store_gbs"] / 1e6,
                            "note": "triangle upload at the DMA rate plus the hits at the march's host-store "
                                    "rate: the copies alone, before any voxelize or build work"}
    cpu = parity = None
    if env.leader and env.world == 1 and not args.no_cpu_baseline:
        # the timed steps' own outputs (the last step's fragment list, pool and hits), compared with the
        # oracle pass the CPU baseline times on the same scene
        ref = {}
        cpu = cpu_baseline(scene, per_step=False, outputs=ref)
        torch.cuda.synchronize()
        parity = parity_vs_oracle(vox.GetVoxelFragmentList(), octree.words(), api.hits_numpy(hits),
                                  api.hits_numpy(bounce_hits) if scene.bounce else None, ref, device)
        del ref
    return {"value": ms, "ms_per_step": ms, "step_ms_all": step_ms, "stages": stages, "roofline": roofline,
            "tuning": tuning,
            "clocks": clocks, "e2e": e2e, "cpu_baseline": cpu, "parity": parity, "gpu_launches": int(launches),
            "config_extra": {"level": scene.level, "triangles": T, "fragments": F, "rays": n_rays}}


def light_result(args, env, scene, F, T, n_rays, ms, stages, roofline, clocks, launches, vox, octree, hits,
                 bounce_hits, device) -> dict:
    """Result of a light engine_arm run, with the oracle comparison of its outputs when the CPU baseline
    leg runs (the oracle pass is timed as this workload's CPU baseline)."""
    import torch

    from sparsevoxeloctree_gb300 import api
    cpu = parity = None
    if env.leader and env.world == 1 and not args.no_cpu_baseline:
        ref = {}
        cpu = cpu_baseline(scene, per_step=False, outputs=ref, repeats=0)  # one pass: seconds at 2^12
        torch.cuda.synchronize()
        parity = parity_vs_oracle(vox.GetVoxelFragmentList(), octree.words(), api.hits_numpy(hits),
                                  api.hits_numpy(bounce_hits) if scene.bounce else None, ref, device)
        del ref
    st = {k: stages[k] for k in ("voxelize_ms", "build_ms", "march_ms", "svo_build_ms", "mfragments_per_s",
                                 "grays_per_s", "rays_traced_per_step", "node_fetches_per_ray", "octree_words",
                                 "hit_fraction", "step_timing")}
    st["kernels_ms_per_step"] = {k: round(v["ms"] / args.steps, 4) for k, v in stages["kernels"].items()}
    summary = {"step_ms": round(ms, 3), "grays_per_s": round(stages["grays_per_s"], 3),
               "svo_build_ms": round(stages["svo_build_ms"], 3),
               "march_frac": round(stages["march_frac"], 4) if stages["march_frac"] is not None else None,
               "dominant_kernel": roofline["kernel"], "dominant_frac": round(roofline.get("frac", 0.0), 4),
               "rays": stages["rays_traced_per_step"]}
    if parity:
        summary["parity"] = {"fragments": parity["fragments"], "octree": parity["octree"],
                             "hits_equal_frac": round(parity["hits_equal_frac"], 6),
                             "bounce_hits_equal_frac": round(parity.get("bounce_hits_equal_frac", 1.0), 6)}
    return {"workload": f"{scene.name}: {len(scene.tris)} triangles at level {scene.level}, "
                        f"{scene.width}x{scene.height} primary rays" + (" plus one diffuse bounce per hit"
                                                                        if scene.bounce else ""),
            "value": ms, "fragments": F, "stages": st, "roofline": roofline, "clocks": clocks,
            "gpu_launches": int(launches), "cpu_baseline": cpu, "parity": parity, "summary": summary}


def e2e_arm(args, scene, tris_host, device, env) -> dict:
    """The same step through the C ABI with host buffers: upload triangles from pinned memory, svo_voxelize
    (count pass, its blocking count readback, exact allocation, emit), svo_build (its blocking range
    readback), svo_raycast_camera_download (the march stores the hits straight into the pinned, mapped host
    buffer).  Scenes with a bounce: svo_raycast_camera + svo_bounce_rays + svo_raycast, one download."""
    import torch

    from sparsevoxeloctree_gb300 import _lib, api
    from sparsevoxeloctree_gb300.formats import HIT_DTYPE

    lib = _lib.load()
    n = scene.n_rays
    n_out = n * (2 if scene.bounce else 1)  # primary hits, then bounce hits
    hits_host = torch.empty(n_out * HIT_DTYPE.itemsize, dtype=torch.uint8).pin_memory()
    tris_dev = torch.empty_like(tris_host, device=device)
    hits_dev = torch.empty(n_out * HIT_DTYPE.itemsize, dtype=torch.uint8, device=device)
    rays_dev = torch.empty(n * 24, dtype=torch.uint8, device=device) if scene.bounce else None
    cam = api.camera_struct(scene.camera)
    s = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    T = len(scene.tris)

    def one():
        tris_dev.copy_(tris_host, non_blocking=True)
        fl = _lib.Fraglist()
        _lib.check(lib.svo_voxelize(ctypes.c_void_p(tris_dev.data_ptr()), T, scene.level, ctypes.byref(fl), s))
        oc = _lib.OctreeC()
        _lib.check(lib.svo_build_fraglist(ctypes.byref(fl), ctypes.byref(oc), None, s))
        if scene.bounce:  # the bounce rays start from the primary hits on the device
            _lib.check(lib.svo_raycast_camera(ctypes.byref(oc), ctypes.byref(cam), scene.width, scene.height,
                                              ctypes.c_void_p(hits_dev.data_ptr()), None, s))
            _lib.check(lib.svo_bounce_rays(ctypes.c_void_p(hits_dev.data_ptr()), n, scene.seed,
                                           ctypes.c_void_p(rays_dev.data_ptr()), s))
            _lib.check(lib.svo_raycast(ctypes.byref(oc), ctypes.c_void_p(rays_dev.data_ptr()), n,
                                       ctypes.c_void_p(hits_dev.data_ptr() + n * HIT_DTYPE.itemsize), None, s))
            hits_host.copy_(hits_dev, non_blocking=True)
        else:  # the hits stored into the pinned host buffer by the march itself (or copied in row bands)
            _lib.check(lib.svo_raycast_camera_download(ctypes.byref(oc), ctypes.byref(cam), scene.width,
                                                       scene.height, ctypes.c_void_p(hits_dev.data_ptr()),
                                                       ctypes.c_void_p(hits_host.data_ptr()), None, s))
        lib.svo_fraglist_destroy(ctypes.byref(fl), s)
        lib.svo_octree_destroy(ctypes.byref(oc), s)
        torch.cuda.current_stream().synchronize()

    for _ in range(args.warmup):
        one()
    torch.cuda.synchronize()
    replicas.barrier(env)
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        one()
        times.append((time.perf_counter() - t0) * 1e3)
    replicas.barrier(env)
    ms = replicas.max_over_ranks(env, float(statistics.mean(times)), device)
    return {"value": ms, "unit": "ms", "h2d_bytes_per_step": int(tris_host.numel()),
            "d2h_bytes_per_step": int(hits_host.numel()) + 8 * 3 + 256,
            "path": "svo_voxelize -> svo_build_fraglist -> svo_raycast_camera_download with pinned host buffers",
            "timing": "host wall clock per step (includes the ABI's blocking readbacks)"}


_HOST_LINK: dict = {}


def host_link_probe(device, width: int = 4096, height: int = 2048) -> dict:
    """GPU -> host bandwidth of this machine, the ceiling of every leg that delivers hits into host memory:
    svo_raycast_camera_download on an empty octree (every ray ends at its first node, so the kernel is
    ray set-up plus the 32 B hit store) into page-locked host memory, and a DMA copy of the same bytes
    (median of 5 after a warm-up; measured once per process)."""
    key = device.index if device.index is not None else 0
    if key in _HOST_LINK:
        return _HOST_LINK[key]
    import numpy as np
    import torch

    from sparsevoxeloctree_gb300 import _lib, api, scenes
    lib = _lib.load()
    n = width * height
    pool = torch.zeros(8, dtype=torch.int32, device=device)  # an empty root block
    oc = _lib.OctreeC()
    oc.words, oc.capacity, oc.range_words, oc.level, oc.owned = pool.data_ptr(), 8, 8, 3, 0
    cam = api.camera_struct(scenes.camera_from_angles((1.5, 1.5, 0.2), 0.0, 0.0, aspect=width / height))
    hits_dev = torch.empty(n * 32, dtype=torch.uint8, device=device)
    hits_host = torch.empty(n * 32, dtype=torch.uint8).pin_memory()
    st = torch.cuda.current_stream()
    s = ctypes.c_void_p(st.cuda_stream)

    def timed(fn, reps=5):
        fn()
        st.synchronize()
        ts = []
        for _ in range(reps):
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(st)
            fn()
            b.record(st)
            st.synchronize()
            ts.append(a.elapsed_time(b))
        return float(np.median(ts))

    store_ms = timed(lambda: _lib.check(lib.svo_raycast_camera_download(
        ctypes.byref(oc), ctypes.byref(cam), width, height, ctypes.c_void_p(hits_dev.data_ptr()),
        ctypes.c_void_p(hits_host.data_ptr()), None, s)))
    dma_ms = timed(lambda: hits_host.copy_(hits_dev, non_blocking=True))
    h2d_ms = timed(lambda: hits_dev.copy_(hits_host, non_blocking=True))
    out = {"bytes": n * 32, "hit_store_gbs": n * 32 / store_ms / 1e6, "dma_d2h_gbs": n * 32 / dma_ms / 1e6,
           "dma_h2d_gbs": n * 32 / h2d_ms / 1e6,
           "method": f"{width}x{height} camera rays on an empty octree, hits stored into page-locked host memory "
                     "by the march (svo_raycast_camera_download); DMA copies of the same bytes"}
    del hits_dev, hits_host, pool
    _HOST_LINK[key] = out
    return out


# ------------------------------------------------------------------------------------------ batched build
def path_trace_stats(api, octree, scene, stream, samples: int = 8) -> dict:
    """PathTracer::CmdRender on the step's octree and camera at the step's image size: device ms per sample
    (one sample per pixel, kDefaultBounce = 4 path vertices: the primary march, up to 3 diffuse bounces
    and, with the environment map, a shadow march per bounce), for the constant light and a seeded
    512x256 environment map with a sun."""
    import numpy as np
    import torch
    g = np.random.default_rng(11)
    env = np.zeros((256, 512, 4), np.float32)
    env[..., :3] = g.random((256, 512, 3), dtype=np.float32)
    env[60:64, 100:104, :3] = 200.0
    out = {"width": scene.width, "height": scene.height, "bounce": api.PathTracer.kDefaultBounce,
           "samples_timed": samples}
    for name, light_type in (("constant", 0), ("envmap", 1)):
        em = api.EnvironmentMap.Create()
        if light_type:
            em.Reset(env)
        light = api.Lighting.Create(em)
        light.m_light_type = light_type
        pt = api.PathTracer.Create(octree, scene.camera, light)
        pt.m_width, pt.m_height = scene.width, scene.height
        pt.Reset()
        pt.CmdRender(stream, samples=2)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        pt.CmdRender(stream, samples=samples)
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / samples
        col = pt.ExtractColorImage()
        out[name] = {"ms_per_sample": ms, "msamples_per_s": scene.width * scene.height / (ms * 1e-3) / 1e6,
                     "mean_radiance": float(col.mean()), "status": pt.GetStatus()}
    return out


def batch_leg(args, device, meshes=None, workload: str | None = None, check_identity: bool = False) -> dict:
    """The batched-build workload: 64 clutter meshes (triangles log-uniform in [1e3, 5e5], levels 7..10)
    voxelized and built (a) in one svo_batcher batch (one count pass, one readback of the counts, one
    recorded launch sequence for emit + every build level over all meshes, one readback of the results)
    and (b) as 64 sequential plain builds through the C ABI (svo_voxelize + svo_build_fraglist per mesh,
    each with its own two blocking readbacks).  Triangles are resident in HBM for both; both are timed on
    the host wall clock per whole batch, blocking readbacks included."""
    import numpy as np
    import torch

    from sparsevoxeloctree_gb300 import _lib, api, scenes

    lib = _lib.load()
    if meshes is None:
        meshes = scenes.batch_64()
        workload = "batch_64: 64 clutter meshes, triangles log-uniform in [1e3, 5e5] (seeded), levels 7..10"
    tris = [api.to_device(t) for t, _ in meshes]
    s = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    bb = api.BatchBuilder(use_graph=True)
    batch = [(t, level) for t, (_, level) in zip(tris, meshes)]

    def batched():
        bb.Build(batch)

    def sequential():
        for t, (_, level) in zip(tris, meshes):
            fl = _lib.Fraglist()
            _lib.check(lib.svo_voxelize(ctypes.c_void_p(t.data_ptr()), t.numel() // 48, level, ctypes.byref(fl), s))
            oc = _lib.OctreeC()
            _lib.check(lib.svo_build_fraglist(ctypes.byref(fl), ctypes.byref(oc), None, s))
            lib.svo_fraglist_destroy(ctypes.byref(fl), s)
            lib.svo_octree_destroy(ctypes.byref(oc), s)
        torch.cuda.current_stream().synchronize()

    def timed(fn, reps):
        for _ in range(args.warmup):
            fn()
        torch.cuda.synchronize()
        out = []
        for _ in range(reps):
            t0 = time.perf_counter()
            fn()
            out.append((time.perf_counter() - t0) * 1e3)
        return out

    batched()  # first build: records the graphs
    tuning = None
    if not args.no_autotune:
        from sparsevoxeloctree_gb300 import autotune
        F0 = sum(bb.GetInfo(i)["fragments"] for i in range(len(meshes)))
        tr = autotune.tune_batch(bb, batch, F0, sum(len(t) for t, _ in meshes))
        tuning = {k: {"best": v["best"], "best_ms": v["best_ms"], "level": v["level"], "size_class": v["size_class"]}
                  for k, v in tr.items()}
    reps = max(3, min(args.steps, 10))
    launches0 = lib.svo_kernel_launches()
    b_ms = timed(batched, reps)
    seq_ms = timed(sequential, reps)
    F = sum(bb.GetInfo(i)["fragments"] for i in range(len(meshes)))
    W = sum(bb.GetInfo(i)["range_words"] for i in range(len(meshes)))
    T = sum(len(t) for t, _ in meshes)
    # device time of one batch (count graph + build graph), profiled launches excluded: CUDA events around
    # a Build on the current stream
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record()
    batched()
    ev1.record()
    torch.cuda.synchronize()
    dev_ms = ev0.elapsed_time(ev1)
    # per-kernel device times of one batch, launches issued directly (no graph) with events around each
    prof_bb = api.BatchBuilder(use_graph=False)
    prof_bb.Build(batch)
    torch.cuda.synchronize()
    lib.svo_profile_enable(1)
    prof_bb.Build(batch)
    kernels = _lib.profile_summary()
    lib.svo_profile_enable(0)
    del prof_bb
    identical = None
    if check_identity:  # every mesh's octree from the batch equals its plain build's, word for word
        identical = True
        bb.Build(batch)
        for i, (t, (_, level)) in enumerate(zip(tris, meshes)):
            fl = _lib.Fraglist()
            _lib.check(lib.svo_voxelize(ctypes.c_void_p(t.data_ptr()), t.numel() // 48, level, ctypes.byref(fl), s))
            oc = _lib.OctreeC()
            _lib.check(lib.svo_build_fraglist(ctypes.byref(fl), ctypes.byref(oc), None, s))
            plain = api._copy_from(oc.words, oc.range_words, torch.int32)
            identical &= bool(torch.equal(plain, bb.GetOctree(i).words()))
            del plain
            lib.svo_fraglist_destroy(ctypes.byref(fl), s)
            lib.svo_octree_destroy(ctypes.byref(oc), s)
        torch.cuda.synchronize()
    peaks = load_peaks()
    alg = 48.0 * T + 40.0 * F + 4.0 * W
    bm, sm = float(np.median(b_ms)), float(np.median(seq_ms))
    frac = alg / (bm * 1e-3) / 1e9 / peaks["hbm_gbs"]
    return {"workload": workload, "summary": {"batched_ms": round(bm, 3), "sequential_ms": round(sm, 3),
                                              "speedup": round(sm / bm, 3), "frac": round(frac, 4),
                                              "bit_identical_to_plain": identical},
            "meshes": len(meshes), "triangles": T, "fragments": F, "octree_words": W,
            "batched_ms": bm, "sequential_plain_ms": sm, "speedup_vs_sequential": sm / bm,
            "batched_mfragments_per_s": F / (bm * 1e-3) / 1e6,
            "sequential_mfragments_per_s": F / (sm * 1e-3) / 1e6,
            "batched_device_ms": dev_ms,
            "roofline": {"bound": "hbm", "algorithmic_bytes": alg,
                         "bytes_formula": "48 B/triangle + 40 B/fragment (8 emit, 16 two sweeps, 8 bucketed copy, "
                                          "8 leaf sweep) + 4 B/node word",
                         "achieved_gbs": alg / (bm * 1e-3) / 1e9, "peak": peaks["hbm_gbs"],
                         "frac": alg / (bm * 1e-3) / 1e9 / peaks["hbm_gbs"]},
            "graph": bb.stats(), "timing": "host wall clock per batch (median), blocking readbacks included",
            "kernels_one_batch": kernels, "autotuned": tuning,
            "reps": reps, "kernel_launches_recorded": int(lib.svo_kernel_launches() - launches0)}


# ------------------------------------------------------------------------------------------ serving
def serve_leg(args, device, rates=(100, 200, 500, 1000, 2000, 5000), seconds=1.0) -> dict:
    """The serving workload: 16 resident octrees (levels 9..11, sphere + boxes + clutter meshes of 50k..2M
    triangles), trace requests with a uniform scene and a log-uniform ray count of 1k..2M (half primary
    camera rays, half diffuse-bounce rays), 2% rebuilds, admission under a 40 GB HBM budget.  Poisson
    arrivals at each rate for `seconds`; latency = server submit -> completion (p50/p99); throughput =
    rays / (last completion - first submission).  Saturation: every request of a set submitted at once.
    One at a time: the same set through the plain C ABI calls (svo_raycast_camera, svo_bounce_rays,
    svo_raycast, hit download, synchronize) one request after another, and through the server with one
    lane and one request per batch."""
    import math
    import threading

    import numpy as np
    import torch

    from sparsevoxeloctree_gb300 import _lib, api, scenes
    from sparsevoxeloctree_gb300.formats import HIT_DTYPE

    lib = _lib.load()
    meshes = scenes.serving_scenes()
    server = api.Server(hbm_budget_bytes=40 << 30, lanes=3)
    tris_dev = [api.to_device(t) for t, _ in meshes]
    octs = []
    for t, (_, level) in zip(tris_dev, meshes):
        octs.append(server.BuildScene(t, level))
    torch.cuda.synchronize()
    g = scenes.rng(55, 0)

    def make_request(k):
        n_rays = int(round(math.exp(g.uniform(math.log(1e3), math.log(2e6)))))
        n = max(1, n_rays // 2)
        w = min(n, 2048)
        h = (n + w - 1) // w
        pos = (float(g.uniform(0.2, 0.8)), float(g.uniform(0.2, 0.8)), float(g.uniform(0.2, 0.8)))
        cam = scenes.camera_from_angles(tuple(p + 1.0 for p in pos), float(g.uniform(0, 2 * math.pi)),
                                        float(g.uniform(-0.3, 0.3)), aspect=w / h)
        return {"scene": int(g.integers(0, len(octs))), "cam": cam, "w": w, "h": h, "n": n,
                "seed": int(g.integers(0, 2**62)), "rebuild": bool(g.uniform() < 0.02)}

    # pinned hit buffers the client reuses: 20 for up to 2M hits, 64 for up to 64k hits
    slot_bytes = 2 * (1 << 20) * HIT_DTYPE.itemsize
    small_bytes = (1 << 16) * HIT_DTYPE.itemsize
    bufs = [torch.empty(slot_bytes, dtype=torch.uint8).pin_memory() for _ in range(20)]
    bufs += [torch.empty(small_bytes, dtype=torch.uint8).pin_memory() for _ in range(64)]
    big_ids, small_ids = list(range(20)), list(range(20, 84))

    def run(reqs, arrivals):
        """Submit reqs at the given arrival offsets (seconds; None = all at once); returns per-request results."""
        free = {True: list(big_ids), False: list(small_ids)}
        cv = threading.Condition()
        out = [None] * len(reqs)
        tickets = []
        done_flag = {"n": 0}

        def collector():
            for i, (t, slot, rb) in enumerate(iter(tickets_q.get, None)):
                res = server.Wait(t)
                out[t_index[t]] = res
                with cv:
                    if slot is not None:
                        free[slot < 20].append(slot)
                    done_flag["n"] += 1
                    cv.notify_all()

        import queue
        tickets_q = queue.Queue()
        t_index = {}
        th = threading.Thread(target=collector, daemon=True)
        th.start()
        t0 = time.perf_counter()
        for i, r in enumerate(reqs):
            if arrivals is not None:
                delay = t0 + arrivals[i] - time.perf_counter()
                if delay > 0:
                    time.sleep(delay)
            if r["rebuild"]:
                sc = r["scene"]
                t = server.SubmitRebuild(octs[sc], tris_dev[sc], meshes[sc][1])
                t_index[t] = i
                tickets_q.put((t, None, True))
                continue
            big = 2 * r["n"] * HIT_DTYPE.itemsize > small_bytes
            with cv:
                while not free[big]:
                    cv.wait()
                slot = free[big].pop()
            t = server.SubmitCamera(octs[r["scene"]], r["cam"], r["w"], r["h"], r["n"], r["seed"], bufs[slot])
            t_index[t] = i
            tickets_q.put((t, slot, False))
        tickets_q.put(None)
        th.join()
        return out

    def summarize(reqs, res):
        lat = [x["done_us"] - x["submit_us"] for x, r in zip(res, reqs) if not r["rebuild"]]
        rays = sum(2 * r["n"] for r in reqs if not r["rebuild"])
        span = (max(x["done_us"] for x in res) - min(x["submit_us"] for x in res)) * 1e-6
        bs = [x["batch_requests"] for x, r in zip(res, reqs) if not r["rebuild"]]
        return {"requests": len(reqs), "rebuilds": sum(r["rebuild"] for r in reqs), "rays": rays,
                "p50_ms": float(np.percentile(lat, 50)) / 1e3, "p99_ms": float(np.percentile(lat, 99)) / 1e3,
                "grays_per_s": rays / span / 1e9, "mean_batch_requests": float(np.mean(bs))}

    # warm-up: one request per scene
    run([dict(make_request(0), scene=i, rebuild=False) for i in range(len(octs))], None)
    sweep = {}
    for lam in rates:
        n_req = max(20, int(lam * seconds))
        reqs = [make_request(k) for k in range(n_req)]
        arrivals = np.cumsum(g.exponential(1.0 / lam, size=n_req))
        sweep[str(lam)] = summarize(reqs, run(reqs, arrivals))
    sat_reqs = [dict(make_request(k), rebuild=False) for k in range(400)]
    saturated = summarize(sat_reqs, run(sat_reqs, None))

    # one request at a time, plain C ABI.  The sweep's rebuilds replaced scenes' octrees (and freed the old
    # ones once their batches retired): take fresh views of the current octrees.
    views = [server.Scene(i) for i in octs]
    one_reqs = sat_reqs[:150]
    s = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    hits_dev = torch.empty(slot_bytes, dtype=torch.uint8, device=device)
    full_dev = torch.empty(2048 * 1024 * HIT_DTYPE.itemsize, dtype=torch.uint8, device=device)
    rays_dev = torch.empty((1 << 20) * 24, dtype=torch.uint8, device=device)

    def plain_one(r):
        oc = views[r["scene"]].c_struct()
        cam = api.camera_struct(r["cam"])
        n = r["n"]
        _lib.check(lib.svo_raycast_camera(ctypes.byref(oc), ctypes.byref(cam), r["w"], r["h"],
                                          ctypes.c_void_p(full_dev.data_ptr()), None, s))
        _lib.check(lib.svo_bounce_rays(ctypes.c_void_p(full_dev.data_ptr()), n, r["seed"],
                                       ctypes.c_void_p(rays_dev.data_ptr()), s))
        _lib.check(lib.svo_raycast(ctypes.byref(oc), ctypes.c_void_p(rays_dev.data_ptr()), n,
                                   ctypes.c_void_p(hits_dev.data_ptr() + n * 32), None, s))
        _lib.check(lib.svo_download(ctypes.c_void_p(bufs[0].data_ptr()), ctypes.c_void_p(full_dev.data_ptr()),
                                    n * 32, 0, s))
        _lib.check(lib.svo_download(ctypes.c_void_p(bufs[0].data_ptr() + n * 32),
                                    ctypes.c_void_p(hits_dev.data_ptr() + n * 32), n * 32, 1, s))

    for r in one_reqs[:5]:
        plain_one(r)
    t0 = time.perf_counter()
    for r in one_reqs:
        plain_one(r)
    plain_s = time.perf_counter() - t0
    one_rays = sum(2 * r["n"] for r in one_reqs)
    one_server = api.Server(hbm_budget_bytes=40 << 30, lanes=1, max_batch_requests=1)
    server_main = server
    for v in views:
        one_server.AddOctree(v)
    server = one_server
    one_res = summarize(one_reqs, run(one_reqs, None))
    server = server_main
    one_server.close()

    # roofline of the served march.  Bytes per ray: 32 B hit out, 4 B per node word read, and 24 B ray in
    # for the bounce half (camera rays are made in the kernel).  The node words are counted by a second
    # server over the same resident octrees (counting costs the march ~7%, so the first server does not
    # count), on the saturated request set with the library's per-launch events on; the delivered rate
    # is the uncounted saturated run's.
    roof_server = api.Server(hbm_budget_bytes=40 << 30, lanes=3, count_fetches=True)
    for v in views:
        roof_server.AddOctree(v)
    server = roof_server
    lib.svo_profile_enable(1)
    prof_sum = summarize(sat_reqs, run(sat_reqs, None))
    prof = _lib.profile_summary()
    lib.svo_profile_enable(0)
    fetches = roof_server.stats()["node_fetches"]
    server = server_main
    roof_server.close()
    rays = prof_sum["rays"]
    bytes_per_ray = (32.0 * rays + 4.0 * fetches + 24.0 * (rays / 2)) / rays
    mj = prof.get("march_jobs", {"ms": 0.0, "launches": 0})
    peaks = load_peaks()
    delivered = saturated["grays_per_s"] * 1e9 * bytes_per_ray / 1e9
    roof = {"bound": "hbm", "unit": "GB/s", "peak": peaks["hbm_gbs"], "peak_source": peaks["source"],
            "rays": rays, "node_fetches_per_ray": fetches / rays, "bytes_per_ray": bytes_per_ray,
            "march_launches": mj["launches"], "launch_ms": mj["ms"] / max(mj["launches"], 1),
            "achieved": delivered, "frac": delivered / peaks["hbm_gbs"],
            "formula": "saturated Grays/s x bytes per ray; bytes per ray = 32 B hit + 24 B ray for the bounce "
                       "half + 4 B x node words read (counted on the same 400 requests by a counting server)",
            "kernels": {k: {"ms": round(v["ms"], 3), "launches": v["launches"]} for k, v in prof.items()}}
    # every served hit is delivered into the client's page-locked host memory: the GPU -> host link is the
    # ceiling the delivered hit bytes are measured against
    link = host_link_probe(device)
    hit_gbs = saturated["grays_per_s"] * 32.0
    roof["host_link"] = {"delivered_hit_gbs": hit_gbs, "hit_store_gbs": link["hit_store_gbs"],
                         "frac": hit_gbs / link["hit_store_gbs"], "ceiling_grays_per_s": link["hit_store_gbs"] / 32.0}
    served_sat = summarize(one_reqs, run(one_reqs, None))
    st = server.stats()
    server.close()
    return {"workload": "serving: 16 resident octrees (levels 9..11, 50k..2M triangles, seeded), requests of "
                        "1k..2M rays (log-uniform; half primary, half diffuse bounce), 2% rebuilds, 40 GB budget",
            "resident_bytes": st["resident_bytes"], "scenes_triangles": int(sum(len(t) for t, _ in meshes)),
            "poisson": sweep, "saturated_400": saturated, "roofline": roof,
            "same_150_requests": {"served_grays_per_s": served_sat["grays_per_s"],
                                  "one_at_a_time_plain_abi_grays_per_s": one_rays / plain_s / 1e9,
                                  "one_at_a_time_server_grays_per_s": one_res["grays_per_s"],
                                  "speedup_vs_plain_abi": served_sat["grays_per_s"] / (one_rays / plain_s / 1e9),
                                  "speedup_vs_unbatched_server": served_sat["grays_per_s"] / one_res["grays_per_s"],
                                  "served_p50_ms": served_sat["p50_ms"], "served_p99_ms": served_sat["p99_ms"]},
            "server_stats": st, "lanes": 3,
            "latency": "server clock, submission to completion of the request's hits in host memory"}


# ------------------------------------------------------------------------------------------ CPU arms
def cpu_model() -> str:
    """The host CPU as /proc/cpuinfo names it (x86: model name; Arm: implementer and part numbers)."""
    try:
        with open("/proc/cpuinfo") as f:
            info = f.read().splitlines()
    except OSError:
        return "unknown"
    fields = {}
    for line in info:
        if ":" in line:
            k, v = (x.strip() for x in line.split(":", 1))
            fields.setdefault(k, v)
    if "model name" in fields:
        return fields["model name"]
    if "CPU part" in fields:
        return f"Arm implementer {fields.get('CPU implementer', '?')} part {fields['CPU part']}"
    return "unknown"


def cpu_baseline(scene, per_step: bool, outputs: dict | None = None, repeats: int = 3) -> dict:
    """The oracle (CPU restatement of the reference's path) on the host cores, full workload: one
    warm-up pass, then the median of `repeats` timed passes per stage (repeats = 0: the one pass is the
    measurement).  With `outputs` (a dict), the first pass's fragment list, node pool and hits are stored
    there for the parity comparison with the engine's outputs of the same workload."""
    import statistics

    import oracle

    def one_pass():
        t0 = time.perf_counter()
        frags = oracle.voxelize(scene.tris, scene.level)
        t1 = time.perf_counter()
        pool = oracle.build_octree(frags, scene.level)
        t2 = time.perf_counter()
        rays = oracle.camera_rays(scene.camera, scene.width, scene.height)
        hits = oracle.raycast(pool, scene.level, rays)
        bounce_hits = None
        if scene.bounce:
            bounce_hits = oracle.raycast(pool, scene.level, oracle.bounce_rays(hits, scene.seed))
        t3 = time.perf_counter()
        times = {"voxelize": (t1 - t0) * 1e3, "build": (t2 - t1) * 1e3, "march": (t3 - t2) * 1e3,
                 "total": (t3 - t0) * 1e3}
        return times, (frags, pool, hits, bounce_hits)

    cold, (frags, pool, hits, bounce_hits) = one_pass()
    if outputs is not None:
        outputs.update(frags=frags, pool=pool, hits=hits, bounce_hits=bounce_hits)
    nfrags = int(len(frags))
    del frags, pool, hits, bounce_hits
    runs = [one_pass()[0] for _ in range(repeats)] or [cold]
    med = {k: statistics.median(r[k] for r in runs) for k in ("voxelize", "build", "march", "total")}
    how = f"one warm-up pass, then the median of {len(runs)} passes" if repeats else "one pass"
    return {"value": med["total"], "unit": "ms", "cores": oracle.threads(), "kind": "port",
            "cpu": cpu_model(), "hardware_threads": os.cpu_count(),
            "sample": f"full {scene.name} workload ({len(scene.tris)} tris, {nfrags} fragments, {scene.n_rays} "
                      f"rays): {how}",
            "fragments": nfrags, "cold_ms": cold["total"],
            "stages_ms": {k: med[k] for k in ("voxelize", "build", "march")}}


def parity_vs_oracle(frags_dev, pool_dev, hits_np, bounce_np, ref: dict, device) -> dict:
    """The engine's outputs of the timed workload against the oracle's on the same scene: the fragment
    multisets (both lists sorted on the device), the node pools word for word (canonical breadth-first
    order on both sides), and every ray's hit field by field; plus the tolerance the engine promises
    (voxel id on >= 99.99% of rays, |dt| <= 1e-5 of the extent)."""
    import numpy as np
    import torch
    rf = torch.from_numpy(np.ascontiguousarray(ref["frags"]).view(np.int64)).to(device)
    ef = frags_dev.view(torch.int64)
    frags_ok = ef.numel() == rf.numel() and bool(torch.equal(torch.sort(ef)[0], torch.sort(rf)[0]))
    rp = torch.from_numpy(np.ascontiguousarray(ref["pool"]).view(np.int32)).to(device)
    ep = pool_dev.view(torch.int32)
    pool_ok = ep.numel() == rp.numel() and bool(torch.equal(ep, rp))
    del rf, rp

    def hit_stats(got, want):
        same = np.ones(len(want), bool)
        for f in want.dtype.names:
            same &= (got[f] == want[f]).reshape(len(want), -1).all(axis=1)
        voxel = (got["voxel"] == want["voxel"]).all(axis=1) & ((got["flags"] & 1) == (want["flags"] & 1))
        both = (got["flags"] & 1).astype(bool) & (want["flags"] & 1).astype(bool)
        dt = float(np.abs(got["t"][both] - want["t"][both]).max()) if both.any() else 0.0
        return float(same.mean()), float(voxel.mean()), dt

    eq, vox, dt = hit_stats(hits_np, ref["hits"])
    out = {"fragments": frags_ok, "fragment_count": int(ef.numel()), "octree": pool_ok, "octree_words": int(ep.numel()),
           "hits_equal_frac": eq, "hits_voxel_frac": vox, "max_abs_dt": dt, "rays": int(len(hits_np))}
    if bounce_np is not None and ref.get("bounce_hits") is not None:
        beq, bvox, bdt = hit_stats(bounce_np, ref["bounce_hits"])
        out.update({"bounce_hits_equal_frac": beq, "bounce_hits_voxel_frac": bvox, "bounce_max_abs_dt": bdt})
    out["within_tolerance"] = bool(frags_ok and pool_ok and vox >= 0.9999 and dt <= 1e-5 and
                                   out.get("bounce_hits_voxel_frac", 1.0) >= 0.9999)
    return out


def reference_arm(args, rank: int) -> dict | None:
    if rank != 0:
        return None
    import oracle
    scene = make_scene(args.workload)
    for _ in range(args.warmup):
        cpu_baseline(scene, True, repeats=0)
    runs = [cpu_baseline(scene, True, repeats=0) for _ in range(args.steps)]
    ms = float(statistics.mean(r["value"] for r in runs))
    cpu = dict(runs[-1])
    cpu["value"] = ms
    return {"value": ms, "ms_per_step": ms, "cpu_baseline": cpu,
            "e2e": {"value": ms, "unit": "ms", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "config_extra": {"level": scene.level, "triangles": len(scene.tris), "fragments": cpu["fragments"],
                             "rays": scene.n_rays}}


# ------------------------------------------------------------------------------------------ main
def summary_block(line: dict) -> dict:
    """Compact copy of the headline figures, printed as the line's last key so that a reader who keeps
    only the end of the output still sees them: parity against the oracle, the batched and served
    speed-ups with their roofline fractions, and served latency per arrival rate."""
    def r(x, n=4):
        return None if x is None else round(float(x), n)
    e2e_link = (line.get("e2e") or {}).get("host_link") or {}
    out = {"step_ms": r(line.get("value")), "e2e_ms": r((line.get("e2e") or {}).get("value")),
           "e2e_copy_floor_ms": r(e2e_link.get("floor_ms")),
           "march_frac": r(line["roofline"].get("frac"))}
    if line["roofline"].get("issue"):
        out["march_issue_frac"] = r(line["roofline"]["issue"]["frac"])
    p = line.get("parity")
    if p:
        out["parity"] = {"fragments": p["fragments"], "octree": p["octree"], "hits_equal_frac": r(p["hits_equal_frac"], 6)}
    b = line.get("batched")
    if b:
        out["batched_speedup"] = r(b["speedup_vs_sequential"], 3)
        out["batched_frac"] = r(b["roofline"]["frac"])
        out["batched_ms"] = r(b["batched_ms"], 3)
    sv = line.get("served")
    if sv:
        same = sv["same_150_requests"]
        out["served_speedup"] = r(same["speedup_vs_plain_abi"], 3)
        out["served_speedup_vs_unbatched"] = r(same["speedup_vs_unbatched_server"], 3)
        out["served_grays_per_s"] = r(sv["saturated_400"]["grays_per_s"], 3)
        if sv.get("roofline"):
            out["served_frac"] = r(sv["roofline"]["frac"])
            out["served_march_launch_ms"] = r(sv["roofline"]["launch_ms"])
            if "host_link" in sv["roofline"]:
                out["served_host_link_frac"] = r(sv["roofline"]["host_link"]["frac"])
        out["served_p50_p99_ms"] = {k: [r(v["p50_ms"], 3), r(v["p99_ms"], 3)] for k, v in sv["poisson"].items()}
    for key in ("large", "large_batched"):
        if line.get(key):
            out[key] = line[key].get("summary")
    return out


def main() -> int:
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["engine", "reference"], default="engine")
    ap.add_argument("--workload", choices=sorted(WORKLOADS), default="room_1024")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-batch", action="store_true", help="skip the batched-build leg")
    ap.add_argument("--no-serve", action="store_true", help="skip the serving leg")
    ap.add_argument("--no-autotune", action="store_true", help="default launch parameters")
    ap.add_argument("--no-path-trace", action="store_true", help="skip the path-tracer statistics")
    ap.add_argument("--no-large", action="store_true",
                    help="skip the 2^12 legs (plain 4M-triangle step; 10M triangles as 4 batched meshes)")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)

    env = replicas.replica_env()

    line = {"metric": METRIC, "unit": "ms", "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "fp32+u32",
            "data": "synthetic (seeded scene with the benchmark configuration's shapes; the reference's OBJ "
                    "scenes are not available)"}
    config = {"workload": f"{args.workload}: {WORKLOADS[args.workload]}",
              "step": "voxelize (count+emit) + octree build + primary-ray march, recorded once as a CUDA graph "
                      "and replayed (stages: eager steps with per-kernel events)",
              "l2": f"flushed between timed steps ({L2_FLUSH_BYTES >> 20} MiB write); fragment list and node "
                    "pool exceed L2", "parallelism": env.parallelism}

    if args.impl == "reference":
        res = reference_arm(args, env.rank)
        if res is None:
            return 0
        line.update({"impl": "reference", "value": res["value"], "ms_per_step": res["ms_per_step"],
                     "cpu_baseline": res["cpu_baseline"], "e2e": res["e2e"], "gpu_launches": 0})
        config.update(res["config_extra"])
        line["config"] = config
        print(json.dumps(line), flush=True)
        return 0

    import torch
    device = torch.device("cuda", env.local_rank)
    torch.cuda.set_device(device)
    replicas.init(env, "nccl")
    res = engine_arm(args, env, device)
    if not args.no_batch and env.leader:
        res["batched"] = batch_leg(args, device)
    if not args.no_serve and env.leader:
        res["served"] = serve_leg(args, device)
    if not args.no_large and env.leader:
        # the 2^12 configuration: one 4M-triangle octree (the largest the 30-bit pointer format holds) with
        # primary and bounce rays, and the full 10M triangles as its 4 clustered groups in one batch
        torch.cuda.empty_cache()
        res["large"] = engine_arm(args, env, device, workload="clusters_4096_4m", light=True)
        torch.cuda.empty_cache()
        from sparsevoxeloctree_gb300 import scenes
        res["large_batched"] = batch_leg(
            args, device, meshes=scenes.clusters_4096_groups(),
            workload="clusters_4096_groups: the 10M-triangle 4-cluster scene as 4 meshes (one per group, "
                     "~2.5M triangles each) at level 12, one batch vs 4 sequential plain builds",
            check_identity=True)
    config.update(res["config_extra"])
    line.update({"value": res["value"], "ms_per_step": res["ms_per_step"], "config": config,
                 "stages": res["stages"], "roofline": res["roofline"], "cpu_baseline": res["cpu_baseline"],
                 "e2e": res["e2e"], "clocks": res["clocks"], "gpu_launches": res["gpu_launches"],
                 "step_ms": res["step_ms_all"], "autotuned": res["tuning"]})
    for key in ("batched", "served", "large", "large_batched"):
        if key in res:
            line[key] = res[key]
    if res.get("parity") is not None:
        line["parity"] = res["parity"]
    # last: the figures a reader of the line's tail needs, compact
    line["summary"] = summary_block(line)
    if env.leader:
        print(json.dumps(line), flush=True)
    replicas.finish(env)
    return 0


if __name__ == "__main__":
    sys.exit(main())
