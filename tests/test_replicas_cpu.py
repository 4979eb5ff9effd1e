"""The multi-GPU path is replicas only: every rank runs the whole voxelize -> build -> march step on its own
scene copy, with no collective on the data path.  These tests run that host-side protocol on CPU with two
gloo ranks (the timing barrier, the max over ranks, rank-0-only output) and the replicas' work as the
oracle's pipeline, and launch bench.py's reference arm the way a two-GPU run launches it.  No GPU needed."""
import json
import os
import socket
import subprocess
import sys
import zlib

import numpy as np
import pytest

from sparsevoxeloctree_gb300 import replicas

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port() -> int:
    with socket.socket(socket.AF_INET, socket.SOCK_STREAM) as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _replica_step(seed: int) -> int:
    """One replica's step on the oracle: voxelize a seeded scene, build its octree, march 16x16 primary rays;
    returns a checksum of the fragments, the node pool and the hits."""
    import oracle
    from sparsevoxeloctree_gb300 import scenes

    verts = np.concatenate([scenes.icosphere(1, 0.3, (0.5, 0.5, 0.5)),
                            scenes.clutter(scenes.rng(seed, 1), 40, np.log(0.05), 0.5)], 0)
    tris = scenes._soup(verts, scenes.random_colors(scenes.rng(seed, 2), len(verts)))
    level = 6
    frags = oracle.voxelize(tris, level)
    pool = oracle.build_octree(frags, level)
    cam = scenes.camera_from_angles((1.5, 1.5, 0.6), 0.05, 0.02)
    hits = oracle.raycast(pool, level, oracle.camera_rays(cam, 16, 16))
    crc = zlib.crc32(frags.tobytes())
    crc = zlib.crc32(oracle.canonicalize(pool).tobytes(), crc)
    return zlib.crc32(hits.tobytes(), crc)


def _rank_main(rank: int, world: int, port: int, out_dir: str) -> None:
    os.environ.update({"MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    env = replicas.replica_env({"RANK": str(rank), "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank)})
    replicas.init(env, "gloo")
    try:
        replicas.barrier(env)
        crc = _replica_step(seed=11)  # every replica runs the same workload
        replicas.barrier(env)
        step_ms = 1.5 + 2.0 * rank  # each rank's own mean step time
        job_ms = replicas.max_over_ranks(env, step_ms)
        crcs = replicas.gather(env, crc)
        ranks = replicas.gather(env, env.rank)
        if env.leader:  # rank 0 alone writes the result line
            with open(os.path.join(out_dir, "line.json"), "w") as f:
                json.dump({"job_ms": job_ms, "crcs": crcs, "ranks": ranks, "parallelism": env.parallelism,
                           "crc_local": _replica_step(seed=11)}, f)
        with open(os.path.join(out_dir, f"rank{rank}.json"), "w") as f:
            json.dump({"job_ms": job_ms}, f)
    finally:
        replicas.finish(env)


def test_replica_env_parsing():
    env = replicas.replica_env({})
    assert (env.rank, env.world, env.local_rank, env.leader) == (0, 1, 0, True)
    assert env.parallelism == "single GPU"
    env = replicas.replica_env({"RANK": "1", "WORLD_SIZE": "4", "LOCAL_RANK": "1"})
    assert not env.leader and env.parallelism == "replicas x4"
    for bad in ({"RANK": "2", "WORLD_SIZE": "2"}, {"WORLD_SIZE": "0"}, {"RANK": "-1", "WORLD_SIZE": "2"},
                {"LOCAL_RANK": "-1"}):
        with pytest.raises(ValueError):
            replicas.replica_env(bad)
    # one replica: the protocol is the identity and needs no process group
    assert replicas.max_over_ranks(replicas.replica_env({}), 2.5) == 2.5
    assert replicas.gather(replicas.replica_env({}), 7) == [7]
    replicas.barrier(replicas.replica_env({}))


def test_two_gloo_replicas(tmp_path):
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp

    import oracle
    oracle.build()  # compile the oracle once, before the ranks load it
    world = 2
    mp.start_processes(_rank_main, args=(world, _free_port(), str(tmp_path)), nprocs=world, join=True,
                       start_method="spawn")
    line = json.loads((tmp_path / "line.json").read_text())
    assert line["job_ms"] == 3.5  # the slowest replica's time
    assert line["ranks"] == [0, 1]
    assert line["crcs"][0] == line["crcs"][1] == line["crc_local"]  # replicas are independent and identical
    assert line["parallelism"] == "replicas x2"
    for r in range(world):  # every rank received the same job time
        assert json.loads((tmp_path / f"rank{r}.json").read_text())["job_ms"] == 3.5
    del torch


def test_bench_reference_arm_two_ranks():
    """`torchrun --nproc-per-node 2 bench.py --impl reference`: rank 0 alone measures and prints one line; the
    other rank exits 0 without work."""
    pytest.importorskip("torch")
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(_free_port()), os.path.join(ROOT, "bench.py"),
           "--impl", "reference", "--workload", "plain_256", "--gpus", "2", "--steps", "1", "--warmup", "3"]
    env = dict(os.environ, OMP_NUM_THREADS="1")
    r = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=600, env=env)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    line = json.loads(lines[0])
    assert line["impl"] == "reference" and line["n_gpus"] == 2
    assert line["value"] > 0 and line["e2e"]["value"] == line["value"]
    assert line["config"]["parallelism"] == "replicas x2"
