"""The multi-GPU path is replicas only (independent frames, no data-path
collective).  Its host logic -- one seeded scene per rank, the job's time
as the maximum over ranks, the reference arm working on rank 0 only -- is
checked here with world_size-2 gloo process groups on CPU."""
import os
import socket
import subprocess
import sys

import numpy as np
import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out_dir):
    sys.path.insert(0, ROOT)
    import bench
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    try:
        local = [1.5 + rank, 10.0 - rank, 0.25 * (rank + 1)]
        got = bench.max_over_ranks(local, dist, "cpu")
        scene = bench.make_scene(rank)
        v = scene.meshes[0].vertices
        np.save(os.path.join(out_dir, f"r{rank}.npy"),
                np.array(got + [float(v["p"][:1000].sum()), float(len(v))], np.float64))
    finally:
        dist.destroy_process_group()


def test_replica_timing_is_the_slowest_rank_and_scenes_differ(tmp_path):
    world = 2
    mp.start_processes(_rank_main, args=(world, _free_port(), str(tmp_path)), nprocs=world, start_method="spawn")
    r0, r1 = (np.load(tmp_path / f"r{k}.npy") for k in range(world))
    assert np.allclose(r0[:3], [2.5, 10.0, 0.5]) and np.allclose(r1[:3], r0[:3])   # max over ranks, on every rank
    assert r0[4] == r1[4] == 3_000_000           # each rank renders a full 1M-triangle frame
    assert r0[3] != r1[3]                        # seeded per rank: independent replicas


def test_max_over_ranks_single_process():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks([1.0, 2.0], None, "cpu") == [1.0, 2.0]


def test_reference_arm_runs_on_rank_zero_only():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--gpus", "2",
                          "--steps", "1", "--warmup", "0"], env=env, capture_output=True, text=True, timeout=300)
    assert out.returncode == 0 and out.stdout.strip() == ""
