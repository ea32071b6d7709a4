"""Host logic of the multi-GPU split (custom-gpgpu-rasterizer_gb300/sharding.py),
on CPU: bands of bin rows and scene partitions, and world_size-2 gloo
process groups in which each rank renders its band of one frame with the
oracle (the CPU restatement, restricted to its bin rows as
gbr_set_bin_rows restricts the GPU path) and the bands are gathered: the
composite equals the one-rank frame.  The GPU side of the split is checked
against the one-GPU frame in test_parity_gpu.py."""
import os
import socket
import sys

import numpy as np
import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "custom-gpgpu-rasterizer_gb300")

import scenes  # noqa: E402
import sharding  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


@pytest.mark.parametrize("rows,world", [(68, 2), (68, 3), (5, 5), (30, 4), (3, 1)])
def test_row_bands_cover_every_row_once(rows, world):
    for weights in (None, np.linspace(1, 50, rows) ** 2):
        bands = sharding.row_bands(rows, world, weights)
        assert len(bands) == world and bands[0][0] == 0 and bands[-1][1] == rows
        assert all(a < b for a, b in bands) and all(bands[k][1] == bands[k + 1][0] for k in range(world - 1))


def test_row_bands_balance_the_weights():
    w = np.ones(100)
    w[:10] = 50.0   # the first rows hold most of the pairs
    bands = sharding.row_bands(100, 2, w)
    load = [w[a:b].sum() for a, b in bands]
    assert max(load) / min(load) < 1.2 and bands[0][1] < 20


def test_scene_partition_covers_and_balances():
    specs = scenes.batch_scene_specs(256, seed=0)
    costs = [sharding.scene_cost(n, w, h) for n, w, h, _ in specs]
    for world in (1, 2, 4, 8):
        parts = sharding.scene_partition(costs, world)
        assert sorted(i for p in parts for i in p) == list(range(256))
        load = [sum(costs[i] for i in p) for p in parts]
        assert max(load) <= sum(costs) / world + max(costs)   # greedy bound
        assert parts == sharding.scene_partition(costs, world)   # the same on every rank


def test_composite_rejects_overlap_and_gaps():
    rows = np.zeros((4, 3), np.uint32)
    with pytest.raises(ValueError):
        sharding.composite([(0, 4, rows), (3, 7, rows)], 7, 3)
    with pytest.raises(ValueError):
        sharding.composite([(0, 4, rows)], 7, 3)


def _band_rank(rank, world, port, out_dir):
    sys.path[:0] = [ROOT, PKG]
    import scenes as sc
    import sharding as sh
    from oracle import oracle
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    try:
        s = sc.soup_scene(20000, 320, 250, 16, seed=5)
        full = oracle.render(s, oracle.RASTER_FIXED, num_threads=2, want_bins=False)
        # bands weighted by the bin rows' pairs, as a driver would from its last frame
        pairs = oracle.render(s, oracle.RASTER_FIXED, num_threads=2, want_image=False)["offsets"]
        per_bin = np.diff(pairs.astype(np.int64)).reshape(s.num_bins_y, s.num_bins_x).sum(1)
        band = sh.row_bands(s.num_bins_y, world, per_bin)[rank]
        mine = oracle.render(s, oracle.RASTER_FIXED, num_threads=2, want_bins=False, bin_rows=band)
        y0, y1 = sh.band_pixel_rows(band, s.bin_h, s.height)
        out = {}
        for key in ("colour", "ids", "depth"):
            rows = np.ascontiguousarray(mine[key][y0:y1])
            out[key] = sh.gather_composite(dist, rows, y0, y1, s.height, s.width)
            out[key + "_full"] = full[key]
        np.savez(os.path.join(out_dir, f"r{rank}.npz"), **out, band=np.array(band))
    finally:
        dist.destroy_process_group()


def test_two_rank_frame_split_composites_to_the_one_rank_frame(tmp_path):
    world = 2
    mp.start_processes(_band_rank, args=(world, _free_port(), str(tmp_path)), nprocs=world, start_method="spawn")
    r = [np.load(tmp_path / f"r{k}.npz") for k in range(world)]
    assert tuple(r[0]["band"]) != tuple(r[1]["band"])
    for k in range(world):
        for key in ("colour", "ids", "depth"):
            assert np.array_equal(r[k][key].view(np.uint32), r[k][key + "_full"].view(np.uint32)), key
