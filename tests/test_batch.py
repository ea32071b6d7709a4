"""Batched frames (gbr_batch_*): many scenes in one graph-replayed launch
chain give, scene by scene, exactly what one-scene frames give -- the same
bin lists, winners, depths and colours -- for every bin size and queue chunk
the autotuner may pick; one batch scene is also checked against the oracle
directly.  The CPU part checks the uneven-batch generator."""
import numpy as np
import pytest

import scenes
from oracle import oracle


def test_batch_scene_generator_is_seeded_and_uneven():
    a = scenes.batch_scenes(12, seed=5, max_tris=20000)
    b = scenes.batch_scenes(12, seed=5, max_tris=20000)
    assert [s.name for s in a] == [s.name for s in b]
    assert all(np.array_equal(x.meshes[0].vertices, y.meshes[0].vertices) for x, y in zip(a, b))
    counts = [s.num_triangles for s in a]
    assert min(counts) >= 1000 and max(counts) <= 20000 and len(set(counts)) > 6
    assert {(s.width, s.height) for s in a} <= set(scenes.BATCH_RESOLUTIONS)


def mixed_scenes():
    """Uneven soups plus a textured, back-face-culled sphere under a
    perspective camera and a two-mesh scene."""
    out = scenes.batch_scenes(7, seed=3, max_tris=40000)
    out.append(scenes.sphere_scene(320, 240, sample=scenes.SAMPLE_LINEAR))
    two = scenes.sphere_scene(256, 256)
    m2 = scenes.uv_sphere_mesh(24, 12, 0.6)
    m2.world = scenes.identity16()
    m2.world[12:15] = [0.9, 0.4, 0.5]
    two.meshes.append(m2)
    out.append(two)
    out.append(scenes.soup_scene(3000, 512, 512, seed=77, cull=scenes.CULL_BACKFACE))
    return out


def single_frame(gbr, scene, bin_size, chunk):
    s = scene
    s.bin_w = s.bin_h = bin_size
    with gbr.Renderer(s.width, s.height) as r:
        r.load_scene(s, chunk)
        r.render_scene(s)
        colour, depth = r.readback()
        ids = r.readback_ids()
        offsets, bins = r.get_bins()
        st = r.stats()
    return colour, depth, ids, offsets, bins, st


def build_batch(gbr, scene_list):
    rs = []
    b = gbr.Batch()
    for s in scene_list:
        r = gbr.Renderer(s.width, s.height)
        r.load_scene(s)
        b.add_scene(r, s)
        rs.append(r)
    return b, rs


def close_batch(b, rs):
    b.close()
    for r in rs:
        r.close()


def assert_batch_equals_single(gbr, b, scene_list, bin_size, chunk):
    for i, s in enumerate(scene_list):
        colour, depth, ids = b.readback(i)
        offsets, bins = b.get_bins(i)
        ref = single_frame(gbr, s, bin_size, chunk)
        assert np.array_equal(offsets, ref[3]) and np.array_equal(bins, ref[4]), f"scene {i}: bin lists differ"
        assert np.array_equal(ids, ref[2]), f"scene {i}: winners differ"
        assert np.array_equal(depth.view(np.uint32), ref[1].view(np.uint32)), f"scene {i}: depth differs"
        assert np.array_equal(colour, ref[0]), f"scene {i}: colour differs"


@pytest.mark.gpu
@pytest.mark.parametrize("bin_size,chunk,threads", [(16, 64, 256), (8, 32, 256), (32, 128, 256), (16, 4096, 256),
                                                    (16, 64, 128), (8, 32, 128), (32, 128, 128), (16, 4096, 128)])
def test_batch_equals_single_frames(gbr_lib, cuda_device, bin_size, chunk, threads):
    """Every scene of a batch frame equals its single frame, for 256- and
    128-thread raster CTAs (a 128-thread CTA depth-sorts 1024 entries at a
    time into 128 buckets: a 4096-entry queue chunk takes four passes)."""
    sl = mixed_scenes()
    b, rs = build_batch(gbr_lib, sl)
    b.set_config(bin_size, chunk, raster_threads=threads)
    assert b.config()["raster_threads"] == threads
    b.render()
    st = b.stats()
    assert st["num_scenes"] == len(sl) and st["graph_captures"] >= 1
    assert st["num_triangles"] == sum(s.num_triangles for s in sl)
    assert_batch_equals_single(gbr_lib, b, sl, bin_size, chunk)
    # the second frame may capture once more (the sub-counters per bin follow
    # the first frame's density); it renders the same bins, and later frames
    # replay the captured graph
    b.render()
    st2 = b.stats()
    assert st2["graph_captures"] <= st["graph_captures"] + 1 and st2["num_pairs"] == st["num_pairs"]
    assert_batch_equals_single(gbr_lib, b, sl, bin_size, chunk)
    b.render()
    st3 = b.stats()
    assert st3["graph_captures"] == st2["graph_captures"] and st3["num_pairs"] == st["num_pairs"]
    close_batch(b, rs)


@pytest.mark.gpu
def test_all_flat_batch_then_textured_scene(gbr_lib, cuda_device):
    """A batch of vertex-coloured soups runs the shade pass's flat variant;
    switching one scene to the normal view (not flat) captures the graph
    anew with the general variant.  Both frames equal single frames."""
    sl = scenes.batch_scenes(6, seed=11, max_tris=30000)
    b, rs = build_batch(gbr_lib, sl)
    b.set_config(16, 128)
    b.render()
    st = b.stats()
    assert_batch_equals_single(gbr_lib, b, sl, 16, 128)
    sl[2].vis = scenes.VIS_NORMAL
    b.set_view(2, sl[2].camera, sl[2].cull, sl[2].sample, sl[2].vis)
    b.render()
    st2 = b.stats()
    assert st2["graph_captures"] > st["graph_captures"]
    assert_batch_equals_single(gbr_lib, b, sl, 16, 128)
    close_batch(b, rs)


@pytest.mark.gpu
def test_batch_scene_matches_oracle(gbr_lib, cuda_device):
    sl = [scenes.soup_scene(20000, 320, 240, seed=21), scenes.sphere_scene(320, 240)]
    b, rs = build_batch(gbr_lib, sl)
    b.set_config(16, 64)
    b.render()
    for i, s in enumerate(sl):
        colour, depth, ids = b.readback(i)
        offsets, bins = b.get_bins(i)
        o = oracle.render(s, oracle.RASTER_FIXED)
        assert np.array_equal(offsets, o["offsets"]) and np.array_equal(bins, o["bins"])
        assert np.array_equal(ids, o["ids"])
        assert np.array_equal(depth.view(np.uint32), o["depth"].view(np.uint32))
        c = lambda x: np.stack([(x >> k) & 255 for k in (0, 8, 16, 24)], -1).astype(np.int64)
        assert np.abs(c(colour) - c(o["colour"])).max() <= 1
    close_batch(b, rs)


@pytest.mark.gpu
def test_batch_view_change_and_overflow_rerun(gbr_lib, cuda_device):
    # 2,000 screen-filling triangles over 8x8 bins: about 65M bin entries,
    # far above the initial bin storage, so the first frame re-renders
    big = scenes.soup_scene(2000, 1920, 1080, seed=5)
    v = big.meshes[0].vertices
    rng = np.random.default_rng(0)
    p = v["p"].reshape(-1, 3, 3)
    p[:, 0, :2] = [-1.0, -1.0]
    p[:, 1, :2] = [3.0, -1.0]
    p[:, 2, :2] = [-1.0, 3.0]
    p[:, :, 2] = rng.uniform(0.01, 0.99, (len(p), 1))
    v["p"] = p.reshape(-1, 3)
    sphere = scenes.sphere_scene(320, 240)
    sl = [big, sphere]
    b, rs = build_batch(gbr_lib, sl)
    b.set_config(8, 64)
    b.render()
    st = b.stats()
    assert st["overflow_reruns"] >= 1
    assert_batch_equals_single(gbr_lib, b, sl, 8, 64)
    # move the sphere's camera: the batch follows the new view
    cam = scenes.perspective_camera(np.array([0.4, 0.2, 2.5], np.float32), 60.0, 320, 240)
    sphere.camera = cam
    b.set_view(1, cam, sphere.cull, sphere.sample, sphere.vis)
    b.render()
    assert_batch_equals_single(gbr_lib, b, [big, sphere], 8, 64)
    close_batch(b, rs)


@pytest.mark.gpu
def test_batch_autotune_keeps_output(gbr_lib, cuda_device):
    sl = scenes.batch_scenes(10, seed=9, max_tris=30000)
    b, rs = build_batch(gbr_lib, sl)
    b.set_config(16, 64)
    b.render()
    before = [b.readback(i) for i in range(len(sl))]
    best = b.autotune(bin_sizes=(8, 16, 32), chunks=(32, 64, 128), raster_ctas=(4, 5), frames=1,
                      raster_threads=(128, 256))
    assert best["bin_size"] in (8, 16, 32) and best["queue_chunk"] in (32, 64, 128)
    assert best["raster_ctas"] in (4, 5) and best["raster_threads"] in (128, 256)
    assert b.config() == best
    b.render()
    for i in range(len(sl)):
        after = b.readback(i)
        for x, y in zip(before[i], after):
            assert np.array_equal(x, y)
    close_batch(b, rs)


@pytest.mark.gpu
def test_batch_readback_all_equals_per_scene_readback(gbr_lib, cuda_device):
    sl = scenes.batch_scenes(6, seed=4, max_tris=20000)
    b, rs = build_batch(gbr_lib, sl)
    b.set_config(16, 64)
    b.render()
    every = b.readback_all()
    some = [np.zeros(s.width * s.height, np.uint32) if i % 2 == 0 else None for i, s in enumerate(sl)]
    b.readback_all(some)
    for i in range(len(sl)):
        colour = b.readback(i)[0]
        assert np.array_equal(every[i], colour)
        if some[i] is not None:
            assert np.array_equal(some[i].reshape(colour.shape), colour)
    close_batch(b, rs)


@pytest.mark.gpu
def test_renderer_in_batch_cannot_be_destroyed(gbr_lib, cuda_device):
    s = scenes.soup_scene(1000, 256, 256, seed=1)
    b, rs = build_batch(gbr_lib, [s])
    with pytest.raises(gbr_lib.GbrError):
        gbr_lib.check(gbr_lib.lib().gbr_destroy(rs[0].h))
    close_batch(b, rs)
