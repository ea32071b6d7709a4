"""GPU parity: the CUDA path, called through the C ABI, against the oracle.

Bar (per pixel, per bin):
  * bin lists: bit-exact against the oracle (which restates TB_Kernel's
    bounding-box rule), after sorting each bin by primitive id;
  * against the oracle in fixed-point mode (same coverage rule as the
    kernels): winning primitive ids and depth bit-exact, colour within 1 LSB;
  * against the oracle in reference mode (float edge functions at integer
    pixels, CUDAROPs.cu:120-145): a pixel's winner may differ only where a
    triangle's coverage flips inside the stated edge band (|e_ref| <= bound,
    bound = 16.16 snapping + float rounding), or where two fragments' depths
    are within 1e-6 relative; depth agrees within 1e-6 relative elsewhere.
"""
import numpy as np
import pytest

import scenes
from oracle import oracle

pytestmark = pytest.mark.gpu

EMPTY = 0xFFFFFFFF
DEPTH_RTOL = 1e-6


def gpu_render(gbr, scene, chunk=256, renderer=None, binning=0, frames=1):
    r = renderer or gbr.Renderer(scene.width, scene.height)
    r.load_scene(scene, chunk)
    r.set_binning(binning)
    for _ in range(frames - 1):   # earlier frames size the work items of the last one
        r.render_scene(scene)
        r.stats()
    r.render_scene(scene)
    colour, depth = r.readback()
    ids = r.readback_ids()
    offsets, bins = r.get_bins()
    stats = r.stats()
    return {"colour": colour, "depth": depth, "ids": ids, "offsets": offsets, "bins": bins, "stats": stats,
            "renderer": r}


def channels(c):
    c = c.astype(np.int64)
    return np.stack([c & 255, (c >> 8) & 255, (c >> 16) & 255, (c >> 24) & 255], -1)


def assert_bins_equal(g, o):
    assert np.array_equal(g["offsets"], o["offsets"]), "bin offsets differ"
    assert np.array_equal(g["bins"], o["bins"]), "bin lists differ"


def assert_matches_fixed(g, o, mask=None):
    m = np.ones(g["ids"].shape, bool) if mask is None else mask
    bad = (g["ids"] != o["ids"]) & m
    assert not bad.any(), f"{bad.sum()} pixels with a different winner, first {np.argwhere(bad)[:5].tolist()}"
    dbad = (g["depth"].view(np.uint32) != o["depth"].view(np.uint32)) & m
    assert not dbad.any(), f"{dbad.sum()} depth mismatches"
    d = np.abs(channels(g["colour"]) - channels(o["colour"])).max(-1)
    assert (d[m] <= 1).all(), f"colour off by {d[m].max()} LSB at {np.argwhere((d > 1) & m)[:5].tolist()}"


def check_reference_band(scene, g, o, limit=400):
    """Every winner difference against reference mode must come from a
    coverage flip inside the edge band or a depth near-tie."""
    diff = np.argwhere(g["ids"] != o["ids"])
    unexplained = []
    for y, x in diff[:limit]:
        a, b = int(g["ids"][y, x]), int(o["ids"][y, x])
        explained = False
        probes = {p: oracle.probe(scene, p, int(x), int(y)) for p in {a, b} - {EMPTY}}
        for p, pr in probes.items():
            if pr["covered_ref"] != pr["covered_fixed"]:
                if any(abs(e) <= bd for e, bd in zip(pr["e_ref"], pr["e_bound"])):
                    explained = True
        if not explained and a != EMPTY and b != EMPTY:
            za, zb = probes[a]["z_fixed"], probes[b]["z_ref"]
            if abs(za - zb) <= DEPTH_RTOL * max(abs(za), abs(zb)) + 1e-30:
                explained = True
        if not explained:
            unexplained.append((int(x), int(y), a, b, probes))
    assert not unexplained, unexplained[:3]
    same = (g["ids"] == o["ids"]) & (g["ids"] != EMPTY)
    zg, zo = g["depth"][same].astype(np.float64), o["depth"][same].astype(np.float64)
    rel = np.abs(zg - zo) / np.maximum(np.abs(zo), 1e-30)
    assert (rel <= DEPTH_RTOL).all(), f"depth rel err {rel.max()}"
    return len(diff)


def run_case(gbr, scene, chunk=256, ref_band=True, frames=1):
    g = gpu_render(gbr, scene, chunk, frames=frames)
    ofx = oracle.render(scene, oracle.RASTER_FIXED)
    assert_bins_equal(g, ofx)
    assert_matches_fixed(g, ofx)
    assert g["stats"]["num_visible"] == ofx["stats"]["num_visible"]
    assert g["stats"]["num_pairs"] == ofx["stats"]["num_pairs"]
    if ref_band:
        oref = oracle.render(scene, oracle.RASTER_REFERENCE)
        assert_bins_equal(g, oref)
        check_reference_band(scene, g, oref)
    g["renderer"].close()
    return g, ofx


@pytest.mark.parametrize("sample", [scenes.SAMPLE_POINT, scenes.SAMPLE_LINEAR])
@pytest.mark.parametrize("vis", [scenes.VIS_PBR, scenes.VIS_DEPTH, scenes.VIS_NORMAL])
def test_sphere_640x480(gbr_lib, cuda_device, sample, vis):
    run_case(gbr_lib, scenes.sphere_scene(sample=sample, vis=vis))


@pytest.mark.parametrize("cull", [scenes.CULL_NONE, scenes.CULL_BACKFACE, scenes.CULL_FRONTFACE])
def test_soup_cull_modes(gbr_lib, cuda_device, cull):
    run_case(gbr_lib, scenes.soup_scene(30000, 320, 240, seed=11, cull=cull))


def test_soup_ivertex_layout(gbr_lib, cuda_device):
    a, _ = run_case(gbr_lib, scenes.soup_scene(20000, 320, 240, seed=12, ivertex=True), ref_band=False)
    b, _ = run_case(gbr_lib, scenes.soup_scene(20000, 320, 240, seed=12, ivertex=False), ref_band=False)
    assert np.array_equal(a["colour"], b["colour"]) and np.array_equal(a["ids"], b["ids"])


@pytest.mark.parametrize("bw,bh,w,h", [(8, 8, 320, 240), (32, 32, 320, 240), (24, 20, 320, 240),
                                       (16, 16, 333, 250), (64, 64, 300, 200), (16, 8, 160, 130)])
def test_soup_bin_geometries(gbr_lib, cuda_device, bw, bh, w, h):
    s = scenes.soup_scene(15000, w, h, seed=13)
    s.bin_w, s.bin_h = bw, bh
    run_case(gbr_lib, s, ref_band=False)


@pytest.mark.parametrize("chunk", [1, 16, 100])
def test_multi_chunk_bins_merge(gbr_lib, cuda_device, chunk):
    """queue_chunk = 1, 16 or 100 entries per raster pass over a tile; on
    the second frame the library splits bins of more than 64 entries into
    several work items (sized from the first frame's pairs), whose tiles
    merge in the frame buffer through 64-bit atomicMin."""
    g, _ = run_case(gbr_lib, scenes.soup_scene(20000, 256, 192, seed=14), chunk=chunk, ref_band=False, frames=2)
    assert g["stats"]["num_work_items"] > 16 * 12


def two_sphere_scene():
    s = scenes.sphere_scene(320, 240)
    m2 = scenes.uv_sphere_mesh(24, 12, 0.6)
    m2.world = scenes.identity16()
    m2.world[12:15] = [0.9, 0.4, 0.5]
    rng = np.random.default_rng(2)
    m2.vertices["c"] = rng.random((len(m2.vertices), 3)).astype(np.float32)
    s.meshes.append(m2)
    return s


def test_multi_mesh_textured_and_vertex_coloured(gbr_lib, cuda_device):
    g, o = run_case(gbr_lib, two_sphere_scene())
    n0 = scenes.sphere_scene(320, 240).num_triangles
    assert (g["ids"][g["ids"] != EMPTY] >= n0).any() and (g["ids"][g["ids"] != EMPTY] < n0).any()


def strip_scene():
    return scenes.strip_grid_scene()


def test_triangle_strip(gbr_lib, cuda_device):
    g, _ = run_case(gbr_lib, strip_scene())
    assert (g["ids"] != EMPTY).sum() > 1000


def test_empty_scene_is_clear_colour(gbr_lib, cuda_device):
    s = scenes.Scene("empty", 100, 60, 16, 16, scenes.identity_camera(), [])
    r = gbr_lib.Renderer(100, 60)
    r.load_scene(s)
    r.render_scene(s)
    colour, depth = r.readback()
    assert (colour == scenes.CLEAR_COLOUR32).all() and (depth == 0).all()
    r.close()


def test_guard_band_triangles_use_float_edges(gbr_lib, cuda_device):
    v = np.zeros(6, scenes.POS3_RGBA8)
    v["p"][0:3] = [(-0.5, -0.5, 0.4), (80.0, 0.2, 0.6), (-0.4, 0.7, 0.5)]  # x_ndc=80 -> 12960 px, outside +-8192
    v["p"][3:6] = [(-0.9, -0.9, 0.2), (-0.9, 0.9, 0.9), (0.9, -0.9, 0.9)]
    v["rgba"] = [0xFF0000FF, 0xFF00FF00, 0xFFFF0000, 0xFF808080, 0xFF101010, 0xFFF0F0F0]
    s = scenes.Scene("guard", 320, 240, 16, 16, scenes.identity_camera(), [scenes.Mesh(vertices=v)],
                     cull=scenes.CULL_NONE)
    g, o = run_case(gbr_lib, s)
    assert g["stats"]["num_float_path"] == 1


def test_bin_storage_overflow_reruns_exactly(gbr_lib, cuda_device):
    rng = np.random.default_rng(7)
    n = 300
    v = np.zeros(3 * n, scenes.POS3_RGBA8)
    big = np.array([(-1.2, -1.2), (-1.2, 1.2), (1.2, -1.2)])
    for t in range(n):
        v["p"][3 * t:3 * t + 3, :2] = big + rng.uniform(-0.1, 0.1, (3, 2))
        v["p"][3 * t:3 * t + 3, 2] = rng.uniform(0, 1)
    v["rgba"] = rng.integers(0, 2**32, 3 * n, dtype=np.uint64).astype(np.uint32)
    s = scenes.Scene("overflow", 640, 480, 8, 8, scenes.identity_camera(), [scenes.Mesh(vertices=v)],
                     cull=scenes.CULL_NONE)
    g, o = run_case(gbr_lib, s, ref_band=False)
    assert g["stats"]["num_pairs"] > 1_000_000
    assert g["stats"]["overflow_reruns"] >= 1


def test_repeated_and_alternating_frames(gbr_lib, cuda_device):
    a = scenes.soup_scene(10000, 256, 192, seed=21)
    b = scenes.sphere_scene(256, 192)
    r = gbr_lib.Renderer(256, 192)
    first = gpu_render(gbr_lib, a, 32, renderer=r)
    for _ in range(3):
        again = gpu_render(gbr_lib, a, 32, renderer=r)
        assert np.array_equal(first["colour"], again["colour"]) and np.array_equal(first["ids"], again["ids"])
    gb = gpu_render(gbr_lib, b, 32, renderer=r)
    ob = oracle.render(b, oracle.RASTER_FIXED)
    assert_matches_fixed(gb, ob)
    again = gpu_render(gbr_lib, a, 32, renderer=r)
    assert np.array_equal(first["colour"], again["colour"])
    r.close()


@pytest.mark.parametrize("bins", [8, 16])
def test_icosphere_4k_subpixel(gbr_lib, cuda_device, bins):
    """Displaced icosphere, 327,680 triangles, 3840x2160, mostly sub-pixel
    triangles, 8x8 and 16x16 bins (the reference's 8x8 bins rasterise nothing,
    so 8x8 is checked against the oracle only)."""
    s = scenes.icosphere_scene(bin_size=bins)
    # the second frame takes the raster's small-triangle variant (a lane per
    # triangle), chosen from the first frame's pairs per visible triangle
    g, o = run_case(gbr_lib, s, ref_band=(bins == 16), frames=2)
    assert g["stats"]["num_visible"] > 100_000 and (g["ids"] != EMPTY).sum() > 100_000
    assert g["stats"]["raster_lanes"] == 1


@pytest.mark.parametrize("lights", [False, True])
def test_bilinear_and_scene_lights_extension(gbr_lib, cuda_device, lights):
    """The build's shading extensions (true bilinear filtering, directional
    and point scene lights; the reference's GPU shader has neither) against
    the oracle, which restates them."""
    s = scenes.sphere_scene(320, 240, sample=scenes.SAMPLE_BILINEAR)
    if lights:
        s.lights = [scenes.Light(scenes.LIGHT_DIRECTIONAL, (1.0, 0.9, 0.8), 5.0, (0.577, -0.577, -0.577)),
                    scenes.Light(scenes.LIGHT_POINT, (0.3, 0.5, 1.0), 12.0, (1.2, 0.8, 2.0))]
    g, o = run_case(gbr_lib, s, ref_band=False)
    assert len(np.unique(g["colour"])) > 500


def test_lit_icosphere_bilinear(gbr_lib, cuda_device):
    """The displaced icosphere with bilinear filtering of its noise texture and
    a directional plus a point light (smaller than 4K so the oracle stays
    quick)."""
    s = scenes.icosphere_lit_scene(960, 540, subdiv=6, tex_size=1024, distance=3.0)
    g, o = run_case(gbr_lib, s, ref_band=False)
    assert (g["ids"] != EMPTY).sum() > 10_000


def test_full_size_soup_1m_1080p(gbr_lib, cuda_device):
    """1M-triangle 1920x1080 soup: bin lists bit-exact at full size, and the
    whole frame -- every pixel's winner and depth bit-exact, colour within
    1 LSB -- against the oracle's fixed-point mode."""
    s = scenes.soup_scene(1_000_000, 1920, 1080, seed=0)
    g = gpu_render(gbr_lib, s)
    ob = oracle.render(s, oracle.RASTER_FIXED)
    assert_bins_equal(g, ob)
    assert_matches_fixed(g, ob)
    assert g["stats"]["num_pairs"] == ob["stats"]["num_pairs"]
    # the second frame counts in block-private rows (the first frame showed
    # about 6 pairs per (block, bin)): same lists, same image
    r = g["renderer"]
    assert g["stats"]["count_blocks"] == 0
    r.render_scene(s)
    offsets, bins = r.get_bins()
    colour, depth = r.readback()
    st = r.stats()
    assert st["count_blocks"] > 0
    assert_bins_equal({"offsets": offsets, "bins": bins}, ob)
    assert np.array_equal(colour, g["colour"]) and np.array_equal(r.readback_ids(), g["ids"])
    r.close()


@pytest.mark.parametrize("bins,n,cull", [(8, 50_000, scenes.CULL_NONE), (32, 120_000, scenes.CULL_BACKFACE),
                                         (24, 30_000, scenes.CULL_NONE)])
def test_block_counter_rows(gbr_lib, cuda_device, bins, n, cull):
    """Exact binning with block-private counter rows, taken once a frame has
    shown at least one (triangle, bin) pair per (block, bin): the second
    frame's bin lists, winners, depth and colour against the oracle."""
    s = scenes.soup_scene(n, 640, 480, bin_size=bins, seed=5, cull=cull)
    r = gbr_lib.Renderer(s.width, s.height)
    first = gpu_render(gbr_lib, s, 64, renderer=r)
    assert first["stats"]["count_blocks"] == 0
    r.render_scene(s)
    offsets, bl = r.get_bins()
    colour, depth = r.readback()
    g = {"offsets": offsets, "bins": bl, "colour": colour, "depth": depth, "ids": r.readback_ids()}
    st = r.stats()
    assert st["count_blocks"] == min((n + 1023) // 1024, cuda_device_sms())
    o = oracle.render(s, oracle.RASTER_FIXED)
    assert_bins_equal(g, o)
    assert_matches_fixed(g, o)
    assert st["num_pairs"] == o["stats"]["num_pairs"] and st["num_visible"] == o["stats"]["num_visible"]
    r.close()


def cuda_device_sms():
    import torch
    return torch.cuda.get_device_properties(0).multi_processor_count


@pytest.mark.parametrize("case", ["soup", "sphere", "soup-predicted"])
def test_frame_split_by_bin_rows_composites_to_the_full_frame(gbr_lib, cuda_device, case):
    """A frame split across GPUs by bin rows (gbr_set_bin_rows), its three
    bands rendered one after another on this GPU by separate renderers:
    every band's rows are the full frame's rows (colour, depth, ids
    bit-identical), and the composite is the full frame.  With predicted
    binning too, whose pre-pass and capacities see the cut rectangles."""
    import sharding
    s = scenes.sphere_scene() if case == "sphere" else scenes.soup_scene(60000, 640, 480, 16, seed=21)
    full = gpu_render(gbr_lib, s)
    full["renderer"].close()
    bands = sharding.row_bands(s.num_bins_y, 3)
    parts = {"colour": [], "depth": [], "ids": []}
    pairs = 0
    for band in bands:
        r = gbr_lib.Renderer(s.width, s.height)
        r.load_scene(s)
        if case.endswith("predicted"):
            import predictor
            predictor.install(r)
        r.set_bin_rows(*band)
        for _ in range(2):   # the second frame: the predicted path with sized storage
            r.render_scene(s)
            st = r.stats()
        colour, depth = r.readback()
        ids = r.readback_ids()
        y0, y1 = sharding.band_pixel_rows(band, s.bin_h, s.height)
        for key, img in (("colour", colour), ("depth", depth), ("ids", ids)):
            parts[key].append((y0, y1, img[y0:y1].copy()))
        pairs += st["num_pairs"]
        r.close()
    for key in parts:
        got = sharding.composite(parts[key], s.height, s.width, full[key].dtype)
        assert np.array_equal(got.view(np.uint32), full[key].view(np.uint32)), key
    # a triangle spanning a band boundary is binned by each band it touches
    assert pairs == full["stats"]["num_pairs"]


@pytest.mark.parametrize("phase", [16, 64])
@pytest.mark.parametrize("case", ["soup", "sphere", "strip"])
def test_tma_record_staging_renders_identically(gbr_lib, cuda_device, case, phase):
    """Setup records staged by bulk asynchronous copies on mbarriers
    (GBR_STAGING_TMA): phase 16 prefetches the next phase's records, phase 64
    copies each phase's own; bin lists, ids, depth and colour equal the
    load-staged frame and the fixed-mode oracle."""
    s = {"soup": lambda: scenes.soup_scene(60000, 640, 480, 16, seed=33), "sphere": scenes.sphere_scene,
         "strip": scenes.strip_grid_scene}[case]()
    out = []
    for tma in (False, True):
        r = gbr_lib.Renderer(s.width, s.height)
        r.set_raster_params(phase=phase)
        r.set_raster_staging(tma)
        out.append(gpu_render(gbr_lib, s, renderer=r))
        r.close()
    for key in ("colour", "depth", "ids", "offsets", "bins"):
        assert np.array_equal(out[0][key], out[1][key]), key
    ofx = oracle.render(s, oracle.RASTER_FIXED)
    assert_matches_fixed(out[1], ofx)


def test_two_pass_frames_keep_clean_bins_clear(gbr_lib, cuda_device):
    """Two-pass frames leave the light pass's quads in bins that were clean
    after the last frame and are not drawn now untouched.  One renderer goes
    through frames whose coverage grows, shrinks and moves, changes of view,
    a one-pass depth frame and a texture blit; each frame equals a fresh
    renderer's frame of the same camera and view, bit for bit."""
    base = scenes.sphere_scene()   # textured: two-pass shading
    W, H = base.width, base.height
    cams = {"near": scenes.perspective_camera((0.0, 0.0, 2.2), 60.0, W, H),
            "far": scenes.perspective_camera((0.0, 0.0, 9.0), 60.0, W, H),
            "left": scenes.perspective_camera((1.6, 0.3, 3.5), 60.0, W, H)}
    seq = [("near", scenes.VIS_PBR), ("far", scenes.VIS_PBR), ("left", scenes.VIS_PBR),
           ("left", scenes.VIS_NORMAL), ("far", scenes.VIS_NORMAL), ("near", scenes.VIS_DEPTH),
           ("far", scenes.VIS_PBR), ("blit", None), ("far", scenes.VIS_PBR), ("left", scenes.VIS_PBR)]

    def frame(r, cam, vis):
        base.camera, base.vis = cams[cam], vis
        r.render_scene(base)
        colour, depth = r.readback()
        return colour.copy(), depth.view(np.uint32).copy(), r.readback_ids().copy()

    r = gbr_lib.Renderer(W, H)
    r.load_scene(base)
    tex = r.add_texture(np.full((64, 64), 0xFFC8C8C8, np.uint32))
    for cam, vis in seq:
        if cam == "blit":
            r.draw_texture(tex)
            continue
        got = frame(r, cam, vis)
        with gbr_lib.Renderer(W, H) as fresh:
            fresh.load_scene(base)
            want = frame(fresh, cam, vis)
        for name, a, b in zip(("colour", "depth", "ids"), got, want):
            assert np.array_equal(a, b), f"{cam}/{vis}: {name} differs at {np.argwhere(a != b)[:3].tolist()}"
    r.close()


def test_small_triangle_variant_is_chosen_from_the_last_frame(gbr_lib, cuda_device):
    """The raster's small-triangle variant (a lane per triangle) follows the
    last frame's (triangle, bin) pairs per visible triangle: the 640x480
    sphere's ~10-pixel triangles keep one triangle per warp, a frame of
    sub-pixel triangles takes the variant, the first frame of a renderer
    (no history) and an explicit phase below 32 never do; the frames are
    the fixed-mode oracle's either way."""
    sphere = scenes.sphere_scene()
    g = gpu_render(gbr_lib, sphere, frames=2)
    assert g["stats"]["raster_lanes"] == 0
    g["renderer"].close()
    s = scenes.icosphere_scene(640, 480, bin_size=16, subdiv=6)
    ofx = oracle.render(s, oracle.RASTER_FIXED)
    first = gpu_render(gbr_lib, s, frames=1)
    assert first["stats"]["raster_lanes"] == 0
    first["renderer"].close()
    g = gpu_render(gbr_lib, s, frames=2)
    assert g["stats"]["raster_lanes"] == 1
    assert_matches_fixed(g, ofx)
    g["renderer"].close()
    r = gbr_lib.Renderer(s.width, s.height)
    r.set_raster_params(16, 0)
    g = gpu_render(gbr_lib, s, renderer=r, frames=2)
    assert g["stats"]["raster_lanes"] == 0
    assert_matches_fixed(g, ofx)
    r.close()
