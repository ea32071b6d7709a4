"""Known-answer tests of the CPU oracle against values derived by hand from
the reference's formulas (CustomCUDARasterizer/CUDAROPs.cu,
CUDATextureSampler.cuh, RGBRaw.h, Matrix4.h, Camera.cpp).  The reference
ships no golden vectors; these pin each restated function on cases whose
answers follow directly from the reference source, including its quirks."""
import math
from fractions import Fraction

import numpy as np
import pytest

import scenes
from oracle import oracle


def f32_round(q: Fraction) -> float:
    """Round a rational to the nearest float32 (ties to even)."""
    if q == 0:
        return 0.0
    sign = -1 if q < 0 else 1
    q = abs(q)
    e = math.floor(math.log2(q.numerator) - math.log2(q.denominator))
    while Fraction(2) ** e > q:
        e -= 1
    while Fraction(2) ** (e + 1) <= q:
        e += 1
    e = max(e, -126)
    scale = Fraction(2) ** (23 - e)
    m = q * scale
    fl = math.floor(m)
    rem = m - fl
    if rem > Fraction(1, 2) or (rem == Fraction(1, 2) and fl % 2 == 1):
        fl += 1
    return sign * float(Fraction(fl) / scale)


def fma32(a, b, c) -> float:
    return f32_round(Fraction(float(a)) * Fraction(float(b)) + Fraction(float(c)))


def f32(x) -> float:
    return float(np.float32(x))


def test_vs_position_follows_fused_order():
    # element (r, c) at [c*4 + r]; row 0 = (a, b, c, d)
    a, b, c, d = f32(1.1), f32(-2.3), f32(0.7), f32(0.3)
    m = np.zeros(16, np.float32)
    m[0], m[4], m[8], m[12] = a, b, c, d
    m[15] = 1.0
    p = [f32(0.123), f32(4.56), f32(-7.89)]
    got = oracle.vs_position(m, p)
    inner = fma32(a, p[0], f32(np.float32(b) * np.float32(p[1])))
    want_x = f32(np.float32(fma32(c, p[2], inner)) + np.float32(d))
    assert got[0] == np.float32(want_x)
    assert got[3] == np.float32(1.0)


def test_mat4_mul_left_to_right():
    rng = np.random.default_rng(3)
    A = rng.standard_normal(16).astype(np.float32)
    B = rng.standard_normal(16).astype(np.float32)
    got = oracle.mat4_mul(A, B)
    want = np.zeros(16, np.float32)
    for r in range(4):
        for c in range(4):
            s = np.float32(A[0 * 4 + r] * B[c * 4 + 0])
            for k in range(1, 4):
                s = np.float32(s + np.float32(A[k * 4 + r] * B[c * 4 + k]))
            want[c * 4 + r] = s
    assert np.array_equal(got, want)


@pytest.mark.parametrize("mode", [0, 1])
def test_cull_counter_clockwise_ndc_is_front(mode):
    fwd = [0.0, 0.0, 1.0]
    ccw = ([0, 0, 0.5], [1, 0, 0.5], [0, 1, 0.5])
    cw = ([0, 0, 0.5], [0, 1, 0.5], [1, 0, 0.5])
    # BackFace and FrontFace run the same test (CUDARenderer.cu:760-777)
    assert oracle.cull(*ccw, fwd, mode) is False
    assert oracle.cull(*cw, fwd, mode) is True
    assert oracle.cull(*cw, fwd, 2) is False
    # degenerate: Normalize gives the zero vector, dot = 0 <= 0 -> culled
    assert oracle.cull([0, 0, 0], [1, 1, 0], [2, 2, 0], fwd, mode) is True


def test_frustum_reject_needs_all_three_outside_one_plane():
    assert oracle.frustum_visible([-2, 0, 0.5], [-3, 0, 0.5], [-1.5, 0, 0.5]) is False
    assert oracle.frustum_visible([-2, 0, 0.5], [0, 0, 0.5], [-1.5, 0, 0.5]) is True
    assert oracle.frustum_visible([0, 0, 1.5], [0, 0, 2.0], [0, 0, 1.01]) is False
    assert oracle.frustum_visible([0, 0, -0.1], [0, 0, 2.0], [0, 0, 0.3]) is True
    # spanning x<-1 and x>1 at once is not rejected (no clipping)
    assert oracle.frustum_visible([-5, 0, 0.5], [5, 0.1, 0.5], [0, 5, 0.5]) is True


def ndc_of(sx, sy, w, h):
    return [f32(2 * sx / w - 1), f32(1 - 2 * sy / h)]


def test_bin_rect_reference_rules():
    W, H, nbx, nby = 64, 64, 4, 4
    # screen (10.5, 20.25), (30.75, 25), (15, 40.5): xmin=(short)10.5-1=9 -> bin 0,
    # xmax=(short)30.75+1=31 -> bin 1, ymin=19 -> bin 1, ymax=41 -> bin 2
    xy = ndc_of(10.5, 20.25, W, H) + ndc_of(30.75, 25.0, W, H) + ndc_of(15.0, 40.5, W, H)
    assert oracle.bin_rect(xy, W, H, nbx, nby, 16, 16) == (0, 1, 1, 2)
    # clamps: xmax -> W -> bin W/16 = 4 -> clamped to nbx-1
    xy = ndc_of(50.0, 2.0, W, H) + ndc_of(70.0, 3.0, W, H) + ndc_of(60.0, 9.0, W, H)
    assert oracle.bin_rect(xy, W, H, nbx, nby, 16, 16) == (3, 0, 3, 0)
    # (short)(-5.5) = -5 -> -6 -> clamp 0
    xy = ndc_of(-5.5, 30.0, W, H) + ndc_of(3.0, 31.0, W, H) + ndc_of(1.0, 33.0, W, H)
    assert oracle.bin_rect(xy, W, H, nbx, nby, 16, 16) == (0, 1, 0, 2)


def test_bin_rect_short_wraparound_drops_far_left_triangle():
    # min x saturates to -32768; -32768 - 1 wraps to 32767 in short, clamps to W,
    # and the min bin clamps to numBins.x (not numBins.x - 1): no bin at all
    W, H = 64, 64
    xy = [-1500.0, 0.0, 0.5, 0.0, 0.0, 0.5]  # x_ndc=-1500 -> screen -47968
    r = oracle.bin_rect(xy, W, H, 4, 4, 16, 16)
    assert r[0] > r[2]


def test_point_sampler_and_u_equals_one_quirk():
    tex = np.arange(16, dtype=np.uint32).reshape(4, 4) * np.uint32(0x010101)
    # u*w+0.5 truncated: u=0.1 -> int(0.9) = 0; v=0.3 -> int(1.7) = 1 -> texel 4
    got = oracle.sample(tex, 0.1, 0.3, 0)
    assert np.allclose(got, [4 / 255.0] * 3)
    # u = 1.0 -> x = 4 = w -> out of range -> magenta (1, 0, 1)
    assert np.array_equal(oracle.sample(tex, 1.0, 0.5, 0), np.array([1, 0, 1], np.float32))
    # u slightly below 0: int(-0.2*4+0.5) = int(-0.3) = 0 -> in range
    assert np.allclose(oracle.sample(tex, -0.05, 0.0, 0), [0.0] * 3)


def test_linear_sampler_is_five_tap_cross_with_row_wrap():
    tex = np.zeros((4, 4), np.uint32)
    vals = {0: 40, 1: 80, 3: 200, 4: 16, 5: 8}
    for i, v in vals.items():
        tex.flat[i] = v  # red channel only
    # uv (0.25, 0.0) -> x = int(1.5) = 1, y = 0 -> centre texel 1
    # neighbours: 0, 2, 5 and 1-4 = -3 < 0 -> centre; r = (40 + 0 + 8 + 80)/8 + 80/2
    got = oracle.sample(tex, 0.25, 0.0, 1)
    want_r = np.float32(np.float32(40 / 8 + 0 + 8 / 8 + 80 / 8) + np.float32(40.0)) * np.float32(np.float32(1) / np.float32(255))
    assert got[0] == np.float32(want_r)
    # centre at x=3, y=0: the +1 neighbour is texel 4 (wraps to the next row)
    got = oracle.sample(tex, 0.7, 0.0, 1)   # int(0.7*4+0.5) = int(3.3) = 3
    r = np.float32(0)
    for nb in (2, 4, 7, 3):  # o-1, o+1 (wraps), o+w, o-w<0 -> o
        r = np.float32(r + np.float32(tex.flat[nb]) * np.float32(0.125))
    r = np.float32(r + np.float32(tex.flat[3]) / np.float32(2))
    assert got[0] == np.float32(r * np.float32(np.float32(1) / np.float32(255)))


def test_bilinear_extension_weights_and_clamping():
    tex = np.array([[0, 100], [40, 200]], np.uint32)   # red channel
    # texel centres reproduce the texels
    assert oracle.sample(tex, 0.25, 0.25, 2)[0] == 0.0
    assert np.isclose(oracle.sample(tex, 0.75, 0.25, 2)[0], 100 / 255, atol=1e-7)
    assert np.isclose(oracle.sample(tex, 0.25, 0.75, 2)[0], 40 / 255, atol=1e-7)
    # the midpoint averages all four
    assert np.isclose(oracle.sample(tex, 0.5, 0.5, 2)[0], (0 + 100 + 40 + 200) / 4 / 255, atol=1e-6)
    # a quarter of the way from texel (0,0) to (1,0) along x, on row 0
    assert np.isclose(oracle.sample(tex, 0.375, 0.25, 2)[0], 25 / 255, atol=1e-6)
    # outside [0, 1] clamps to the edge texels (no magenta)
    assert np.isclose(oracle.sample(tex, -3.0, 0.25, 2)[0], 0.0, atol=1e-7)
    assert np.isclose(oracle.sample(tex, 7.0, 9.0, 2)[0], 200 / 255, atol=1e-7)


def test_scene_lights_extension_in_the_oracle():
    """No lights: the reference's constant light.  A directional light
    against the viewer darkens the lit side; a point light adds falloff."""
    base = scenes.sphere_scene(160, 120)
    a = oracle.render(base, oracle.RASTER_FIXED, want_bins=False)
    lit = scenes.sphere_scene(160, 120)
    lit.lights = [scenes.Light(scenes.LIGHT_DIRECTIONAL, (1.0, 1.0, 1.0), 7.0, (0.577, -0.577, -0.577))]
    b = oracle.render(lit, oracle.RASTER_FIXED, want_bins=False)
    assert np.array_equal(a["ids"], b["ids"]) and np.array_equal(a["depth"], b["depth"])
    # same light as the constant one: identical wherever the Lambert term is
    # non-negative (the constant light keeps negative terms, CUDAROPs.cu:439)
    cov = a["ids"] != 0xFFFFFFFF
    same = (a["colour"] == b["colour"]) & cov
    assert same.sum() > 0.4 * cov.sum()
    pt = scenes.sphere_scene(160, 120)
    pt.lights = [scenes.Light(scenes.LIGHT_POINT, (1.0, 1.0, 1.0), 20.0, (0.0, 0.0, 2.5))]
    c = oracle.render(pt, oracle.RASTER_FIXED, want_bins=False)
    ch = lambda x: (x >> 8) & 255
    # the point light sits in front of the sphere: the centre is brighter than the rim
    cy, cx = 60, 80
    centre = ch(c["colour"][cy, cx].astype(np.int64))
    rim_x = cx + int(np.argmax(~cov[cy, cx:])) - 2
    assert centre > ch(c["colour"][cy, rim_x].astype(np.int64))


def test_rgba_swizzle_and_truncation():
    # GetRGBAFromColour: r8 = b*255, g8 = g*255, b8 = r*255, truncating
    c = oracle.rgba_from_colour([1.0, 0.5, 0.25])
    assert c == (63 | (127 << 8) | (255 << 16))
    assert oracle.rgba_from_colour([-0.5, 2.0, 0.0]) == (0 | (255 << 8) | (0 << 16))


def test_camera_matches_reference_construction():
    cam = scenes.perspective_camera((0.0, 0.0, 3.0), 60.0, 640, 480)
    assert cam.proj[15] == 1.0 and cam.proj[11] == -1.0  # data[3][3] stays 1
    assert np.array_equal(cam.view[12:15], np.array([0, 0, -3], np.float32))
    fov = np.float32(math.tan(np.float32(60.0) * (np.float32(math.pi) / np.float32(180.0)) / np.float32(2.0)))
    assert cam.proj[5] == np.float32(np.float32(1.0) / fov)


def _one_triangle_scene(pts, cols=((255, 0, 0), (0, 255, 0), (0, 0, 255)), z=(0.5, 0.5, 0.5), W=16, H=16):
    v = np.zeros(3, scenes.POS3_RGBA8)
    for k, (sx, sy) in enumerate(pts):
        v["p"][k] = (2 * sx / W - 1, 1 - 2 * sy / H, z[k])
        r, g, b = cols[k]
        v["rgba"][k] = r | (g << 8) | (b << 16) | (255 << 24)
    return scenes.Scene("tri", W, H, 16, 16, scenes.identity_camera(), [scenes.Mesh(vertices=v)],
                        cull=scenes.CULL_NONE)


@pytest.mark.parametrize("mode", [oracle.RASTER_REFERENCE, oracle.RASTER_FIXED])
def test_single_triangle_coverage_is_inclusive_at_integer_pixels(mode):
    # right triangle (0,0), (0,8), (8,0) in screen space: covered winding;
    # pixels (x, y) with x >= 0, y >= 0, x + y <= 8 (edges inclusive)
    s = _one_triangle_scene([(0, 0), (0, 8), (8, 0)])
    out = oracle.render(s, mode, num_threads=1)
    ys, xs = np.nonzero(out["ids"] != 0xFFFFFFFF)
    got = set(zip(xs.tolist(), ys.tolist()))
    want = {(x, y) for x in range(16) for y in range(16) if x + y <= 8}
    assert got == want
    assert np.all(out["depth"][out["ids"] == 0] == np.float32(0.5))
    # vertex colour at the corner pixel (0, 0) is vertex 0's red, bytes B,G,R,0
    assert out["colour"][0, 0] == (255 << 16)
    # the opposite winding covers nothing (one-winding rule, CUDAROPs.cu:144)
    s2 = _one_triangle_scene([(0, 0), (8, 0), (0, 8)])
    out2 = oracle.render(s2, mode, num_threads=1)
    assert np.all(out2["ids"] == 0xFFFFFFFF)
    assert np.all(out2["colour"] == scenes.CLEAR_COLOUR32)


def test_depth_test_strict_less_keeps_lowest_id_on_ties():
    v = np.zeros(6, scenes.POS3_RGBA8)
    W = H = 16
    tri = [(0, 0), (0, 8), (8, 0)]
    for t, zv in enumerate((0.5, 0.5)):
        for k, (sx, sy) in enumerate(tri):
            v["p"][3 * t + k] = (2 * sx / W - 1, 1 - 2 * sy / H, zv)
    s = scenes.Scene("tie", W, H, 16, 16, scenes.identity_camera(), [scenes.Mesh(vertices=v)], cull=scenes.CULL_NONE)
    out = oracle.render(s, oracle.RASTER_FIXED, num_threads=1)
    assert set(np.unique(out["ids"]).tolist()) == {0, 0xFFFFFFFF}
    v["p"][3:6, 2] = 0.25  # second triangle in front now
    out = oracle.render(s, oracle.RASTER_FIXED, num_threads=1)
    assert set(np.unique(out["ids"]).tolist()) == {1, 0xFFFFFFFF}


def test_reference_and_fixed_modes_differ_only_inside_the_edge_band():
    s = scenes.soup_scene(4000, 160, 120, seed=5)
    ref = oracle.render(s, oracle.RASTER_REFERENCE)
    fx = oracle.render(s, oracle.RASTER_FIXED)
    assert np.array_equal(ref["offsets"], fx["offsets"]) and np.array_equal(ref["bins"], fx["bins"])
    diff = np.argwhere(ref["ids"] != fx["ids"])
    for y, x in diff[:200]:
        for prim in {int(ref["ids"][y, x]), int(fx["ids"][y, x])} - {0xFFFFFFFF}:
            p = oracle.probe(s, prim, int(x), int(y))
            if p["covered_ref"] != p["covered_fixed"]:
                assert any(abs(e) <= b for e, b in zip(p["e_ref"], p["e_bound"])), (x, y, prim, p)


def test_sphere_scene_shapes():
    s = scenes.sphere_scene()
    assert s.num_triangles == 3968 and len(s.meshes[0].vertices) == 2145
    out = oracle.render(s, oracle.RASTER_FIXED)
    st = out["stats"]
    assert st["num_visible"] > 1000 and st["covered_pixels"] > 20000
    # back half is culled: no visible triangle has a normal pointing away
    assert st["num_visible"] < s.num_triangles / 2
