"""gbr_render_noalloc: the entry point for callers that may not allocate
device memory while they render (a host that owns a fixed device-memory
budget, a real-time loop that cannot take cudaMalloc's implicit
synchronisation, a process under a hard memory cap).  It renders from the
caller's device buffers into the caller's device buffers and keeps its own
scratch in one static device array, shared by every call.

Checked here through the C ABI: calls in a row, on different scenes -- a
non-indexed soup of compact vertices (two resolutions, two cull modes), the
indexed UV sphere of 56-byte IVertex vertices, and an IVertex triangle
strip -- each match the regular entry point (gbr_create / gbr_render /
gbr_readback / gbr_readback_ids) within the tolerance the parity tests use
(colour within 1 LSB per channel, depth within 1e-6 relative, winning
primitive ids identical), so nothing left in the shared scratch by one call
leaks into the next; and inputs beyond the scratch's limits are refused with
an error before any GPU work.  This file is collected last so
that a run stopping at the first failure has already run every other test.
"""
import ctypes as C

import numpy as np
import pytest

import scenes

pytestmark = pytest.mark.gpu


def _channels(c):
    c = c.astype(np.int64)
    return np.stack([c & 255, (c >> 8) & 255, (c >> 16) & 255, (c >> 24) & 255], -1)


def _noalloc(gbr, scene, torch, dev):
    L = gbr.lib()
    mesh = scene.meshes[0]
    d_v = torch.from_numpy(mesh.vertices.view(np.uint8).copy()).to(dev)
    d_ix = None
    if mesh.indices is not None:
        d_ix = torch.from_numpy(np.ascontiguousarray(mesh.indices, np.uint32).view(np.int32)).to(dev)
    npx = scene.width * scene.height
    d_col = torch.empty(npx, dtype=torch.int32, device=dev)
    d_dep = torch.empty(npx, dtype=torch.float32, device=dev)
    d_ids = torch.empty(npx, dtype=torch.int32, device=dev)
    cam = gbr.make_camera(scene.camera)
    world = (C.c_float * 16)(*[float(x) for x in mesh.world])
    st = L.gbr_render_noalloc(C.c_void_p(d_v.data_ptr()), len(mesh.vertices), mesh.vertex_format,
                              C.c_void_p(d_ix.data_ptr()) if d_ix is not None else None,
                              0 if d_ix is None else len(mesh.indices), mesh.topology, world, C.byref(cam),
                              scene.width, scene.height, scene.num_bins_x, scene.num_bins_y, scene.bin_w,
                              scene.bin_h, 256, scene.cull, scene.sample, scene.vis,
                              C.c_void_p(d_col.data_ptr()), C.c_void_p(d_dep.data_ptr()),
                              C.c_void_p(d_ids.data_ptr()), None)
    assert st == 0, L.gbr_last_error_string()
    torch.cuda.synchronize(dev)
    colour = d_col.cpu().numpy().view(np.uint32).reshape(scene.height, scene.width)
    depth = d_dep.cpu().numpy().reshape(scene.height, scene.width)
    ids = d_ids.cpu().numpy().view(np.uint32).reshape(scene.height, scene.width)
    return colour, depth, ids


def _regular(gbr, scene):
    with gbr.Renderer(scene.width, scene.height) as r:
        r.load_scene(scene)
        r.render_scene(scene)
        colour, depth = r.readback()
        return colour, depth, r.readback_ids()


def _assert_close(a, b):
    (a_colour, a_depth, a_ids), (b_colour, b_depth, b_ids) = a, b
    assert np.array_equal(a_ids, b_ids), f"{(a_ids != b_ids).sum()} pixels with a different winner"
    assert np.abs(_channels(a_colour) - _channels(b_colour)).max() <= 1
    za, zb = a_depth.astype(np.float64), b_depth.astype(np.float64)
    assert (np.abs(za - zb) <= 1e-6 * np.maximum(np.abs(zb), 1e-30)).all()


def _untextured_sphere():
    s = scenes.sphere_scene(640, 480)
    for m in s.meshes:
        m.textures = [None] * 4
    return s


def test_noalloc_matches_the_allocating_entry_point_on_calls_in_a_row(gbr_lib, cuda_device):
    import torch
    cases = [scenes.soup_scene(20000, 512, 384, seed=31),
             scenes.soup_scene(12000, 400, 300, seed=32, cull=scenes.CULL_BACKFACE),
             _untextured_sphere(),          # indexed triangle list, IVertex
             scenes.strip_grid_scene()]     # indexed triangle strip, IVertex
    for scene in cases:
        got = _noalloc(gbr_lib, scene, torch, cuda_device)
        _assert_close(got, _regular(gbr_lib, scene))
        assert (got[2] != 0xFFFFFFFF).sum() > 1000  # the frame is actually drawn


def test_noalloc_refuses_inputs_beyond_its_limits(gbr_lib, cuda_device):
    import torch
    L = gbr_lib.lib()
    dev = cuda_device
    big = scenes.soup_vertices(70000, 64, 64, seed=1)
    d_v = torch.from_numpy(big.view(np.uint8).copy()).to(dev)
    out = torch.empty(64 * 64, dtype=torch.int32, device=dev)
    cam = gbr_lib.make_camera(scenes.identity_camera())
    world = (C.c_float * 16)(*[float(x) for x in scenes.identity16()])
    st = L.gbr_render_noalloc(C.c_void_p(d_v.data_ptr()), len(big), 1, None, 0, 0, world, C.byref(cam), 64, 64,
                              4, 4, 16, 16, 256, 2, 0, 0, C.c_void_p(out.data_ptr()), C.c_void_p(out.data_ptr()), None,
                              None)
    assert st == 1 and b"65536" in L.gbr_last_error_string()
    st = L.gbr_render_noalloc(C.c_void_p(d_v.data_ptr()), 300, 1, None, 0, 0, world, C.byref(cam), 2048, 1024,
                              128, 64, 16, 16, 256, 2, 0, 0, C.c_void_p(out.data_ptr()), C.c_void_p(out.data_ptr()), None,
                              None)
    assert st == 1 and b"pixels" in L.gbr_last_error_string()
