"""ctypes wrapper of the CPU oracle (TEST INFRASTRUCTURE ONLY).

Loaded by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg to
check or time against; never by the product path.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build_oracle

RASTER_REFERENCE = 0
RASTER_FIXED = 1


MAX_LIGHTS = 8


class OrcLight(C.Structure):
    _fields_ = [("type", C.c_uint32), ("colour", C.c_float * 3), ("intensity", C.c_float), ("vec", C.c_float * 3)]


class OrcFrame(C.Structure):
    _fields_ = [("width", C.c_uint32), ("height", C.c_uint32),
                ("num_bins_x", C.c_uint32), ("num_bins_y", C.c_uint32),
                ("bin_w", C.c_uint32), ("bin_h", C.c_uint32),
                ("cull", C.c_uint32), ("sample", C.c_uint32), ("vis", C.c_uint32),
                ("raster_mode", C.c_uint32), ("clear_colour32", C.c_uint32), ("num_threads", C.c_uint32),
                ("bin_stride", C.c_uint32), ("bin_phase", C.c_uint32),
                ("cam_pos", C.c_float * 3), ("cam_fwd", C.c_float * 3),
                ("view", C.c_float * 16), ("proj", C.c_float * 16),
                ("num_lights", C.c_uint32), ("lights", OrcLight * MAX_LIGHTS),
                ("bin_row0", C.c_uint32), ("bin_row1", C.c_uint32)]


class OrcMesh(C.Structure):
    _fields_ = [("vertices", C.c_void_p), ("num_vertices", C.c_uint32), ("vertex_format", C.c_uint32),
                ("indices", C.c_void_p), ("num_indices", C.c_uint32), ("topology", C.c_uint32),
                ("world", C.c_float * 16), ("tex", C.c_void_p * 4),
                ("tex_w", C.c_uint32 * 4), ("tex_h", C.c_uint32 * 4)]


class OrcStats(C.Structure):
    _fields_ = [("num_triangles", C.c_uint64), ("num_visible", C.c_uint64), ("num_pairs", C.c_uint64),
                ("num_float_path", C.c_uint64), ("fragments", C.c_uint64), ("covered_pixels", C.c_uint64)]


class OrcProbe(C.Structure):
    _fields_ = [("covered_ref", C.c_int32), ("covered_fixed", C.c_int32),
                ("e_ref", C.c_float * 3), ("e_bound", C.c_float * 3),
                ("z_ref", C.c_float), ("z_fixed", C.c_float),
                ("visible", C.c_int32), ("float_path", C.c_int32)]


_LIB = None


def lib():
    global _LIB
    if _LIB is None:
        path = build_oracle.build()
        _LIB = C.CDLL(path)
        _LIB.orc_render.restype = C.c_int
        _LIB.orc_render.argtypes = [C.POINTER(OrcFrame), C.POINTER(OrcMesh), C.c_uint32,
                                    C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                    C.c_uint64, C.POINTER(OrcStats)]
        _LIB.orc_probe.restype = C.c_int
        _LIB.orc_probe.argtypes = [C.POINTER(OrcFrame), C.POINTER(OrcMesh), C.c_uint32,
                                   C.c_uint32, C.c_uint32, C.c_uint32, C.POINTER(OrcProbe)]
        _LIB.orc_rgba_from_colour.restype = C.c_uint32
        _LIB.orc_cull.restype = C.c_int
        _LIB.orc_frustum_visible.restype = C.c_int
    return _LIB


def _fptr(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p)


class _Prepared:
    """Keeps the numpy buffers alive while the C structs point at them."""

    def __init__(self, scene, raster_mode: int, num_threads: int, bin_stride: int = 0, bin_phase: int = 0,
                 bin_rows=(0, 0)):
        f = OrcFrame()
        f.width, f.height = scene.width, scene.height
        f.num_bins_x, f.num_bins_y = scene.num_bins_x, scene.num_bins_y
        f.bin_w, f.bin_h = scene.bin_w, scene.bin_h
        f.cull, f.sample, f.vis = scene.cull, scene.sample, scene.vis
        f.raster_mode = raster_mode
        f.clear_colour32 = 0x003F3F3F
        f.num_threads = num_threads
        f.bin_stride, f.bin_phase = bin_stride, bin_phase
        f.bin_row0, f.bin_row1 = bin_rows
        cam = scene.camera
        f.cam_pos[:] = [float(x) for x in cam.pos]
        f.cam_fwd[:] = [float(x) for x in cam.fwd]
        f.view[:] = [float(x) for x in cam.view]
        f.proj[:] = [float(x) for x in cam.proj]
        lights = list(getattr(scene, "lights", []) or [])
        if len(lights) > MAX_LIGHTS:
            raise ValueError(f"at most {MAX_LIGHTS} lights")
        f.num_lights = len(lights)
        for k, lt in enumerate(lights):
            f.lights[k].type = lt.type
            f.lights[k].colour[:] = [float(x) for x in lt.colour]
            f.lights[k].intensity = float(lt.intensity)
            f.lights[k].vec[:] = [float(x) for x in lt.vec]
        self.frame = f
        self.keep = []
        meshes = (OrcMesh * max(len(scene.meshes), 1))()
        for i, m in enumerate(scene.meshes):
            om = meshes[i]
            v = np.ascontiguousarray(m.vertices)
            self.keep.append(v)
            om.vertices = _fptr(v)
            om.num_vertices = len(v)
            om.vertex_format = m.vertex_format
            if m.indices is not None:
                ix = np.ascontiguousarray(m.indices, dtype=np.uint32)
                self.keep.append(ix)
                om.indices = _fptr(ix)
                om.num_indices = len(ix)
            om.topology = m.topology
            om.world[:] = [float(x) for x in m.world]
            for k in range(4):
                t = m.textures[k]
                if t is not None:
                    t = np.ascontiguousarray(t, dtype=np.uint32)
                    self.keep.append(t)
                    om.tex[k] = t.ctypes.data
                    om.tex_w[k] = t.shape[1]
                    om.tex_h[k] = t.shape[0]
        self.meshes = meshes
        self.num_meshes = len(scene.meshes)


def render(scene, raster_mode: int = RASTER_FIXED, num_threads: int = 0, want_bins: bool = True,
           want_image: bool = True, bin_stride: int = 0, bin_phase: int = 0, bin_rows=(0, 0)):
    """Render one frame; returns dict(colour, depth, ids, offsets, bins, stats).
    bin_stride > 1 rasterises only bins b with b % bin_stride == bin_phase;
    bin_rows = (r0, r1) only bin rows [r0, r1) (one GPU's band of a frame
    split by bin rows; pixels of other rows are the clear colour);
    want_image=False runs the vertex stage and binning only."""
    L = lib()
    if num_threads <= 0:
        num_threads = os.cpu_count() or 1
    P = _Prepared(scene, raster_mode, num_threads, bin_stride, bin_phase, bin_rows)
    n = scene.width * scene.height
    colour = np.empty(n, np.uint32)
    depth = np.empty(n, np.float32)
    ids = np.empty(n, np.uint32)
    nb = scene.num_bins_x * scene.num_bins_y
    offsets = np.zeros(nb + 1, np.uint32)
    stats = OrcStats()
    cap = 0
    bins = np.zeros(1, np.uint32)
    if want_bins:
        rc = L.orc_render(C.byref(P.frame), P.meshes, P.num_meshes, None, None, None, _fptr(offsets), None, 0,
                          C.byref(stats))
        if rc != 0:
            raise RuntimeError(f"orc_render failed: {rc}")
        cap = int(offsets[-1])
        bins = np.zeros(max(cap, 1), np.uint32)
    img = [_fptr(colour), _fptr(depth), _fptr(ids)] if want_image else [None, None, None]
    rc = L.orc_render(C.byref(P.frame), P.meshes, P.num_meshes, *img,
                      _fptr(offsets), _fptr(bins) if want_bins else None, cap, C.byref(stats))
    if rc != 0:
        raise RuntimeError(f"orc_render failed: {rc}")
    st = {k: int(getattr(stats, k)) for k, _ in OrcStats._fields_}
    return {"colour": colour.reshape(scene.height, scene.width), "depth": depth.reshape(scene.height, scene.width),
            "ids": ids.reshape(scene.height, scene.width), "offsets": offsets, "bins": bins[:cap], "stats": st}


def probe(scene, prim: int, px: int, py: int):
    L = lib()
    P = _Prepared(scene, RASTER_FIXED, 1)
    out = OrcProbe()
    rc = L.orc_probe(C.byref(P.frame), P.meshes, P.num_meshes, prim, px, py, C.byref(out))
    if rc != 0:
        raise RuntimeError(f"orc_probe failed: {rc}")
    return {"covered_ref": bool(out.covered_ref), "covered_fixed": bool(out.covered_fixed),
            "e_ref": list(out.e_ref), "e_bound": list(out.e_bound), "z_ref": out.z_ref, "z_fixed": out.z_fixed,
            "visible": bool(out.visible), "float_path": bool(out.float_path)}


def vs_position(wvp, p):
    out = (C.c_float * 4)()
    lib().orc_vs_position((C.c_float * 16)(*wvp), (C.c_float * 3)(*p), out)
    return np.array(out[:], np.float32)


def mat4_mul(a, b):
    out = (C.c_float * 16)()
    lib().orc_mat4_mul((C.c_float * 16)(*a), (C.c_float * 16)(*b), out)
    return np.array(out[:], np.float32)


def cull(p0, p1, p2, fwd, mode):
    f3 = C.c_float * 3
    return bool(lib().orc_cull(f3(*p0), f3(*p1), f3(*p2), f3(*fwd), mode))


def frustum_visible(p0, p1, p2):
    f3 = C.c_float * 3
    return bool(lib().orc_frustum_visible(f3(*p0), f3(*p1), f3(*p2)))


def bin_rect(ndc_xy, width, height, nbx, nby, bw, bh):
    out = (C.c_int32 * 4)()
    lib().orc_bin_rect((C.c_float * 6)(*ndc_xy), width, height, nbx, nby, bw, bh, out)
    return tuple(out[:])


def sample(tex: np.ndarray, u: float, v: float, mode: int):
    t = np.ascontiguousarray(tex, np.uint32)
    out = (C.c_float * 3)()
    lib().orc_sample(_fptr(t), t.shape[1], t.shape[0], C.c_float(u), C.c_float(v), mode, out)
    return np.array(out[:], np.float32)


def rgba_from_colour(rgb):
    return int(lib().orc_rgba_from_colour((C.c_float * 3)(*rgb)))
