"""Python binding of libgbr (include/gbr.h) -- the ctypes stub a host
application would bind, shaped like the reference's CUDARenderer
(CustomCUDARasterizer/CUDARenderer.h:31-141):

    r = Renderer(width, height)                 # CUDARenderer(windowHelper)
    r.setup_bins(nbx, nby, bw, bh, chunk)       # SetupBins
    tex = r.add_texture(rgba8)                  # CUDATextureManager::AddCUDATexture
    r.load_scene(scene)                         # LoadScene
    r.render(camera, cull, sample, vis)         # EnterValidRenderingState + Render
    colour, depth = r.readback()                # Present (headless)

There is no CPU fallback: constructing a Renderer without the CUDA library
or without a GPU raises.
"""
from __future__ import annotations

import ctypes as C
import os
from typing import Optional

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libgbr.so")

GBR_OK = 0
STATUS_NAMES = {0: "OK", 1: "INVALID_ARG", 2: "CUDA", 3: "OVERFLOW_RERUN", 4: "TIMEOUT",
                5: "OUT_OF_MEMORY", 6: "NOT_FOUND"}
BINNING_EXACT, BINNING_PREDICTED = 0, 1
TIMING_OFF, TIMING_STAGES, TIMING_TOTAL = 0, 1, 2

EXPORTED = ["gbr_create", "gbr_destroy", "gbr_setup_bins", "gbr_mesh_upload", "gbr_mesh_update_vertices",
            "gbr_mesh_bind_device", "gbr_mesh_set_world", "gbr_mesh_set_textures", "gbr_scene_clear",
            "gbr_texture_upload", "gbr_texture_remove", "gbr_set_lights", "gbr_set_binning", "gbr_set_predictor",
            "gbr_collect_bin_features", "gbr_predicted_capacities", "gbr_mlp_num_params", "gbr_mlp_predict", "gbr_mlp_loss_grad", "gbr_mlp_adam",
            "gbr_set_raster_params", "gbr_set_scan_wait", "gbr_set_bin_rows", "gbr_set_raster_staging", "gbr_set_timing", "gbr_render", "gbr_readback", "gbr_readback_ids", "gbr_device_buffers",
            "gbr_get_bins", "gbr_get_stats", "gbr_batch_create", "gbr_batch_destroy", "gbr_batch_add",
            "gbr_batch_set_view", "gbr_batch_set_config", "gbr_batch_get_config", "gbr_batch_autotune",
            "gbr_batch_set_timing", "gbr_batch_render", "gbr_batch_get_stats", "gbr_batch_scene_bins",
            "gbr_batch_readback", "gbr_batch_readback_all", "gbr_batch_get_bins", "gbr_render_noalloc", "gbr_draw_texture", "gbr_draw_texture_global", "gbr_obj_read_file", "gbr_obj_read_text",
            "gbr_obj_free", "gbr_last_error_string", "gbr_version"]


class GbrError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"gbr status {STATUS_NAMES.get(status, status)}: {msg}")
        self.status = status


class Camera(C.Structure):
    _fields_ = [("pos", C.c_float * 3), ("fwd", C.c_float * 3), ("view", C.c_float * 16), ("proj", C.c_float * 16)]


class Stats(C.Structure):
    _fields_ = [("num_triangles", C.c_uint64), ("num_visible", C.c_uint64), ("num_pairs", C.c_uint64),
                ("num_work_items", C.c_uint64), ("num_float_path", C.c_uint64),
                ("overflow_reruns", C.c_uint32), ("predicted_overflow", C.c_uint32),
                ("predicted_capacity", C.c_uint64),
                ("ms_setup", C.c_float), ("ms_bin", C.c_float), ("ms_raster", C.c_float), ("ms_total", C.c_float),
                ("ms_shade", C.c_float), ("count_blocks", C.c_uint32), ("raster_lanes", C.c_uint32),
                ("reserved", C.c_uint32)]


class Light(C.Structure):
    _fields_ = [("type", C.c_uint32), ("colour", C.c_float * 3), ("intensity", C.c_float), ("vec", C.c_float * 3)]


class ObjMesh(C.Structure):
    _fields_ = [("vertices", C.c_void_p), ("indices", C.c_void_p), ("num_vertices", C.c_uint32),
                ("num_indices", C.c_uint32), ("num_faces", C.c_uint32), ("vertex_type", C.c_int32)]


class BatchConfig(C.Structure):
    _fields_ = [("bin_size", C.c_uint32), ("queue_chunk", C.c_uint32), ("raster_ctas", C.c_uint32),
                ("raster_phase", C.c_uint32), ("raster_threads", C.c_uint32)]


class BatchStats(C.Structure):
    _fields_ = [("num_scenes", C.c_uint32), ("graph_captures", C.c_uint32), ("overflow_reruns", C.c_uint32),
                ("pad", C.c_uint32), ("num_triangles", C.c_uint64), ("num_visible", C.c_uint64),
                ("num_pairs", C.c_uint64), ("num_work_items", C.c_uint64), ("ms_frame", C.c_float),
                ("pad2", C.c_float)]


_LIB = None


def library_path() -> str:
    return LIB_PATH


def lib():
    """Load libgbr.so (built by build.py); raises if it is missing."""
    global _LIB
    if _LIB is None:
        if not os.path.exists(LIB_PATH):
            raise FileNotFoundError(f"{LIB_PATH} is missing: build it with custom-gpgpu-rasterizer_gb300/build.py")
        L = C.CDLL(LIB_PATH)
        vp, u32, i32, u64 = C.c_void_p, C.c_uint32, C.c_int32, C.c_uint64
        sig = {
            "gbr_create": [u32, u32, C.POINTER(vp)],
            "gbr_destroy": [vp],
            "gbr_setup_bins": [vp, u32, u32, u32, u32, u32],
            "gbr_mesh_upload": [vp, vp, u32, u32, vp, u32, u32, vp, vp, C.POINTER(u32)],
            "gbr_mesh_update_vertices": [vp, u32, vp, u32, vp],
            "gbr_mesh_bind_device": [vp, vp, u32, u32, vp, u32, u32, vp, vp, C.POINTER(u32)],
            "gbr_mesh_set_world": [vp, u32, vp],
            "gbr_mesh_set_textures": [vp, u32, vp],
            "gbr_scene_clear": [vp],
            "gbr_texture_upload": [vp, vp, u32, u32, C.POINTER(i32)],
            "gbr_texture_remove": [vp, i32],
            "gbr_set_lights": [vp, vp, u32],
            "gbr_set_binning": [vp, u32],
            "gbr_set_predictor": [vp, vp, u32, C.c_float, C.c_float, C.c_float],
            "gbr_collect_bin_features": [vp, C.POINTER(Camera), u32, u32, u32, vp, vp, vp],
            "gbr_predicted_capacities": [vp, vp, vp],
            "gbr_mlp_predict": [vp, vp, u32, vp, vp],
            "gbr_mlp_loss_grad": [vp, vp, vp, u32, vp, vp, vp],
            "gbr_mlp_adam": [vp, vp, vp, vp, vp, u32, C.c_float, C.c_float, vp],
            "gbr_set_raster_params": [vp, u32, u32],
            "gbr_set_timing": [vp, C.c_int],
            "gbr_set_scan_wait": [vp, u32, i32],
            "gbr_set_bin_rows": [vp, u32, u32],
            "gbr_set_raster_staging": [vp, u32],
            "gbr_render": [vp, C.POINTER(Camera), u32, u32, u32, vp],
            "gbr_readback": [vp, vp, vp, vp],
            "gbr_readback_ids": [vp, vp, vp],
            "gbr_device_buffers": [vp, C.POINTER(vp), C.POINTER(vp)],
            "gbr_get_bins": [vp, vp, vp, u64, C.POINTER(u64), vp],
            "gbr_get_stats": [vp, C.POINTER(Stats), vp],
            "gbr_render_noalloc": [vp, u32, u32, vp, u32, u32, vp, C.POINTER(Camera), u32, u32, u32, u32, u32, u32,
                                   u32, u32, u32, u32, vp, vp, vp, vp],
            "gbr_batch_create": [C.POINTER(vp)],
            "gbr_batch_destroy": [vp],
            "gbr_batch_add": [vp, vp, C.POINTER(Camera), u32, u32, u32, C.POINTER(u32)],
            "gbr_batch_set_view": [vp, u32, C.POINTER(Camera), u32, u32, u32],
            "gbr_batch_set_config": [vp, C.POINTER(BatchConfig)],
            "gbr_batch_get_config": [vp, C.POINTER(BatchConfig)],
            "gbr_batch_autotune": [vp, vp, u32, vp, u32, vp, u32, vp, u32, u32, vp, C.POINTER(BatchConfig)],
            "gbr_batch_set_timing": [vp, C.c_int],
            "gbr_batch_render": [vp, vp],
            "gbr_batch_get_stats": [vp, C.POINTER(BatchStats), vp],
            "gbr_batch_scene_bins": [vp, u32, C.POINTER(u32), C.POINTER(u32)],
            "gbr_batch_readback": [vp, u32, vp, vp, vp, vp],
            "gbr_batch_readback_all": [vp, vp, vp],
            "gbr_batch_get_bins": [vp, u32, vp, vp, u64, C.POINTER(u64), vp],
            "gbr_draw_texture": [vp, C.c_int32, vp],
            "gbr_draw_texture_global": [vp, C.c_int32, C.c_int, u32, vp],
            "gbr_obj_read_file": [C.c_char_p, C.c_int, C.POINTER(ObjMesh)],
            "gbr_obj_read_text": [C.c_char_p, C.c_size_t, C.c_int, C.POINTER(ObjMesh)],
        }
        for name, args in sig.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = C.c_int
        L.gbr_last_error_string.restype = C.c_char_p
        L.gbr_last_error_string.argtypes = []
        L.gbr_version.restype = C.c_uint32
        L.gbr_version.argtypes = []
        L.gbr_obj_free.restype = None
        L.gbr_obj_free.argtypes = [C.POINTER(ObjMesh)]
        L.gbr_mlp_num_params.restype = C.c_uint32
        L.gbr_mlp_num_params.argtypes = []
        _LIB = L
    return _LIB


def check(status: int):
    if status != GBR_OK:
        raise GbrError(status, lib().gbr_last_error_string().decode(errors="replace"))


def read_obj(source, invert_y: bool = False, text: bool = False):
    """ObjParser::ReadFromObjFile (ObjParser.cpp) through gbr_obj_read_file, or
    gbr_obj_read_text when `text` (source: str or bytes).  Returns
    (vertices: float32 (n, 14) IVertex rows [p3 uv2 n3 tan3 c3], indices:
    uint32, vertex type: GBR_VT_* flags, faces read)."""
    L = lib()
    m = ObjMesh()
    if text:
        data = source.encode() if isinstance(source, str) else bytes(source)
        check(L.gbr_obj_read_text(data, len(data), 1 if invert_y else 0, C.byref(m)))
    else:
        check(L.gbr_obj_read_file(os.fsencode(source), 1 if invert_y else 0, C.byref(m)))
    try:
        nv, ni = m.num_vertices, m.num_indices
        verts = np.ctypeslib.as_array(C.cast(m.vertices, C.POINTER(C.c_float)), shape=(max(nv, 1) * 14,))
        verts = verts[:nv * 14].reshape(nv, 14).copy()
        idx = np.ctypeslib.as_array(C.cast(m.indices, C.POINTER(C.c_uint32)), shape=(max(ni, 1),))[:ni].copy()
        return verts, idx, int(m.vertex_type), int(m.num_faces)
    finally:
        L.gbr_obj_free(C.byref(m))


def _ptr(a: Optional[np.ndarray]):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def _f16(m) -> C.Array:
    return (C.c_float * 16)(*[float(x) for x in np.asarray(m, np.float32).reshape(16)])


def make_camera(cam) -> Camera:
    c = Camera()
    c.pos[:] = [float(x) for x in cam.pos]
    c.fwd[:] = [float(x) for x in cam.fwd]
    c.view[:] = [float(x) for x in cam.view]
    c.proj[:] = [float(x) for x in cam.proj]
    return c


class Renderer:
    """Headless CUDARenderer on the current CUDA device."""

    def __init__(self, width: int, height: int):
        self._lib = lib()
        h = C.c_void_p()
        check(self._lib.gbr_create(width, height, C.byref(h)))
        self.h = h
        self.width, self.height = width, height
        self.nbx = self.nby = 0
        self._keep = []

    def close(self):
        if self.h:
            self._lib.gbr_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # -- setup ---------------------------------------------------------
    def setup_bins(self, nbx: int, nby: int, bw: int, bh: int, chunk: int = 4096):
        check(self._lib.gbr_setup_bins(self.h, nbx, nby, bw, bh, chunk))
        self.nbx, self.nby = nbx, nby

    def add_texture(self, rgba8: np.ndarray) -> int:
        t = np.ascontiguousarray(rgba8, np.uint32)
        tid = C.c_int32()
        check(self._lib.gbr_texture_upload(self.h, _ptr(t), t.shape[1], t.shape[0], C.byref(tid)))
        return tid.value

    def remove_texture(self, tid: int):
        check(self._lib.gbr_texture_remove(self.h, tid))

    def add_mesh(self, vertices: np.ndarray, vertex_format: int, indices=None, topology: int = 0,
                 world=None, tex_ids=(-1, -1, -1, -1)) -> int:
        v = np.ascontiguousarray(vertices)
        ix = None if indices is None else np.ascontiguousarray(indices, np.uint32)
        w = _f16(np.eye(4, dtype=np.float32) if world is None else world)
        ids = (C.c_int32 * 4)(*tex_ids)
        mid = C.c_uint32()
        check(self._lib.gbr_mesh_upload(self.h, _ptr(v), len(v), vertex_format, _ptr(ix),
                                        0 if ix is None else len(ix), topology, w, ids, C.byref(mid)))
        return mid.value

    def bind_mesh_device(self, d_vertices: int, num_vertices: int, vertex_format: int, d_indices: int = 0,
                         num_indices: int = 0, topology: int = 0, world=None, tex_ids=(-1, -1, -1, -1)) -> int:
        w = _f16(np.eye(4, dtype=np.float32) if world is None else world)
        ids = (C.c_int32 * 4)(*tex_ids)
        mid = C.c_uint32()
        check(self._lib.gbr_mesh_bind_device(self.h, C.c_void_p(d_vertices), num_vertices, vertex_format,
                                             C.c_void_p(d_indices) if d_indices else None, num_indices, topology,
                                             w, ids, C.byref(mid)))
        return mid.value

    def update_vertices(self, mesh_id: int, host_ptr: int, num_vertices: int, stream: int = 0):
        check(self._lib.gbr_mesh_update_vertices(self.h, mesh_id, C.c_void_p(host_ptr), num_vertices,
                                                 C.c_void_p(stream) if stream else None))

    def clear_scene(self):
        check(self._lib.gbr_scene_clear(self.h))

    def load_scene(self, scene, chunk: int = 4096):
        """LoadScene: bins from the scene, textures, meshes."""
        self.setup_bins(scene.num_bins_x, scene.num_bins_y, scene.bin_w, scene.bin_h, chunk)
        self.clear_scene()
        self.scene = scene
        for m in scene.meshes:
            tex_ids = [self.add_texture(t) if t is not None else -1 for t in m.textures]
            self.add_mesh(m.vertices, m.vertex_format, m.indices, m.topology, m.world, tex_ids)
        self.set_lights(getattr(scene, "lights", []) or [])

    def set_lights(self, lights):
        """Scene lights (objects with type, colour, intensity, vec); empty:
        the reference shader's constant light."""
        arr = (Light * max(len(lights), 1))()
        for k, lt in enumerate(lights):
            arr[k].type = int(lt.type)
            arr[k].colour[:] = [float(x) for x in lt.colour]
            arr[k].intensity = float(lt.intensity)
            arr[k].vec[:] = [float(x) for x in lt.vec]
        check(self._lib.gbr_set_lights(self.h, C.cast(arr, C.c_void_p) if lights else None, len(lights)))

    def set_binning(self, method: int):
        check(self._lib.gbr_set_binning(self.h, method))

    def set_raster_params(self, phase: int = 0, ctas_per_sm: int = 0):
        check(self._lib.gbr_set_raster_params(self.h, phase, ctas_per_sm))

    def set_raster_staging(self, tma: bool):
        """Setup records staged by bulk asynchronous copies (TMA) or loads."""
        check(self._lib.gbr_set_raster_staging(self.h, 1 if tma else 0))

    def set_bin_rows(self, row0: int = 0, row1: int = 0):
        """This renderer's share of a frame split by bin rows: bin rows
        [row0, row1) ((0, 0): every row)."""
        check(self._lib.gbr_set_bin_rows(self.h, row0, row1))

    def set_scan_wait(self, spin_limit: int = 0, silent_tile: int = -1):
        """Test hook: bound of the bin scan's waits (0: the library's) and a
        tile of 1024 bins that publishes nothing (-1: none)."""
        check(self._lib.gbr_set_scan_wait(self.h, spin_limit, silent_tile))

    def set_timing(self, on: bool, total_only: bool = False):
        """CUDA-event times in stats(): per stage (an event between every
        stage), or with total_only the frame time alone, which leaves the
        stages' launches free to overlap."""
        mode = (TIMING_TOTAL if total_only else TIMING_STAGES) if on else TIMING_OFF
        check(self._lib.gbr_set_timing(self.h, mode))

    # -- frame ---------------------------------------------------------
    def render(self, camera, cull: int, sample: int, vis: int, stream: int = 0):
        cam = camera if isinstance(camera, Camera) else make_camera(camera)
        check(self._lib.gbr_render(self.h, C.byref(cam), cull, sample, vis, C.c_void_p(stream) if stream else None))

    def render_scene(self, scene, stream: int = 0):
        self.render(scene.camera, scene.cull, scene.sample, scene.vis, stream)

    def readback(self, colour: Optional[np.ndarray] = None, depth: Optional[np.ndarray] = None, stream: int = 0,
                 want_depth: bool = True):
        n = self.width * self.height
        colour = np.empty(n, np.uint32) if colour is None else colour
        if want_depth and depth is None:
            depth = np.empty(n, np.float32)
        check(self._lib.gbr_readback(self.h, _ptr(colour), _ptr(depth) if want_depth else None,
                                     C.c_void_p(stream) if stream else None))
        c = colour.reshape(self.height, self.width)
        return (c, depth.reshape(self.height, self.width)) if want_depth else (c, None)

    def draw_texture(self, tex_id: int, stream: int = 0):
        """DrawTexture: the texture stretched over the colour buffer through
        the texture hardware (readback() returns it)."""
        check(self._lib.gbr_draw_texture(self.h, tex_id, _stream(stream)))

    def draw_texture_global(self, tex_id: int, stretch_to_window: bool = True, sample: int = 0, stream: int = 0):
        """DrawTextureGlobal: the shader's sampler over the colour buffer."""
        check(self._lib.gbr_draw_texture_global(self.h, tex_id, 1 if stretch_to_window else 0, sample,
                                                _stream(stream)))

    def predicted_capacities(self, stream: int = 0) -> np.ndarray:
        """Per-bin capacities of the last predicted-binning frame."""
        out = np.empty(self.nbx * self.nby, np.uint32)
        check(self._lib.gbr_predicted_capacities(self.h, _ptr(out), _stream(stream)))
        return out

    def readback_ids(self, stream: int = 0) -> np.ndarray:
        ids = np.empty(self.width * self.height, np.uint32)
        check(self._lib.gbr_readback_ids(self.h, _ptr(ids), C.c_void_p(stream) if stream else None))
        return ids.reshape(self.height, self.width)

    def device_buffers(self):
        c, d = C.c_void_p(), C.c_void_p()
        check(self._lib.gbr_device_buffers(self.h, C.byref(c), C.byref(d)))
        return c.value, d.value

    def get_bins(self, stream: int = 0):
        """(offsets[num_bins+1], ids) of the last frame; ids sorted within each bin."""
        nb = self.nbx * self.nby
        offsets = np.empty(nb + 1, np.uint32)
        n = C.c_uint64()
        s = C.c_void_p(stream) if stream else None
        check(self._lib.gbr_get_bins(self.h, _ptr(offsets), None, 0, C.byref(n), s))
        ids = np.empty(max(n.value, 1), np.uint32)
        check(self._lib.gbr_get_bins(self.h, _ptr(offsets), _ptr(ids), n.value, C.byref(n), s))
        ids = ids[: n.value]
        bin_of = np.repeat(np.arange(nb, dtype=np.uint32), np.diff(offsets.astype(np.int64)))
        return offsets, ids[np.lexsort((ids, bin_of))]

    def stats(self, stream: int = 0) -> dict:
        st = Stats()
        check(self._lib.gbr_get_stats(self.h, C.byref(st), C.c_void_p(stream) if stream else None))
        return {k: getattr(st, k) for k, _ in Stats._fields_}


def _stream(stream: int):
    return C.c_void_p(stream) if stream else None


def _u32_list(values):
    if values is None:
        return None, 0
    arr = (C.c_uint32 * len(values))(*[int(v) for v in values])
    return arr, len(values)


class Batch:
    """Many renderers' scenes rendered as one batch frame (gbr_batch_*): one
    persistent launch chain over the (scene, bin) work items of every scene,
    replayed from a CUDA graph."""

    def __init__(self):
        self._lib = lib()
        h = C.c_void_p()
        check(self._lib.gbr_batch_create(C.byref(h)))
        self.h = h
        self.renderers = []

    def close(self):
        if self.h:
            self._lib.gbr_batch_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def add(self, renderer: Renderer, camera, cull: int, sample: int, vis: int) -> int:
        cam = camera if isinstance(camera, Camera) else make_camera(camera)
        idx = C.c_uint32()
        check(self._lib.gbr_batch_add(self.h, renderer.h, C.byref(cam), cull, sample, vis, C.byref(idx)))
        self.renderers.append(renderer)
        return idx.value

    def add_scene(self, renderer: Renderer, scene) -> int:
        return self.add(renderer, scene.camera, scene.cull, scene.sample, scene.vis)

    def set_view(self, index: int, camera, cull: int, sample: int, vis: int):
        cam = camera if isinstance(camera, Camera) else make_camera(camera)
        check(self._lib.gbr_batch_set_view(self.h, index, C.byref(cam), cull, sample, vis))

    def set_config(self, bin_size: int = 16, queue_chunk: int = 64, raster_ctas: int = 0, raster_phase: int = 0,
                   raster_threads: int = 0):
        cfg = BatchConfig(bin_size, queue_chunk, raster_ctas, raster_phase, raster_threads)
        check(self._lib.gbr_batch_set_config(self.h, C.byref(cfg)))

    def config(self) -> dict:
        cfg = BatchConfig()
        check(self._lib.gbr_batch_get_config(self.h, C.byref(cfg)))
        return {k: getattr(cfg, k) for k, _ in BatchConfig._fields_}

    def autotune(self, bin_sizes=(8, 16, 32), chunks=(128, 512, 2048), raster_ctas=None, frames: int = 2,
                 stream: int = 0, raster_threads=None) -> dict:
        b, nb = _u32_list(bin_sizes)
        c, nc = _u32_list(chunks)
        r, nr = _u32_list(raster_ctas)
        t, nt = _u32_list(raster_threads)
        best = BatchConfig()
        check(self._lib.gbr_batch_autotune(self.h, b, nb, c, nc, r, nr, t, nt, frames, _stream(stream),
                                           C.byref(best)))
        return {k: getattr(best, k) for k, _ in BatchConfig._fields_}

    def set_timing(self, on: bool):
        check(self._lib.gbr_batch_set_timing(self.h, 1 if on else 0))

    def render(self, stream: int = 0):
        check(self._lib.gbr_batch_render(self.h, _stream(stream)))

    def stats(self, stream: int = 0) -> dict:
        st = BatchStats()
        check(self._lib.gbr_batch_get_stats(self.h, C.byref(st), _stream(stream)))
        return {k: getattr(st, k) for k, _ in BatchStats._fields_ if not k.startswith("pad")}

    def readback(self, index: int, stream: int = 0):
        """(colour, depth, ids) of scene `index`, each [height, width]."""
        r = self.renderers[index]
        n = r.width * r.height
        colour = np.empty(n, np.uint32)
        depth = np.empty(n, np.float32)
        ids = np.empty(n, np.uint32)
        check(self._lib.gbr_batch_readback(self.h, index, _ptr(colour), _ptr(depth), _ptr(ids), _stream(stream)))
        shp = (r.height, r.width)
        return colour.reshape(shp), depth.reshape(shp), ids.reshape(shp)

    def readback_all(self, colours=None, stream: int = 0):
        """Every scene's colour buffer, [height, width] each, with one wait:
        into `colours` (arrays of the scenes' sizes, or host pointers; None
        entries are skipped) or into new arrays."""
        if colours is None:
            colours = [np.empty(r.width * r.height, np.uint32) for r in self.renderers]
        ptrs = (C.c_void_p * len(colours))(*[None if c is None else (c if isinstance(c, int) else _ptr(c))
                                              for c in colours])
        check(self._lib.gbr_batch_readback_all(self.h, ptrs, _stream(stream)))
        return [c.reshape(r.height, r.width) if isinstance(c, np.ndarray) else c
                for c, r in zip(colours, self.renderers)]

    def get_bins(self, index: int, stream: int = 0):
        """(offsets[num_bins+1], ids) of scene `index`; ids sorted within each bin."""
        nbx, nby = C.c_uint32(), C.c_uint32()
        check(self._lib.gbr_batch_scene_bins(self.h, index, C.byref(nbx), C.byref(nby)))
        nb = nbx.value * nby.value
        offsets = np.empty(nb + 1, np.uint32)
        n = C.c_uint64()
        s = _stream(stream)
        check(self._lib.gbr_batch_get_bins(self.h, index, _ptr(offsets), None, 0, C.byref(n), s))
        ids = np.empty(max(n.value, 1), np.uint32)
        check(self._lib.gbr_batch_get_bins(self.h, index, _ptr(offsets), _ptr(ids), n.value, C.byref(n), s))
        ids = ids[: n.value]
        bin_of = np.repeat(np.arange(nb, dtype=np.uint32), np.diff(offsets.astype(np.int64)))
        return offsets, ids[np.lexsort((ids, bin_of))]
