"""Scene and result files of the reference harness (TEST INFRASTRUCTURE ONLY).

write_scene() serialises a scenes.Scene for oracle/ref/ref_harness.cu;
read_result() parses what the harness writes back.  Compact soup vertices
are widened to the reference's IVertex (colour = byte / 255, as
RGBA::GetRGBColor reads it); non-indexed meshes get an explicit 0..n-1
index buffer, which TA_Kernel reads three at a time.
"""
import struct

import numpy as np

SCENE_MAGIC = 0x53524247
RESULT_MAGIC = 0x4F524247


def _ivertex(mesh):
    import scenes
    v = mesh.vertices
    return v if v.dtype == scenes.IVERTEX56 else scenes.pos3_to_ivertex(v)


def write_scene(scene, path, queue_max: int = 256):
    tex_list, mesh_tex = [], []
    for m in scene.meshes:
        ids = []
        for t in m.textures:
            if t is None:
                ids.append(-1)
            else:
                tex_list.append(np.ascontiguousarray(t, np.uint32))
                ids.append(len(tex_list) - 1)
        mesh_tex.append(ids)
    cam = scene.camera
    with open(path, "wb") as f:
        f.write(struct.pack("<11I", SCENE_MAGIC, scene.width, scene.height, scene.num_bins_x, scene.num_bins_y,
                            scene.bin_w, scene.bin_h, queue_max, scene.cull, scene.sample, scene.vis))
        f.write(np.asarray(cam.pos, np.float32).tobytes())
        f.write(np.asarray(cam.fwd, np.float32).tobytes())
        f.write(np.asarray(cam.view, np.float32).tobytes())
        f.write(np.asarray(cam.proj, np.float32).tobytes())
        f.write(struct.pack("<I", len(tex_list)))
        for t in tex_list:
            f.write(struct.pack("<II", t.shape[1], t.shape[0]))
            f.write(t.tobytes())
        f.write(struct.pack("<I", len(scene.meshes)))
        for m, ids in zip(scene.meshes, mesh_tex):
            v = np.ascontiguousarray(_ivertex(m))
            f.write(struct.pack("<I", len(v)))
            f.write(v.tobytes())
            ix = np.arange(len(v) - len(v) % 3, dtype=np.uint32) if m.indices is None else np.asarray(m.indices, np.uint32)
            f.write(struct.pack("<I", len(ix)))
            f.write(ix.tobytes())
            f.write(struct.pack("<I", m.topology))
            f.write(np.asarray(m.world, np.float32).tobytes())
            f.write(struct.pack("<4i", *ids))


def read_result(path):
    data = open(path, "rb").read()
    magic, w, h, visible = struct.unpack_from("<4I", data, 0)
    assert magic == RESULT_MAGIC, "not a harness result"
    off = 16
    n = w * h
    colour = np.frombuffer(data, np.uint32, n, off).reshape(h, w).copy()
    off += 4 * n
    z = np.frombuffer(data, np.float32, n, off).reshape(h, w).copy()
    off += 4 * n
    (npairs,) = struct.unpack_from("<Q", data, off)
    off += 8
    pairs = np.frombuffer(data, np.uint32, 2 * npairs, off).reshape(-1, 2).copy()
    return {"colour": colour, "z": z, "pairs": pairs, "visible": visible}


def bins_from_pairs(pairs, num_bins):
    """(offsets[num_bins+1], ids sorted within each bin) from (bin, prim) pairs."""
    order = np.lexsort((pairs[:, 1], pairs[:, 0]))
    p = pairs[order]
    counts = np.bincount(p[:, 0].astype(np.int64), minlength=num_bins)
    offsets = np.zeros(num_bins + 1, np.uint32)
    offsets[1:] = np.cumsum(counts)
    return offsets, p[:, 1].copy()
