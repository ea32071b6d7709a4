"""Generates the golden fixtures in tests/golden/ from the reference itself.

Runs on a machine with a GPU: builds oracle/_ref/ref_harness (the
reference's CUDARenderer compiled from the staged, patched sources; see
oracle/ref/build_ref.py), renders each case through it and stores what the
reference produced:

  * the sha256 of the scene file fed to the harness (tests regenerate the
    scene from its recipe and check this hash before comparing);
  * the framebuffer words and PixelShade::zInterpolated per pixel (all
    pixels for small cases, a band of rows for the 1080p case);
  * the per-bin triangle lists as sorted (bin, primitive id) pairs (small
    cases) or a sha256 of the sorted lists (1080p case), and the number of
    visible triangles;
  * for the full-size cases, a 64-bit hash of every band of BAND_ROWS rows
    of the whole framebuffer and of the whole zInterpolated frame
    (band_hash), so tests can compare complete frames with the reference.

usage: python tests/golden/make_golden.py OUT_DIR [case ...]
"""
import hashlib
import json
import os
import subprocess
import sys
import tempfile

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
for p in (ROOT, os.path.join(ROOT, "custom-gpgpu-rasterizer_gb300")):
    if p not in sys.path:
        sys.path.insert(0, p)

import numpy as np  # noqa: E402

import scenes  # noqa: E402
from oracle.ref import build_ref, ref_io  # noqa: E402



def two_sphere_scene():
    s = scenes.sphere_scene(320, 240)
    m2 = scenes.uv_sphere_mesh(24, 12, 0.6)
    m2.world = scenes.identity16()
    m2.world[12:15] = [0.9, 0.4, 0.5]
    rng = np.random.default_rng(2)
    m2.vertices["c"] = rng.random((len(m2.vertices), 3)).astype(np.float32)
    s.meshes.append(m2)
    return s


CASES = {
    "sphere640_point": lambda: scenes.sphere_scene(),
    "sphere640_linear": lambda: scenes.sphere_scene(sample=scenes.SAMPLE_LINEAR),
    "sphere640_depth": lambda: scenes.sphere_scene(vis=scenes.VIS_DEPTH),
    "sphere640_normal": lambda: scenes.sphere_scene(vis=scenes.VIS_NORMAL),
    "two_spheres320": two_sphere_scene,
    "soup5k_256x192": lambda: scenes.soup_scene(5000, 256, 192, seed=101),
    "soup5k_256x192_backface": lambda: scenes.soup_scene(5000, 256, 192, seed=102, cull=scenes.CULL_BACKFACE),
    "soup1m_1080p": lambda: scenes.soup_scene(1_000_000, 1920, 1080, seed=0),
    "icosphere7_4k": lambda: scenes.icosphere_scene(),
}
FULL_SIZE = {"soup1m_1080p": (500, 532), "icosphere7_4k": (1064, 1096)}   # the rows stored pixel by pixel
BAND_ROWS = 8


def band_hash(img):
    """64-bit hashes (the first 8 bytes of sha256) of each band of
    BAND_ROWS rows of a 4-byte-per-pixel frame, as uint64."""
    a = np.ascontiguousarray(img).view(np.uint32)
    out = []
    for y0 in range(0, a.shape[0], BAND_ROWS):
        out.append(int.from_bytes(hashlib.sha256(a[y0:y0 + BAND_ROWS].tobytes()).digest()[:8], "little"))
    return np.array(out, np.uint64)


def scene_hash(path):
    return hashlib.sha256(open(path, "rb").read()).hexdigest()


def bins_hash(offsets, ids):
    h = hashlib.sha256()
    h.update(np.ascontiguousarray(offsets, np.uint32).tobytes())
    h.update(np.ascontiguousarray(ids, np.uint32).tobytes())
    return h.hexdigest()


def run_case(name, out_dir, harness):
    scene = CASES[name]()
    with tempfile.TemporaryDirectory() as td:
        sp, rp = os.path.join(td, "scene.bin"), os.path.join(td, "out.bin")
        ref_io.write_scene(scene, sp)
        sha = scene_hash(sp)
        p = subprocess.run([harness, sp, rp], capture_output=True, text=True)
        if p.returncode != 0:
            raise RuntimeError(f"{name}: harness failed ({p.returncode}): {p.stderr[-2000:]}")
        res = ref_io.read_result(rp)
    nb = scene.num_bins_x * scene.num_bins_y
    offsets, ids = ref_io.bins_from_pairs(res["pairs"], nb)
    meta = {"case": name, "scene_sha256": sha, "visible": int(res["visible"]), "num_pairs": int(len(ids)),
            "bins_sha256": bins_hash(offsets, ids), "width": scene.width, "height": scene.height}
    arrays = {}
    if name in FULL_SIZE:
        band = FULL_SIZE[name]
        meta["rows"] = list(band)
        arrays["colour"] = res["colour"][band[0]:band[1]]
        arrays["z"] = res["z"][band[0]:band[1]]
        arrays["colour_band_hash"] = band_hash(res["colour"])
        arrays["z_band_hash"] = band_hash(res["z"])
    else:
        meta["rows"] = [0, scene.height]
        arrays["colour"] = res["colour"]
        arrays["z"] = res["z"]
        arrays["bin_offsets"] = offsets
        arrays["bin_ids"] = ids
    np.savez_compressed(os.path.join(out_dir, f"{name}.npz"), meta=json.dumps(meta), **arrays)
    print(f"{name}: visible={meta['visible']} pairs={meta['num_pairs']} stdout={p.stdout.strip()}")


def main():
    out_dir = sys.argv[1] if len(sys.argv) > 1 else os.path.dirname(os.path.abspath(__file__))
    os.makedirs(out_dir, exist_ok=True)
    names = sys.argv[2:] or list(CASES)
    harness = build_ref.build()
    for n in names:
        run_case(n, out_dir, harness)


if __name__ == "__main__":
    main()
