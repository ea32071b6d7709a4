"""The reference's own CPU renderer (ERenderer.cpp), built from the staged
reference sources with the adapter patches of oracle/ref/build_ref.py, is
the timed CPU baseline of bench.py.  Its semantics differ from the GPU path
(ties pass, colour without the 1/w factor, lights looped), so it is checked
for agreement in coverage, not bit-exactly."""
import json
import os
import subprocess

import numpy as np
import pytest

import scenes
from oracle import oracle
from oracle.ref import build_ref, ref_io

pytestmark = pytest.mark.skipif(not os.path.isdir(build_ref.SRC) and not os.path.isdir(build_ref.CCR),
                                reason="reference sources are not staged here")


def render_eref(scene, tmp_path, frames=1, stride=1):
    exe = build_ref.build_erenderer()
    path = str(tmp_path / "scene.bin")
    out = str(tmp_path / "frame.bin")
    ref_io.write_scene(scene, path)
    p = subprocess.run([exe, path, str(frames), str(stride), out], capture_output=True, text=True, check=True)
    info = json.loads(p.stdout.strip().splitlines()[-1])
    px = np.fromfile(out, np.uint32).reshape(scene.height, scene.width)
    return info, px


def test_erenderer_sphere_coverage_matches_the_gpu_path_rule(tmp_path):
    s = scenes.sphere_scene(320, 240)
    info, px = render_eref(s, tmp_path)
    assert info["triangles"] == s.num_triangles and info["ms_per_frame"] > 0
    o = oracle.render(s, oracle.RASTER_REFERENCE, want_bins=False)
    covered_ref = o["ids"] != 0xFFFFFFFF
    clear = px[0, 0]
    covered_cpu = px != clear
    # same geometry and edge rule: coverage agrees up to edge pixels
    assert abs(int(covered_cpu.sum()) - int(covered_ref.sum())) <= 0.02 * covered_ref.sum()
    assert (covered_cpu & covered_ref).sum() >= 0.97 * covered_ref.sum()
    assert len(np.unique(px[covered_cpu])) > 50   # lit and textured, not flat


def test_erenderer_stride_sample_renders_a_subset(tmp_path):
    s = scenes.soup_scene(4000, 256, 192, seed=3)
    full, _ = render_eref(s, tmp_path, stride=1)
    part, _ = render_eref(s, tmp_path, stride=4)
    assert full["triangles"] == 4000 and part["triangles"] == 1000
