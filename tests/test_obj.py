"""The OBJ reader (gbr_obj_read_text / gbr_obj_read_file, restating
ObjParser.cpp): the oracle restatement and the library against the
reference's own parser (tests/golden/obj_cases.npz, made by
tests/golden/make_obj_golden.py), the library against the oracle on a larger
mesh, the error cases, and (GPU) a parsed mesh rendered through the
reference's full normal-mapped Phong branch against the oracle renderer."""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import obj_oracle  # noqa: E402

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "obj_cases.npz")
CASES = ["sphere_vtn", "sphere_vtn_invert_y", "cube_positions", "quirks"]


def golden(name):
    g = np.load(GOLDEN)
    return (bytes(g[name + "__text"]).decode(), int(g[name + "__invert"]), g[name + "__vertices"],
            g[name + "__indices"], int(g[name + "__type"]))


def assert_same_mesh(verts, idx, vt, gv, gi, gt):
    """Bit-exact positions, uvs, normals and tangents; colours only where the
    reference sets them (without uvs; elsewhere it leaves them unset)."""
    assert vt == gt
    assert np.array_equal(idx, gi)
    assert verts.shape == gv.shape
    cols = list(range(11)) if gt & obj_oracle.VT_UV else list(range(14))
    a, b = verts[:, cols].view(np.uint32), gv[:, cols].view(np.uint32)
    assert np.array_equal(a, b), f"{int((a != b).sum())} values differ"


@pytest.mark.parametrize("name", CASES)
def test_oracle_matches_reference_parser(name):
    text, inv, gv, gi, gt = golden(name)
    verts, idx, vt, _ = obj_oracle.read(text, bool(inv))
    assert_same_mesh(verts, idx, vt, gv, gi, gt)


@pytest.mark.parametrize("name", CASES)
def test_reader_matches_reference_parser(gbr_lib, name):
    text, inv, gv, gi, gt = golden(name)
    verts, idx, vt, faces = gbr_lib.read_obj(text, bool(inv), text=True)
    assert_same_mesh(verts, idx, vt, gv, gi, gt)
    assert faces == text.count("\nf ") + text.startswith("f ")


def test_reader_matches_oracle_on_a_larger_mesh(gbr_lib, tmp_path):
    import scenes
    text = scenes.obj_sphere_text(96, 48)
    path = tmp_path / "sphere.obj"
    path.write_text(text)
    verts, idx, vt, faces = gbr_lib.read_obj(str(path))
    ov, oi, ot, of = obj_oracle.read(text)
    assert (vt, faces) == (ot, of) and faces == 2 * 96 * 48
    assert np.array_equal(idx, oi)
    assert np.array_equal(verts.view(np.uint32), ov.view(np.uint32))
    # one vertex per (position, uv) pair: the seam column stays apart
    assert len(verts) <= 49 * 97
    t = verts[:, 8:11]
    norm = np.linalg.norm(t, axis=1)
    assert np.all((np.abs(norm - 1.0) < 1e-5) | (norm == 0.0))   # zero only where the sum vanishes
    assert (norm > 0).mean() > 0.9
    assert np.all(np.abs(np.sum(t * verts[:, 5:8], axis=1)) < 1e-4)   # tangents orthogonal to normals


@pytest.mark.parametrize("text, what", [
    ("v  0 0 0\nv  1 0 0\nv  0 1 0\nf 1//1 2//1 3//1\n", "face index is not a number"),
    ("v  0 0 0\nv  1 0 0\nf 1 2 3\n", "position index out of range"),
    ("v  0 0 x\n", "coordinate is not a number"),
    ("v  0 0 0\nv  1 0 0\nv  0 1 0\nf 0 1 2\n", "face index below 1"),
    ("v\n", "field missing"),
])
def test_reader_rejects_what_the_reference_cannot_read(gbr_lib, text, what):
    with pytest.raises(gbr_lib.GbrError) as e:
        gbr_lib.read_obj(text, text=True)
    assert e.value.status == 1 and what in str(e.value)


def test_reader_file_rules(gbr_lib, tmp_path):
    p = tmp_path / "mesh.txt"
    p.write_text("v  0 0 0\n")
    with pytest.raises(gbr_lib.GbrError) as e:   # OpenFile: extension must be ".obj"
        gbr_lib.read_obj(str(p))
    assert e.value.status == 1
    with pytest.raises(gbr_lib.GbrError) as e:
        gbr_lib.read_obj(str(tmp_path / "missing.obj"))
    assert e.value.status == 6
    empty = tmp_path / "empty.obj"
    empty.write_text("# nothing\n\n")
    verts, idx, vt, faces = gbr_lib.read_obj(str(empty))
    assert len(verts) == 0 and len(idx) == 0 and vt == 0 and faces == 0


@pytest.mark.gpu
@pytest.mark.parametrize("sample", [0, 1])
def test_obj_mesh_renders_like_the_oracle(gbr_lib, cuda_device, sample):
    """A parsed mesh (uv + normal + generated tangents) with all four maps:
    bins bit-exact, ids and depth bit-exact, colour within 1 LSB of the
    oracle renderer; the normal map must change the image."""
    import scenes
    from test_parity_gpu import run_case
    verts, idx, vt, _ = gbr_lib.read_obj(scenes.obj_sphere_text(), text=True)
    assert vt == obj_oracle.VT_UV | obj_oracle.VT_NORM | obj_oracle.VT_TAN
    s = scenes.obj_scene(verts, idx, sample=sample)
    g, _ = run_case(gbr_lib, s, ref_band=False)
    flat = scenes.obj_scene(verts, idx, sample=sample)
    flat.meshes[0].textures[1] = scenes.flat_texture(256, (128, 128, 255))
    g2, _ = run_case(gbr_lib, flat, ref_band=False)
    covered = g["ids"] != 0xFFFFFFFF
    assert covered.sum() > 50_000
    assert (g["colour"][covered] != g2["colour"][covered]).mean() > 0.2
