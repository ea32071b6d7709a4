"""Golden fixtures for the OBJ reader: synthetic OBJ texts run through the
reference's own ObjParser (ObjParser.cpp, compiled by oracle/ref/build_ref.py
into oracle/_ref/obj_harness).  Writes tests/golden/obj_cases.npz: for each
case the OBJ text, the invert-y flag and the reference's vertices (n x 14
float32: p3 uv2 n3 tan3 c3), indices and vertex type.

    python tests/golden/make_obj_golden.py

The texts are generated here (seeded); none comes from the reference.  The
case with uvs but no normals is left out: the reference reads an empty
normal list there.
"""
import math
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))


def f6(x: float) -> str:
    return f"{x:.6f}"


def sphere_obj(lon: int = 8, lat: int = 6, seed: int = 0, crlf: bool = True) -> str:
    """UV sphere: shared positions, a uv grid with a duplicated seam column,
    per-position normals listed twice (the second copy nudged by one ulp in
    some components, so AreEqual-equal but not bit-equal), faces v/vt/vn."""
    rng = np.random.default_rng(seed)
    eol = "\r\n" if crlf else "\n"
    lines = ["# synthetic sphere", "# made by make_obj_golden.py", "", "mtllib none.mtl", "o Sphere", "g body"]
    pos, nrm = [], []
    for j in range(lat + 1):
        th = math.pi * j / lat
        for i in range(lon):
            ph = 2.0 * math.pi * i / lon
            p = (math.sin(th) * math.cos(ph), math.cos(th), math.sin(th) * math.sin(ph))
            pos.append(p)
    for p in pos:
        lines.append("v  " + " ".join(f6(c * 1.5) for c in p))
    for j in range(lat + 1):
        for i in range(lon + 1):
            lines.append("vt " + f6(i / lon) + " " + f6(j / lat) + " 0.000000")
    for p in pos:
        lines.append("vn " + " ".join(f6(c) for c in p))
    for p in pos:   # second copies, some nudged in the 6th decimal
        q = [c + (1e-6 if rng.random() < 0.3 else 0.0) for c in p]
        lines.append("vn " + " ".join(f6(c) for c in q))
    lines.append("s 1")
    lines.append("usemtl none")
    nv = len(pos)
    for j in range(lat):
        for i in range(lon):
            a = j * lon + i
            b = j * lon + (i + 1) % lon
            c = (j + 1) * lon + i
            d = (j + 1) * lon + (i + 1) % lon
            ta, tb = j * (lon + 1) + i, j * (lon + 1) + i + 1
            tc, td = (j + 1) * (lon + 1) + i, (j + 1) * (lon + 1) + i + 1
            na = a + (nv if rng.random() < 0.5 else 0)
            nb, nc, nd = b, c + (nv if rng.random() < 0.5 else 0), d

            def corner(v, t, n):
                return f"{v + 1}/{t + 1}/{n + 1}"
            lines.append("f " + " ".join([corner(a, ta, na), corner(c, tc, nc), corner(b, tb, nb)]) + " ")
            lines.append("f " + " ".join([corner(b, tb, nb), corner(c, tc, nc), corner(d, td, nd)]) + " ")
    lines.append("# " + str(2 * lat * lon) + " faces")
    return eol.join(lines) + eol


def positions_obj() -> str:
    """A cube with position-only faces (and one quad, read as its first
    three corners), 3ds Max spacing."""
    vs = [(-1, -1, -1), (1, -1, -1), (1, 1, -1), (-1, 1, -1), (-1, -1, 1), (1, -1, 1), (1, 1, 1), (-1, 1, 1)]
    lines = ["# cube"] + ["v  " + " ".join(f6(c) for c in v) for v in vs]
    faces = [(1, 2, 3), (1, 3, 4), (5, 7, 6), (5, 8, 7), (1, 5, 6), (1, 6, 2), (2, 6, 7), (2, 7, 3), (3, 7, 8),
             (3, 8, 4), (4, 8, 5), (4, 5, 1)]
    lines += ["f " + " ".join(str(i) for i in f) + " " for f in faces]
    lines.append("f 1 2 3 4")
    return "\n".join(lines) + "\n"


def quirks_obj() -> str:
    """Single-space "v" lines (the reference drops their first character),
    vt lines without a third field, repeated v/vt/vn faces."""
    lines = ["v -1.250000 0.500000 0.000000", "v 12.500000 -3.000000 1.000000", "v 0.75 0.25 4.5",
             "v  2.000000 2.000000 2.000000"]
    lines += ["vt 0.25 0.75", "vt 0.5 0.125", "vt 1.0 1.0"]
    lines += ["vn 0.0 0.0 1.0", "vn 0.0 1.0 0.0"]
    faces = ["f 1/1/1 2/2/1 3/3/1", "f 2/2/2 4/3/2 3/1/2", "f 4/1/1 1/2/1 2/3/2"]
    # the reference sizes its vertex array by the face count (ObjParser.cpp:
    # 218): repeated faces keep the distinct corners below it
    lines += faces * 4
    return "\n".join(lines) + "\n"


CASES = [("sphere_vtn", sphere_obj(), 0), ("sphere_vtn_invert_y", sphere_obj(seed=1, crlf=False), 1),
         ("cube_positions", positions_obj(), 0), ("quirks", quirks_obj(), 0)]


def run_reference(text: str, invert: int):
    sys.path.insert(0, os.path.join(ROOT, "oracle", "ref"))
    import build_ref
    exe = build_ref.build_objparser()
    with tempfile.TemporaryDirectory() as d:
        src, out = os.path.join(d, "mesh.obj"), os.path.join(d, "out.bin")
        with open(src, "wb") as f:
            f.write(text.encode())
        subprocess.run([exe, src, str(invert), out], check=True, stdout=subprocess.DEVNULL)
        raw = open(out, "rb").read()
    nv, ni, vt = np.frombuffer(raw[:12], dtype=np.uint32)
    vt = int(np.int32(vt))
    verts = np.frombuffer(raw[12:12 + 56 * nv], dtype=np.float32).reshape(nv, 14).copy()
    idx = np.frombuffer(raw[12 + 56 * nv:12 + 56 * nv + 4 * ni], dtype=np.uint32).copy()
    return verts, idx, vt


def main():
    out = {}
    for name, text, invert in CASES:
        verts, idx, vt = run_reference(text, invert)
        out[f"{name}__text"] = np.frombuffer(text.encode(), dtype=np.uint8)
        out[f"{name}__invert"] = np.array(invert, dtype=np.int32)
        out[f"{name}__vertices"] = verts
        out[f"{name}__indices"] = idx
        out[f"{name}__type"] = np.array(vt, dtype=np.int32)
        print(name, verts.shape, idx.shape, vt)
    np.savez_compressed(os.path.join(HERE, "obj_cases.npz"), **out)


if __name__ == "__main__":
    main()
