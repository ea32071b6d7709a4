"""CPU restatement of the reference's OBJ reader (ObjParser.cpp) --
TEST INFRASTRUCTURE ONLY: the checker of gbr_obj_read_text, pinned to the
reference's own parser by tests/golden/obj_cases.npz
(tests/golden/make_obj_golden.py runs ObjParser.cpp on synthetic files).

Pure Python; every float operation is a float32 operation (numpy float32
scalars round each step), in the reference's order.
"""
import re
from fractions import Fraction

import numpy as np

F = np.float32
FLT_EPS = F(np.finfo(np.float32).eps)
FLT_MIN = F(np.finfo(np.float32).tiny)
VT_UV, VT_NORM, VT_TAN = 1, 4, 8


def _fields(s: str, n: int = 3):
    """std::getline(ss, f, ' ') n times (ObjParser.cpp:196-205)."""
    out, at = [], 0
    for _ in range(n):
        if at > len(s):
            out.append("")
            continue
        sp = s.find(" ", at)
        if sp < 0:
            out.append(s[at:])
            at = len(s) + 1
        else:
            out.append(s[at:sp])
            at = sp + 1
    return out


_FLOAT_PREFIX = re.compile(r"[+-]?(\d+\.?\d*|\.\d+)([eE][+-]?\d+)?")


def _to_f32(text: str) -> F:
    """The float32 nearest to the decimal `text` (ties to even), as strtof
    rounds: exact rational comparison, no double rounding."""
    exact = Fraction(text)
    if exact == 0:
        return F(-0.0) if text.startswith("-") else F(0.0)
    x = F(float(exact))
    best = x
    for y in (np.nextafter(x, F(-np.inf)), np.nextafter(x, F(np.inf))):
        if not np.isfinite(y):
            continue
        dy, db = abs(Fraction(float(y)) - exact), abs(Fraction(float(best)) - exact)
        if dy < db or (dy == db and (int(y.view(np.uint32)) & 1) == 0):
            best = y
    return F(best)


def _stof(f: str) -> F:
    """std::stof: leading whitespace skipped, the longest decimal prefix."""
    t = f.lstrip(" \t\r\n\v\f")
    m = _FLOAT_PREFIX.match(t)
    if not m:
        raise ValueError(f"not a number: {f!r}")
    return _to_f32(m.group(0))


def _stoi(f: str) -> int:
    t = f.lstrip(" \t\r\n\v\f")
    k = 0
    if k < len(t) and t[k] in "+-":
        k += 1
    d = k
    while k < len(t) and t[k].isdigit():
        k += 1
    if k == d:
        raise ValueError(f"not an integer: {f!r}")
    return int(t[:k])


def _normalized(x: F, y: F, z: F):
    """GetNormalized (Vector.h:41-64)."""
    m = np.sqrt(x * x + y * y + z * z, dtype=np.float32)
    if m == F(0):
        return F(0), F(0), F(0)
    inv = F(1) / m
    return x * inv, y * inv, z * inv


def _are_equal(a: F, b: F) -> bool:
    """AreEqual<float>(a, b, 2) (MathUtilities.h:29-38)."""
    d = abs(a - b)
    return bool(d <= FLT_EPS * abs(a + b) * F(2) or d < FLT_MIN)


def parse(text: str, invert_y: bool = False):
    """ParseData (ObjParser.cpp:23-92): positions, uvs, normals, index lists,
    face count."""
    pos, uvs, nrm, pi, ti, ni = [], [], [], [], [], []
    faces = 0
    lines = text.split("\n")
    if text.endswith("\n"):
        lines = lines[:-1]
    for line in lines:
        if not line or line[0] == "#":
            continue
        prefix = line.split(" ", 1)[0]
        if prefix in ("v", "vt", "vn"):
            if len(line) < 3:
                raise ValueError("field missing")
            a, b, c = _fields(line[3:])
            if prefix == "vt":
                v = _stof(b)
                u = _stof(a)
                if invert_y:
                    v = F(1) - v
                uvs.append((u, v))
            elif prefix == "v":
                pos.append((_stof(a), _stof(b), _stof(c)))
            else:
                nrm.append(_normalized(_stof(a), _stof(b), _stof(c)))
        elif prefix == "f":
            idx = []
            for corner in _fields(line[2:]):
                start, slash = 0, 0
                while True:
                    cut = corner.find("/", start)
                    idx.append(_stoi(corner[start:] if cut < 0 else corner[start:cut]) - 1)
                    slash = corner.find("/", slash + 1)
                    if slash < 0:
                        break
                    start = slash + 1
            per = len(idx) // 3
            for k, v in enumerate(idx):
                if v < 0:
                    raise ValueError("face index below 1")
                if k % per < 3:   # ObjParser.cpp:166-181
                    (pi, ti, ni)[k % per].append(v)
            faces += 1
    return pos, uvs, nrm, pi, ti, ni, faces


def read(text: str, invert_y: bool = False):
    """ReadFromObjFile, pointer form (ObjParser.cpp:100-108, 216-355), with
    the values this build sets where the reference reads unset memory
    (tangent 0, colour 1, normal 0 without normals).  Returns (vertices
    n x 14 float32 [p3 uv2 n3 tan3 c3], indices uint32, vertex type, faces)."""
    pos, uvs, nrm, pi, ti, ni, faces = parse(text, invert_y)
    has_uv, has_n = bool(uvs), bool(nrm)
    verts, index, seen = [], [], {}
    for i in range(len(pi)):
        key = (pi[i], ti[i] if has_uv else 0)
        n = nrm[ni[i]] if has_n else None
        found = None
        for c in seen.get(key, []):
            if n is not None:
                o = verts[c]
                if not (_are_equal(o[5], n[0]) and _are_equal(o[6], n[1]) and _are_equal(o[7], n[2])):
                    continue
            found = c
            break
        if found is None:
            v = [F(0)] * 14
            v[0:3] = pos[pi[i]]
            if has_uv:
                v[3:5] = uvs[ti[i]]
            if n is not None:
                v[5:8] = n
            v[11:14] = [F(1)] * 3
            found = len(verts)
            verts.append(v)
            seen.setdefault(key, []).append(found)
        index.append(found)
    vt = (VT_UV if has_uv else 0) | (VT_NORM if has_n else 0)
    if has_uv and has_n:
        vt |= VT_TAN
        for i in range(0, len(index) - 2, 3):   # ObjParser.cpp:280-300
            a, b, c = verts[index[i]], verts[index[i + 1]], verts[index[i + 2]]
            e0 = [b[k] - a[k] for k in range(3)]
            e1 = [c[k] - a[k] for k in range(3)]
            dx0, dx1 = b[3] - a[3], c[3] - a[3]
            dy0, dy1 = b[4] - a[4], c[4] - a[4]
            r = F(1) / (dx0 * dy1 - dx1 * dy0)
            t = [(e0[k] * dy1 - e1[k] * dy0) * r for k in range(3)]
            for v in (a, b, c):
                for k in range(3):
                    v[8 + k] = v[8 + k] + t[k]
        for v in verts:   # GetNormalized(Reject(tan, n))
            t, nn = v[8:11], v[5:8]
            s = (t[0] * nn[0] + t[1] * nn[1] + t[2] * nn[2]) / (nn[0] * nn[0] + nn[1] * nn[1] + nn[2] * nn[2])
            rej = [t[k] - nn[k] * s for k in range(3)]
            v[8:11] = _normalized(*rej)
    out = np.array(verts, dtype=np.float32).reshape(-1, 14)
    return out, np.array(index, dtype=np.uint32), vt, faces
