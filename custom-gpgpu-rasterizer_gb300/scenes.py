"""Seeded synthetic scenes for the frame hot path.

No asset files or datasets are read: every workload is generated here from a
seed.  Vertices use the reference's IVertex layout (56 B: p3 uv2 n3 tan3 c3,
CustomCUDARasterizer/Vertex.h:113-145) or the compact soup layout (16 B:
p3 float + RGBA8).  Matrices are column-major, element (r, c) at [c*4 + r]
(CustomCUDARasterizer/Matrix.h:9-21).
"""
from __future__ import annotations

import dataclasses
import math
from typing import List, Optional

import numpy as np

IVERTEX56 = np.dtype([("p", "<f4", 3), ("uv", "<f4", 2), ("n", "<f4", 3),
                      ("tan", "<f4", 3), ("c", "<f4", 3)])
POS3_RGBA8 = np.dtype([("p", "<f4", 3), ("rgba", "<u4")])
assert IVERTEX56.itemsize == 56 and POS3_RGBA8.itemsize == 16

VERTEX_IVERTEX56 = 0
VERTEX_POS3_RGBA8 = 1

CULL_BACKFACE, CULL_FRONTFACE, CULL_NONE = 0, 1, 2
SAMPLE_POINT, SAMPLE_LINEAR = 0, 1
SAMPLE_BILINEAR = 2   # the build's extension: true bilinear filtering
LIGHT_DIRECTIONAL, LIGHT_POINT = 0, 1
VIS_PBR, VIS_DEPTH, VIS_NORMAL = 0, 1, 2
TOPOLOGY_LIST, TOPOLOGY_STRIP = 0, 1

CLEAR_COLOUR32 = 0x003F3F3F  # RGBA{RGBColor{0.25,0.25,0.25}} (CUDARenderer.h:135, RGBRaw.h:24-32)


def identity16() -> np.ndarray:
    return np.eye(4, dtype=np.float32).reshape(16)


@dataclasses.dataclass
class Mesh:
    vertices: np.ndarray                  # structured, IVERTEX56 or POS3_RGBA8
    indices: Optional[np.ndarray] = None  # uint32, None: non-indexed list
    topology: int = TOPOLOGY_LIST
    world: np.ndarray = dataclasses.field(default_factory=identity16)
    textures: List[Optional[np.ndarray]] = dataclasses.field(default_factory=lambda: [None] * 4)

    @property
    def vertex_format(self) -> int:
        return VERTEX_IVERTEX56 if self.vertices.dtype == IVERTEX56 else VERTEX_POS3_RGBA8

    @property
    def num_triangles(self) -> int:
        if self.indices is None:
            return len(self.vertices) // 3
        if self.topology == TOPOLOGY_LIST:
            return len(self.indices) // 3
        return max(len(self.indices) - 2, 0)


@dataclasses.dataclass
class Light:
    """A scene light (DirectionalLight / PointLight of the reference's scene
    graph): vec is the direction the light travels, or the point light's
    world position."""
    type: int
    colour: tuple
    intensity: float
    vec: tuple


@dataclasses.dataclass
class Camera:
    pos: np.ndarray   # (3,) f32
    fwd: np.ndarray   # (3,) f32
    view: np.ndarray  # (16,) f32
    proj: np.ndarray  # (16,) f32


@dataclasses.dataclass
class Scene:
    name: str
    width: int
    height: int
    bin_w: int
    bin_h: int
    camera: Camera
    meshes: List[Mesh]
    cull: int = CULL_BACKFACE
    sample: int = SAMPLE_POINT
    vis: int = VIS_PBR
    seed: int = 0
    lights: List[Light] = dataclasses.field(default_factory=list)   # empty: the shader's constant light

    @property
    def num_bins_x(self) -> int:
        return (self.width + self.bin_w - 1) // self.bin_w

    @property
    def num_bins_y(self) -> int:
        return (self.height + self.bin_h - 1) // self.bin_h

    @property
    def num_triangles(self) -> int:
        return sum(m.num_triangles for m in self.meshes)


def identity_camera() -> Camera:
    """w == 1 everywhere: NDC positions pass through the vertex stage exactly."""
    return Camera(np.zeros(3, np.float32), np.array([0, 0, 1], np.float32), identity16(), identity16())


def _inverse_translation(pos: np.ndarray) -> np.ndarray:
    # Inverse of the look-at matrix of an un-rotated camera (Camera.h:26):
    # for a pure translation the FGED1 inverse (Matrix4.h:329-361) is exact.
    v = identity16()
    v[12:15] = -pos.astype(np.float32)
    return v


def perspective_camera(pos, fov_deg: float, width: int, height: int,
                       near: float = 0.1, far: float = 100.0) -> Camera:
    """Camera as CustomCUDARasterizer/Camera.cpp:6-36, 97-108 builds it: looks
    down -z, forward vector (0,0,1), projection with data[3][3] left at 1 from
    the identity it starts from."""
    f32 = np.float32
    pos = np.asarray(pos, np.float32)
    radians = f32(fov_deg) * (f32(math.pi) / f32(180.0))
    fov = f32(math.tan(radians / f32(2.0)))
    aspect = f32(width) / f32(height)
    A = f32(far) / (f32(near) - f32(far))
    B = (f32(far) * f32(near)) / (f32(near) - f32(far))
    proj = identity16()
    proj[0] = f32(1.0) / (aspect * fov)
    proj[5] = f32(1.0) / fov
    proj[10] = A
    proj[11] = f32(-1.0)
    proj[14] = B
    return Camera(pos, np.array([0, 0, 1], np.float32), _inverse_translation(pos), proj)


def checker_texture(size: int = 512, cells: int = 8, c0=(230, 230, 230), c1=(40, 60, 160)) -> np.ndarray:
    y, x = np.mgrid[0:size, 0:size]
    cell = size // cells
    odd = ((x // cell) + (y // cell)) & 1
    rgb = np.where(odd[..., None] == 1, np.array(c1, np.uint32), np.array(c0, np.uint32))
    return (rgb[..., 0] | (rgb[..., 1] << 8) | (rgb[..., 2] << 16) | (255 << 24)).astype(np.uint32)


def flat_texture(size: int, rgb) -> np.ndarray:
    v = rgb[0] | (rgb[1] << 8) | (rgb[2] << 16) | (255 << 24)
    return np.full((size, size), v, np.uint32)


def uv_sphere_mesh(lon: int = 64, lat: int = 32, radius: float = 1.0) -> Mesh:
    """UV sphere with a seam column (lat+1)*(lon+1) vertices; single triangles
    at the poles, two per quad elsewhere: 2*lon*(lat-1) triangles.  Front
    faces are counter-clockwise seen from outside."""
    i = np.arange(lat + 1, dtype=np.float64)[:, None]
    j = np.arange(lon + 1, dtype=np.float64)[None, :]
    theta = i * math.pi / lat
    phi = j * 2.0 * math.pi / lon
    x = np.sin(theta) * np.cos(phi)
    y = np.cos(theta) * np.ones_like(phi)
    z = np.sin(theta) * np.sin(phi)
    v = np.zeros((lat + 1) * (lon + 1), IVERTEX56)
    p = np.stack([x, y, z], -1).reshape(-1, 3)
    v["p"] = (p * radius).astype(np.float32)
    v["n"] = p.astype(np.float32)
    v["uv"] = np.stack([np.broadcast_to(j / lon, x.shape), np.broadcast_to(i / lat, x.shape)], -1).reshape(-1, 2)
    tan = np.stack([-np.sin(phi) * np.ones_like(theta), np.zeros_like(x), np.cos(phi) * np.ones_like(theta)], -1)
    v["tan"] = tan.reshape(-1, 3).astype(np.float32)
    v["c"] = 1.0
    idx = []
    vid = lambda a, b: a * (lon + 1) + b
    for a in range(lat):
        for b in range(lon):
            q0, q1, q2, q3 = vid(a, b), vid(a + 1, b), vid(a + 1, b + 1), vid(a, b + 1)
            if a != 0:
                idx.append((q0, q1, q3))
            if a != lat - 1:
                idx.append((q1, q2, q3) if a != 0 else (q0, q1, q2))
    tri = np.array(idx, np.int64)
    pp = v["p"].astype(np.float64)
    nrm = np.cross(pp[tri[:, 1]] - pp[tri[:, 0]], pp[tri[:, 2]] - pp[tri[:, 0]])
    cen = pp[tri].mean(axis=1)
    flip = (nrm * cen).sum(-1) < 0
    tri[flip] = tri[flip][:, [0, 2, 1]]
    return Mesh(vertices=v, indices=tri.reshape(-1).astype(np.uint32))


def sphere_scene(width: int = 640, height: int = 480, bin_size: int = 16, lon: int = 64, lat: int = 32,
                 tex_size: int = 512, sample: int = SAMPLE_POINT, vis: int = VIS_PBR) -> Scene:
    """UV sphere (64x32), r=1 at the origin, camera at distance 3 with a 60 deg
    FOV, 512^2 checker with 8x8 cells.  Lambert + ambient shading is the
    reference's shader with all four maps bound: checker diffuse, flat normal
    map (128,128,255), black specular, grey gloss (ShadePixelSafe,
    CustomCUDARasterizer/CUDAROPs.cu:411-470)."""
    mesh = uv_sphere_mesh(lon, lat)
    mesh.textures = [checker_texture(tex_size, 8), flat_texture(tex_size, (128, 128, 255)),
                     flat_texture(tex_size, (0, 0, 0)), flat_texture(tex_size, (128, 128, 128))]
    cam = perspective_camera((0.0, 0.0, 3.0), 60.0, width, height)
    return Scene("sphere", width, height, bin_size, bin_size, cam, [mesh], cull=CULL_BACKFACE,
                 sample=sample, vis=vis)


def obj_sphere_text(lon: int = 48, lat: int = 24, radius: float = 1.0, bumps: float = 0.04, seed: int = 5) -> str:
    """A Wavefront OBJ text (3ds Max style, as the reference's parser reads
    it: "v  x y z", "f v/vt/vn ...") of a bumpy UV sphere: positions shared
    across the uv seam, a uv grid with a seam column, one normal per
    position, two triangles per quad (counter-clockwise from outside)."""
    rng = np.random.default_rng(seed)
    lines = ["# sphere written by scenes.obj_sphere_text", "o Sphere"]
    pos = []
    for j in range(lat + 1):
        th = np.pi * j / lat
        for i in range(lon):
            ph = 2.0 * np.pi * i / lon
            r = radius * (1.0 + bumps * float(rng.uniform(-1.0, 1.0)) * (0 < j < lat))
            pos.append((r * np.sin(th) * np.cos(ph), r * np.cos(th), r * np.sin(th) * np.sin(ph)))
    lines += ["v  %.6f %.6f %.6f" % p for p in pos]
    lines += ["vt %.6f %.6f 0.000000" % (i / lon, j / lat) for j in range(lat + 1) for i in range(lon + 1)]
    for p in pos:
        n = np.asarray(p) / max(np.linalg.norm(p), 1e-12)
        lines.append("vn %.6f %.6f %.6f" % tuple(n))
    for j in range(lat):
        for i in range(lon):
            a, b = j * lon + i, j * lon + (i + 1) % lon
            c, d = (j + 1) * lon + i, (j + 1) * lon + (i + 1) % lon
            ta, tb = j * (lon + 1) + i, j * (lon + 1) + i + 1
            tc, td = (j + 1) * (lon + 1) + i, (j + 1) * (lon + 1) + i + 1
            corner = lambda v, t: "%d/%d/%d" % (v + 1, t + 1, v + 1)
            lines.append("f %s %s %s " % (corner(a, ta), corner(c, tc), corner(b, tb)))
            lines.append("f %s %s %s " % (corner(b, tb), corner(c, tc), corner(d, td)))
    return "\n".join(lines) + "\n"


def ivertex_array(rows: np.ndarray) -> np.ndarray:
    """(n, 14) float32 rows [p3 uv2 n3 tan3 c3] -> IVERTEX56 records."""
    rows = np.ascontiguousarray(rows, dtype=np.float32)
    return rows.view(IVERTEX56).reshape(-1)


def bump_normal_texture(size: int = 256, cells: int = 16) -> np.ndarray:
    """A tangent-space normal map with tilted stripes, so the shader's TBN
    transform (ShadePixelSafe, CUDAROPs.cu:429-435) changes the lighting."""
    y, x = np.mgrid[0:size, 0:size]
    t = np.sin(2.0 * np.pi * cells * (x + 0.5 * y) / size)
    nx, ny, nz = 0.45 * t, 0.2 * np.cos(2.0 * np.pi * cells * y / size), np.ones_like(t)
    n = np.stack([nx, ny, nz], -1)
    n /= np.linalg.norm(n, axis=-1, keepdims=True)
    c = np.clip(np.round((n * 0.5 + 0.5) * 255.0), 0, 255).astype(np.uint32)
    return c[..., 0] | (c[..., 1] << 8) | (c[..., 2] << 16) | np.uint32(255 << 24)


def obj_scene(vertices: np.ndarray, indices: np.ndarray, width: int = 800, height: int = 600,
              bin_size: int = 16, sample: int = SAMPLE_POINT, vis: int = VIS_PBR, tex_size: int = 256) -> Scene:
    """A mesh read by the OBJ reader (vertices as (n, 14) rows, uv + normal +
    tangent) with all four maps bound -- checker diffuse, a non-flat normal
    map, a striped specular map and a grey gloss map -- so every term of the
    reference's Phong branch (ShadePixelSafe, CUDAROPs.cu:411-470) and its
    tangent frame are exercised; camera 3 units away, 60 deg."""
    mesh = Mesh(ivertex_array(vertices), np.ascontiguousarray(indices, dtype=np.uint32))
    spec = flat_texture(tex_size, (0, 0, 0))
    spec[:, ::8] = flat_texture(1, (200, 180, 160))[0, 0]
    mesh.textures = [checker_texture(tex_size, 8), bump_normal_texture(tex_size), spec,
                     flat_texture(tex_size, (200, 200, 200))]
    cam = perspective_camera((0.0, 0.0, 3.0), 60.0, width, height)
    return Scene("obj_sphere", width, height, bin_size, bin_size, cam, [mesh], cull=CULL_BACKFACE,
                 sample=sample, vis=vis)


def soup_vertices(n: int, width: int, height: int, seed: int = 0, blob_frac: float = 0.2,
                  blob_sigma: float = 100.0, area_min: float = 0.5, area_max: float = 4096.0) -> np.ndarray:
    """Triangle soup in NDC with w == 1: centroids uniform over the screen plus
    a Gaussian blob (sigma px) at the centre, area log-uniform in
    [area_min, area_max] px^2, random orientation and winding, depth uniform in
    [0.1, 100] mapped to z_ndc = (d - 0.1) / 99.9, RGBA8 vertex colours."""
    rng = np.random.default_rng(seed)
    nb = int(round(n * blob_frac))
    cx = np.empty(n)
    cy = np.empty(n)
    cx[: n - nb] = rng.uniform(0, width, n - nb)
    cy[: n - nb] = rng.uniform(0, height, n - nb)
    cx[n - nb:] = rng.normal(width / 2, blob_sigma, nb)
    cy[n - nb:] = rng.normal(height / 2, blob_sigma, nb)
    perm = rng.permutation(n)
    cx, cy = cx[perm], cy[perm]
    area = np.exp(rng.uniform(math.log(area_min), math.log(area_max), n))
    base = rng.uniform(0, 2 * math.pi, n)
    ang = base[:, None] + np.arange(3)[None, :] * (2 * math.pi / 3) + rng.uniform(-0.6, 0.6, (n, 3))
    ux, uy = np.cos(ang), np.sin(ang)
    unit_area = 0.5 * np.abs((ux[:, 1] - ux[:, 0]) * (uy[:, 2] - uy[:, 0]) - (uy[:, 1] - uy[:, 0]) * (ux[:, 2] - ux[:, 0]))
    r = np.sqrt(area / np.maximum(unit_area, 1e-6))
    px = cx[:, None] + r[:, None] * ux
    py = cy[:, None] + r[:, None] * uy
    flip = rng.random(n) < 0.5
    px[flip] = px[flip][:, [0, 2, 1]]
    py[flip] = py[flip][:, [0, 2, 1]]
    d = rng.uniform(0.1, 100.0, n)[:, None] * (1.0 + rng.uniform(-0.01, 0.01, (n, 3)))
    d = np.clip(d, 0.1, 100.0)
    v = np.zeros(3 * n, POS3_RGBA8)
    xn = (2.0 * px / width - 1.0).astype(np.float32)
    yn = (1.0 - 2.0 * py / height).astype(np.float32)
    zn = ((d - 0.1) / 99.9).astype(np.float32)
    v["p"] = np.stack([xn, yn, zn], -1).reshape(-1, 3)
    rgb = rng.integers(0, 256, (3 * n, 3), dtype=np.uint32)
    v["rgba"] = rgb[:, 0] | (rgb[:, 1] << 8) | (rgb[:, 2] << 16) | np.uint32(255 << 24)
    return v


def soup_scene(n: int = 1_000_000, width: int = 1920, height: int = 1080, bin_size: int = 16, seed: int = 0,
               cull: int = CULL_NONE, ivertex: bool = False) -> Scene:
    v = soup_vertices(n, width, height, seed)
    if ivertex:
        v = pos3_to_ivertex(v)
    return Scene(f"soup{n}", width, height, bin_size, bin_size, identity_camera(), [Mesh(vertices=v)],
                 cull=cull, seed=seed)


def strip_grid_scene(nx: int = 20, ny: int = 12, width: int = 200, height: int = 160) -> Scene:
    """An nx x ny vertex grid (IVertex, vertex colours) drawn as one
    triangle strip: a strip per row pair, joined by two repeated indices
    (degenerate triangles), in the covered winding."""
    xs, ys = np.meshgrid(np.linspace(-0.9, 0.9, nx), np.linspace(-0.8, 0.8, ny))
    v = np.zeros(nx * ny, IVERTEX56)
    v["p"][:, 0], v["p"][:, 1] = xs.ravel(), ys.ravel()
    v["p"][:, 2] = 0.3 + 0.2 * np.sin(xs.ravel() * 3)
    v["c"] = np.stack([xs.ravel() * 0.5 + 0.5, ys.ravel() * 0.5 + 0.5, np.full(nx * ny, 0.3)], -1)
    idx = []
    for j in range(ny - 1):
        row = []
        for i in range(nx):
            row += [(j + 1) * nx + i, j * nx + i]  # counter-clockwise in NDC: the covered winding
        if idx:
            idx += [idx[-1], row[0]]
        idx += row
    m = Mesh(vertices=v, indices=np.array(idx, np.uint32), topology=TOPOLOGY_STRIP)
    return Scene("strip", width, height, 16, 16, identity_camera(), [m], cull=CULL_NONE)


BATCH_RESOLUTIONS = ((256, 256), (512, 512), (1024, 768), (1920, 1080))


def batch_scene_specs(n: int = 256, seed: int = 0, min_tris: int = 1000, max_tris: int = 500_000,
                      resolutions=BATCH_RESOLUTIONS) -> list:
    """(triangles, width, height, seed) of each scene of batch_scenes, without
    generating any vertex."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        count = int(math.exp(rng.uniform(math.log(min_tris), math.log(max_tris))))
        w, h = resolutions[int(rng.integers(0, len(resolutions)))]
        out.append((count, w, h, int(rng.integers(1 << 31))))
    return out


def batch_scenes(n: int = 256, seed: int = 0, min_tris: int = 1000, max_tris: int = 500_000,
                 bin_size: int = 16, resolutions=BATCH_RESOLUTIONS, only=None) -> list:
    """Uneven batch of soups: scene i has a triangle count log-uniform in
    [min_tris, max_tris] and a resolution drawn from `resolutions`; each is
    drawn like the 1M soup (uniform centroids plus a 20% Gaussian blob of
    sigma 100 px, area log-uniform in 0.5-4096 px^2, random winding, depth
    uniform in [0.1, 100], RGBA8 colours), seeded by (seed, i).  `only`: the
    indices of the scenes to build (a rank's share of a partitioned batch)."""
    specs = batch_scene_specs(n, seed, min_tris, max_tris, resolutions)
    out = []
    for i in (range(n) if only is None else only):
        count, w, h, sseed = specs[i]
        s = soup_scene(count, w, h, bin_size, seed=sseed)
        s.name = f"batch{i}_soup{count}_{w}x{h}"
        out.append(s)
    return out


def pos3_to_ivertex(v: np.ndarray) -> np.ndarray:
    out = np.zeros(len(v), IVERTEX56)
    out["p"] = v["p"]
    rgba = v["rgba"]
    out["c"] = np.stack([(rgba & 0xFF), (rgba >> 8) & 0xFF, (rgba >> 16) & 0xFF], -1).astype(np.float32) / np.float32(255.0)
    return out


# ---------------------------------------------------------------------------
# Dense sub-pixel mesh: displaced icosphere at 4K
# ---------------------------------------------------------------------------
def _value_noise_table(seed: int):
    rng = np.random.default_rng(seed)
    return rng.permutation(256).astype(np.int64), rng.uniform(-1.0, 1.0, 256)


def _fade(t):
    return t * t * (3.0 - 2.0 * t)


def value_noise3(p: np.ndarray, seed: int, octaves: int = 3, base_freq: float = 4.0) -> np.ndarray:
    """Seeded lattice value noise in [-1, 1] (trilinear, smoothstep fade),
    `octaves` octaves with doubling frequency and halving amplitude."""
    perm, vals = _value_noise_table(seed)
    out = np.zeros(len(p))
    amp_sum = 0.0
    for o in range(octaves):
        f = base_freq * (2 ** o)
        a = 0.5 ** o
        q = p * f
        i0 = np.floor(q).astype(np.int64)
        t = _fade(q - i0)
        acc = 0.0
        for dx in (0, 1):
            for dy in (0, 1):
                for dz in (0, 1):
                    h = perm[(perm[(perm[(i0[:, 0] + dx) & 255] + i0[:, 1] + dy) & 255] + i0[:, 2] + dz) & 255]
                    w = (t[:, 0] if dx else 1 - t[:, 0]) * (t[:, 1] if dy else 1 - t[:, 1]) * \
                        (t[:, 2] if dz else 1 - t[:, 2])
                    acc = acc + w * vals[h]
        out += a * acc
        amp_sum += a
    return out / amp_sum


def value_noise2(w: int, h: int, seed: int, octaves: int = 4, base_cells: int = 8) -> np.ndarray:
    perm, vals = _value_noise_table(seed)
    ys, xs = np.mgrid[0:h, 0:w]
    out = np.zeros((h, w))
    amp_sum = 0.0
    for o in range(octaves):
        cells = base_cells * (2 ** o)
        qx, qy = xs * cells / w, ys * cells / h
        ix, iy = np.floor(qx).astype(np.int64), np.floor(qy).astype(np.int64)
        tx, ty = _fade(qx - ix), _fade(qy - iy)
        acc = 0.0
        for dx in (0, 1):
            for dy in (0, 1):
                hh = perm[(perm[(ix + dx) & 255] + iy + dy) & 255]
                acc = acc + (tx if dx else 1 - tx) * (ty if dy else 1 - ty) * vals[hh]
        out += 0.5 ** o * acc
        amp_sum += 0.5 ** o
    return out / amp_sum


def noise_texture(size: int = 2048, seed: int = 7) -> np.ndarray:
    n = 0.5 + 0.5 * value_noise2(size, size, seed)
    r = np.clip(40 + 180 * n, 0, 255).astype(np.uint32)
    g = np.clip(80 + 150 * n * n, 0, 255).astype(np.uint32)
    b = np.clip(200 - 150 * n, 0, 255).astype(np.uint32)
    return r | (g << 8) | (b << 16) | np.uint32(255 << 24)


def icosphere_mesh(subdiv: int = 7, amplitude: float = 0.05, seed: int = 3) -> Mesh:
    """Icosahedron subdivided `subdiv` times (20*4^n triangles, 10*4^n+2
    vertices), radially displaced by seeded 3-octave value noise of the given
    amplitude; normals from the displaced surface, spherical UVs."""
    t = (1.0 + 5 ** 0.5) / 2.0
    V = np.array([(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0), (0, -1, t), (0, 1, t), (0, -1, -t), (0, 1, -t),
                  (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)], np.float64)
    V /= np.linalg.norm(V, axis=1, keepdims=True)
    F = np.array([(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4), (11, 10, 2),
                  (10, 7, 6), (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8), (3, 8, 9), (4, 9, 5),
                  (2, 4, 11), (6, 2, 10), (8, 6, 7), (9, 8, 1)], np.int64)
    for _ in range(subdiv):
        nf = len(F)
        e = np.concatenate([F[:, [0, 1]], F[:, [1, 2]], F[:, [2, 0]]])
        uniq, inv = np.unique(np.sort(e, axis=1), axis=0, return_inverse=True)
        inv = inv.reshape(-1)
        mid = V[uniq[:, 0]] + V[uniq[:, 1]]
        mid /= np.linalg.norm(mid, axis=1, keepdims=True)
        mid_idx = len(V) + np.arange(len(uniq))
        V = np.concatenate([V, mid])
        a, b, c = mid_idx[inv[:nf]], mid_idx[inv[nf:2 * nf]], mid_idx[inv[2 * nf:]]
        F = np.concatenate([np.stack([F[:, 0], a, c], 1), np.stack([F[:, 1], b, a], 1),
                            np.stack([F[:, 2], c, b], 1), np.stack([a, b, c], 1)])
    r = 1.0 + amplitude * value_noise3(V, seed)
    P = V * r[:, None]
    fn = np.cross(P[F[:, 1]] - P[F[:, 0]], P[F[:, 2]] - P[F[:, 0]])
    flip = (fn * P[F].mean(axis=1)).sum(-1) < 0
    F[flip] = F[flip][:, [0, 2, 1]]
    fn[flip] = -fn[flip]
    N = np.zeros_like(P)
    for k in range(3):
        np.add.at(N, F[:, k], fn)
    N /= np.maximum(np.linalg.norm(N, axis=1, keepdims=True), 1e-12)
    T = np.cross(np.array([0.0, 1.0, 0.0]), N)
    tl = np.linalg.norm(T, axis=1, keepdims=True)
    T = np.where(tl > 1e-6, T / np.maximum(tl, 1e-12), np.array([1.0, 0.0, 0.0]))
    v = np.zeros(len(P), IVERTEX56)
    v["p"] = P.astype(np.float32)
    v["n"] = N.astype(np.float32)
    v["tan"] = T.astype(np.float32)
    v["uv"] = np.stack([0.5 + np.arctan2(V[:, 2], V[:, 0]) / (2 * math.pi), np.arccos(np.clip(V[:, 1], -1, 1)) / math.pi],
                       -1).astype(np.float32)
    v["c"] = 1.0
    return Mesh(vertices=v, indices=F.reshape(-1).astype(np.uint32))


def icosphere_scene(width: int = 3840, height: int = 2160, bin_size: int = 16, subdiv: int = 7,
                    tex_size: int = 2048, distance: float = 8.0, sample: int = SAMPLE_LINEAR,
                    vis: int = VIS_PBR) -> Scene:
    """Displaced icosphere (327,680 triangles at 7 subdivisions) 8 units from
    a 60 deg camera at 4K, so most triangles cover under 1 px^2; a 2048^2
    noise texture with the reference's shader (all four maps bound, as the
    sphere scene) and its "linear" sampler."""
    mesh = icosphere_mesh(subdiv)
    mesh.textures = [noise_texture(tex_size), flat_texture(tex_size, (128, 128, 255)),
                     flat_texture(tex_size, (0, 0, 0)), flat_texture(tex_size, (128, 128, 128))]
    cam = perspective_camera((0.0, 0.0, distance), 60.0, width, height)
    return Scene(f"icosphere{subdiv}", width, height, bin_size, bin_size, cam, [mesh], cull=CULL_BACKFACE,
                 sample=sample, vis=vis)


def icosphere_lit_scene(width: int = 3840, height: int = 2160, bin_size: int = 16, subdiv: int = 7,
                        tex_size: int = 2048, distance: float = 8.0) -> Scene:
    """The displaced icosphere with the build's shading extensions: bilinear
    filtering of the 2048^2 noise texture, one directional and one point
    light (the reference's GPU shader has neither)."""
    s = icosphere_scene(width, height, bin_size, subdiv, tex_size, distance, sample=SAMPLE_BILINEAR)
    s.name = f"icosphere{subdiv}_lit"
    s.lights = [Light(LIGHT_DIRECTIONAL, (1.0, 0.95, 0.9), 4.0, (0.577, -0.577, -0.577)),
                Light(LIGHT_POINT, (0.4, 0.6, 1.0), 30.0, (2.0, 1.5, 3.0))]
    return s
