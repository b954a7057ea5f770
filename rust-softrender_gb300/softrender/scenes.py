"""Seeded synthetic workloads for the rendering path.

Every generator is deterministic for a given seed and returns plain numpy
arrays (float32 attribute planes, uint32 indices, uint32 RGBA8 texels) that
are handed unchanged to the GPU library and to any CPU checker, so both see
bit-identical inputs.  Geometry math runs in float64 and is rounded to
float32 once at the end.

Workloads (sizes as in the benchmark configurations):
  icosphere_scene      icosphere subdivided 4x (2,562 v / 5,120 tris), radial
                       jitter +-2%, 1024x1024 RGBA f32 + depth, Blinn-Phong
  grid_sphere_scene    displaced grid-sphere 512x1024 quads (1,048,576 tris),
                       3-octave value noise 5%, camera near the surface, clip
                       GS, 3840x2160 RGBA8 + depth, textured Blinn-Phong
  stress_scene         16,777,216 tiny (~0.5 px^2) clip-space triangles plus
                       4,096 large alpha triangles, over-blend, stencil
  batch_instances      256 displaced spheres, 500..200k tris, 256^2..2048^2
  serve_requests       Poisson request stream for the serving loop
"""
import math
from dataclasses import dataclass, field
from typing import List, Optional

import numpy as np

from . import _abi as A


# ------------------------------------------------------------------ matrices
def perspective(aspect, fovy, znear, zfar):
    """nalgebra Perspective3::new(aspect, fovy, znear, zfar).to_homogeneous()."""
    f = 1.0 / math.tan(fovy / 2.0)
    m = np.zeros((4, 4))
    m[0, 0] = f / aspect
    m[1, 1] = f
    m[2, 2] = (zfar + znear) / (znear - zfar)
    m[2, 3] = 2.0 * zfar * znear / (znear - zfar)
    m[3, 2] = -1.0
    return m


def look_at_rh(eye, target, up):
    """nalgebra Isometry3::look_at_rh(eye, target, up).to_homogeneous()."""
    eye, target, up = (np.asarray(v, dtype=np.float64) for v in (eye, target, up))
    f = target - eye
    f /= np.linalg.norm(f)
    s = np.cross(f, up)
    s /= np.linalg.norm(s)
    u = np.cross(s, f)
    m = np.eye(4)
    m[0, :3], m[1, :3], m[2, :3] = s, u, -f
    m[0, 3], m[1, 3], m[2, 3] = -s @ eye, -u @ eye, f @ eye
    return m


def make_uniforms(model=None, view=None, projection=None, camera=(0, 0, 3),
                  light_dir=(1.0, 1.0, 1.0), color=(0.1, 0.5, 0.1), intensity=4.0,
                  shininess=32.0, ior=1.45, gamma=2.2):
    """sr_uniforms with the derived pv / mvp filled by the same FP32 product
    the library uses (projection*view, then *model)."""
    u = A.SrUniforms()
    model = np.eye(4) if model is None else np.asarray(model, dtype=np.float64)
    mit = np.linalg.inv(model).T
    view = np.eye(4) if view is None else view
    projection = np.eye(4) if projection is None else projection
    for name, m in (("model", model), ("mit", mit), ("view", view), ("projection", projection)):
        getattr(u, name)[:] = [float(v) for v in np.asarray(m, dtype=np.float32).reshape(-1)]
    u.camera[:] = [float(v) for v in np.float32([camera[0], camera[1], camera[2], 1.0])]
    ld = np.asarray(light_dir, dtype=np.float64)
    ld = ld / np.linalg.norm(ld)
    u.light_dir[:] = [float(v) for v in np.float32([ld[0], ld[1], ld[2], 0.0])]
    u.light_pos[:] = [5.0, 5.0, 5.0, 1.0]
    lin = np.float32(np.asarray(color, dtype=np.float64) ** 2.2)
    u.color[:] = [float(lin[0]), float(lin[1]), float(lin[2]), 1.0]
    u.intensity, u.shininess, u.ior, u.gamma = intensity, shininess, ior, gamma
    lights = [((-1, 1, -1), 9.0, (1.0, 1.0, 1.0)), ((1, 1, 1), 9.0, (0.6, 0.6, 1.0)),
              ((0, 3, -1), 25.0, (1.0, 0.3, 0.3)), ((-2, -1, 1), 25.0, (0.7, 1.0, 0.7))]
    for i, (p, inten, c) in enumerate(lights):
        u.light_pos4[i][:] = [float(p[0]), float(p[1]), float(p[2]), 1.0]
        u.light_color[i][:] = [c[0], c[1], c[2], 1.0]
        u.light_int4[i] = inten
    derive_uniforms(u)
    return u


def _mm(a, b):
    """FP32 Matrix4*Matrix4 with each element summed k = 0..3 left to right."""
    a = np.asarray(a, dtype=np.float32).reshape(4, 4)
    b = np.asarray(b, dtype=np.float32).reshape(4, 4)
    out = np.zeros((4, 4), dtype=np.float32)
    for i in range(4):
        for j in range(4):
            acc = np.float32(a[i, 0] * b[0, j])
            for k in range(1, 4):
                acc = np.float32(acc + np.float32(a[i, k] * b[k, j]))
            out[i, j] = acc
    return out


def derive_uniforms(u):
    pv = _mm(np.array(u.projection[:]), np.array(u.view[:]))
    mvp = _mm(pv, np.array(u.model[:]))
    u.pv[:] = [float(v) for v in pv.reshape(-1)]
    u.mvp[:] = [float(v) for v in mvp.reshape(-1)]


# ------------------------------------------------------------------- scene
@dataclass
class Scene:
    """One draw: mesh planes + indices + pipeline state + framebuffer shape."""
    planes: List[np.ndarray]
    indices: np.ndarray
    width: int
    height: int
    color_format: int = A.SR_COLOR_RGBA32F
    depth: bool = True
    stencil: bool = False
    prim: int = A.SR_PRIM_TRIANGLE
    vs: str = "mvp_pos_nrm"
    gs_mode: int = A.SR_GS_NONE
    gs: str = "clip"
    fs: str = "blinn_phong_dir"
    blend: str = "replace"
    cull: int = A.SR_CULL_NONE
    aa_lines: bool = False
    tile: tuple = (128, 128)
    stencil_ref: int = 0
    stencil_test: int = A.SR_STENCIL_ALWAYS
    stencil_op: int = A.SR_STENCIL_KEEP
    stencil_wrap: int = 1
    viewport: tuple = None
    uniforms: A.SrUniforms = None
    texture: Optional[np.ndarray] = None      # (h, w) uint32 RGBA8 or (h, w, 4) float32 RGBA
    tex_filter: int = A.SR_SAMPLE_BILINEAR
    tex_edge: int = A.SR_SAMPLE_CLAMP
    clear_color: tuple = (0.0, 0.0, 0.0, 1.0)
    name: str = ""
    extra: dict = field(default_factory=dict)

    def __post_init__(self):
        if self.viewport is None:
            self.viewport = (0.0, 0.0, float(self.width), float(self.height), 0.0, 1.0)
        if self.uniforms is None:
            self.uniforms = make_uniforms()

    @property
    def n_verts(self):
        return int(self.planes[0].shape[0])

    @property
    def n_tris(self):
        return int(self.indices.shape[0]) // 3

    def clear_bytes(self):
        if self.color_format == A.SR_COLOR_RGBA8:
            return bytes(int(min(255, max(0, c * 255.0))) for c in self.clear_color)
        return np.asarray(self.clear_color, dtype=np.float32).tobytes()

    def mesh_bytes(self):
        return sum(p.nbytes for p in self.planes) + self.indices.nbytes

    def fb_bytes_per_pixel(self):
        b = 16 if self.color_format == A.SR_COLOR_RGBA32F else 4 if self.color_format == A.SR_COLOR_RGBA8 else 0
        return b + (4 if self.depth else 0) + (1 if self.stencil else 0)

    def algorithmic_bytes(self):
        """Attribute planes + u32 indices + texture (once) + 2 x W x H x planes."""
        tex = 0 if self.texture is None else self.texture.nbytes
        return self.mesh_bytes() + tex + 2 * self.width * self.height * self.fb_bytes_per_pixel()


# ----------------------------------------------------------------- geometry
def icosphere(subdiv):
    t = (1.0 + math.sqrt(5.0)) / 2.0
    verts = [(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0), (0, -1, t), (0, 1, t),
             (0, -1, -t), (0, 1, -t), (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)]
    verts = [np.array(v, dtype=np.float64) / np.linalg.norm(v) for v in verts]
    faces = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4),
             (11, 10, 2), (10, 7, 6), (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8),
             (3, 8, 9), (4, 9, 5), (2, 4, 11), (6, 2, 10), (8, 6, 7), (9, 8, 1)]
    for _ in range(subdiv):
        cache = {}
        nf = []

        def mid(a, b):
            key = (a, b) if a < b else (b, a)
            if key not in cache:
                m = verts[a] + verts[b]
                verts.append(m / np.linalg.norm(m))
                cache[key] = len(verts) - 1
            return cache[key]
        for a, b, c in faces:
            ab, bc, ca = mid(a, b), mid(b, c), mid(c, a)
            nf += [(a, ab, ca), (b, bc, ab), (c, ca, bc), (ab, bc, ca)]
        faces = nf
    return np.array(verts), np.array(faces, dtype=np.uint32)


def _value_noise3(p, seed, octaves=3):
    """3-octave value noise in [-1, 1]: hashed lattice values, smoothstep
    trilinear interpolation, frequency x2 / amplitude x0.5 per octave."""
    rng = np.random.default_rng(seed)
    perm = rng.permutation(256).astype(np.int64)
    vals = rng.uniform(-1.0, 1.0, 256)
    total = np.zeros(p.shape[0])
    norm = 0.0
    amp, freq = 1.0, 2.0
    for _ in range(octaves):
        q = p * freq + 17.0
        i0 = np.floor(q).astype(np.int64)
        f = q - i0
        s = f * f * (3.0 - 2.0 * f)
        acc = np.zeros(p.shape[0])
        for dx in (0, 1):
            for dy in (0, 1):
                for dz in (0, 1):
                    h = perm[(i0[:, 0] + dx) & 255]
                    h = perm[(h + i0[:, 1] + dy) & 255]
                    h = perm[(h + i0[:, 2] + dz) & 255]
                    w = ((s[:, 0] if dx else 1 - s[:, 0]) * (s[:, 1] if dy else 1 - s[:, 1])
                         * (s[:, 2] if dz else 1 - s[:, 2]))
                    acc += w * vals[h]
        total += amp * acc
        norm += amp
        amp *= 0.5
        freq *= 2.0
    return total / norm


def _vertex_normals(pos, tris):
    a, b, c = pos[tris[:, 0]], pos[tris[:, 1]], pos[tris[:, 2]]
    fn = np.cross(b - a, c - a)
    n = np.zeros_like(pos)
    for k in range(3):
        np.add.at(n, tris[:, k], fn)
    ln = np.linalg.norm(n, axis=1, keepdims=True)
    ln[ln == 0] = 1.0
    return n / ln


def grid_sphere(n_lat, n_lon, seed, amplitude=0.05):
    """(n_lat+1) x (n_lon+1) lat-long grid, 2*n_lat*n_lon triangles, uv in [0,1]^2,
    radius 1 + amplitude * value_noise."""
    th = np.linspace(0.0, math.pi, n_lat + 1)
    ph = np.linspace(0.0, 2.0 * math.pi, n_lon + 1)
    T, P = np.meshgrid(th, ph, indexing="ij")
    unit = np.stack([np.sin(T) * np.cos(P), np.cos(T), np.sin(T) * np.sin(P)], axis=-1).reshape(-1, 3)
    r = 1.0 + amplitude * _value_noise3(unit, seed)
    pos = unit * r[:, None]
    uv = np.stack([np.broadcast_to(ph[None, :] / (2 * math.pi), T.shape),
                   np.broadcast_to(th[:, None] / math.pi, T.shape)], axis=-1).reshape(-1, 2)
    i = np.arange(n_lat)[:, None]
    j = np.arange(n_lon)[None, :]
    v00 = (i * (n_lon + 1) + j).reshape(-1)
    v01 = v00 + 1
    v10 = v00 + (n_lon + 1)
    v11 = v10 + 1
    tris = np.stack([np.stack([v00, v10, v01], 1), np.stack([v01, v10, v11], 1)], 1).reshape(-1, 3)
    tris = tris.astype(np.uint32)
    nrm = _vertex_normals(pos, tris)
    return pos, nrm, uv, tris


def procedural_texture(size, seed):
    """size x size RGBA8 (alpha 255): value-noise colour bands over a checker."""
    rng = np.random.default_rng(seed)
    y, x = np.mgrid[0:size, 0:size]
    p = np.stack([x.reshape(-1) / size * 4.0, y.reshape(-1) / size * 4.0,
                  np.zeros(size * size)], axis=1)
    n = _value_noise3(p, int(rng.integers(1 << 30)))
    checker = (((x // 32) + (y // 32)) & 1).reshape(-1)
    base = rng.uniform(0.2, 0.9, (2, 3))
    col = base[checker] * (0.75 + 0.25 * n[:, None])
    col8 = np.clip(np.round(col * 255.0), 0, 255).astype(np.uint32)
    tex = col8[:, 0] | (col8[:, 1] << 8) | (col8[:, 2] << 16) | (np.uint32(255) << 24)
    return tex.astype(np.uint32).reshape(size, size)


def _planes(*cols):
    out = []
    for c in cols:
        c = np.asarray(c)
        if c.ndim == 1:
            out.append(np.ascontiguousarray(c, dtype=np.float32))
        else:
            out += [np.ascontiguousarray(c[:, k], dtype=np.float32) for k in range(c.shape[1])]
    return out


# ------------------------------------------------------------------ scenes
def icosphere_scene(width=1024, height=1024, seed=1, subdiv=4, **kw):
    """Plain pipeline, small: icosphere subdiv 4 (2,562 v, 5,120 tris), radial
    jitter uniform +-2%, fov 60 deg, near 0.1, far 100, camera at distance 3,
    RGBA f32 + f32 depth, Blinn-Phong with one directional light."""
    v, f = icosphere(subdiv)
    rng = np.random.default_rng(seed)
    pos = v * rng.uniform(0.98, 1.02, v.shape[0])[:, None]
    nrm = v
    cam = (0.0, 0.0, 3.0)
    proj = perspective(width / height, math.radians(60.0), 0.1, 100.0)
    view = look_at_rh(cam, (0, 0, 0), (0, 1, 0))
    u = make_uniforms(view=view, projection=proj, camera=cam)
    sc = Scene(planes=_planes(pos, nrm), indices=f.reshape(-1).astype(np.uint32), width=width,
               height=height, color_format=A.SR_COLOR_RGBA32F, vs="mvp_pos_nrm",
               fs="blinn_phong_dir", uniforms=u, clear_color=(0.01, 0.01, 0.01, 1.0),
               name="icosphere4_%dx%d" % (width, height))
    for k, val in kw.items():
        setattr(sc, k, val)
    return sc


GRID_SPHERE_CAMERA = dict(eye=(0.55, 0.35, 1.45), target=(-0.1, -0.05, 0.0))


def grid_sphere_scene(width=3840, height=2160, n_lat=512, n_lon=1024, seed=2, tex_seed=3,
                      tex_size=1024, camera=None, **kw):
    """Plain pipeline, large: displaced grid-sphere (n_lat x n_lon quads), camera
    close to the surface so a large share of triangles leaves the frustum,
    clip geometry shader, RGBA8 + f32 depth, bilinear textured Blinn-Phong."""
    pos, nrm, uv, tris = grid_sphere(n_lat, n_lon, seed)
    cam = camera or GRID_SPHERE_CAMERA
    proj = perspective(width / height, math.radians(60.0), 0.1, 100.0)
    view = look_at_rh(cam["eye"], cam["target"], (0, 1, 0))
    u = make_uniforms(view=view, projection=proj, camera=cam["eye"], color=(0.8, 0.8, 0.8))
    tex = procedural_texture(tex_size, tex_seed)
    sc = Scene(planes=_planes(pos, nrm, uv), indices=tris.reshape(-1), width=width, height=height,
               color_format=A.SR_COLOR_RGBA8, vs="mvp_pos_nrm_uv", gs_mode=A.SR_GS_CLIP,
               fs="textured_blinn_phong", uniforms=u, texture=tex,
               clear_color=(0.05, 0.05, 0.08, 1.0),
               name="gridsphere_%dx%d_%dx%d" % (n_lat, n_lon, width, height))
    for k, val in kw.items():
        setattr(sc, k, val)
    return sc


def _clip_from_screen(sx, sy, z_ndc, W, H):
    """Inverse of ClipVertex::normalize for w = 1 and viewport (0,0,W,H,0,1)."""
    x = (sx - W / 2.0) / (W / 2.0)
    y = (H / 2.0 - sy) / (H / 2.0)
    return x, y, z_ndc


def _pack_rgba8(r, g, b, a):
    c = (np.clip(r, 0, 255).astype(np.uint32) | (np.clip(g, 0, 255).astype(np.uint32) << 8)
         | (np.clip(b, 0, 255).astype(np.uint32) << 16) | (np.clip(a, 0, 255).astype(np.uint32) << 24))
    return c.astype(np.uint32)


def stress_scene(n_tiny=16777216, n_large=4096, size=2048, seed=6, seed_large=7, wrap=1, **kw):
    """Stress on ordering and tiny triangles: n_tiny triangles of area ~0.5 px^2
    (fixed right-isosceles shape, random orientation, centroid uniform in
    [0,size)^2), then n_large large overlapping triangles with alpha uniform in
    [0.2, 0.8] drawn back to front after them; given in clip space with w = 1,
    RGBA8 + f32 depth + u8 stencil, over-blend, stencil Always / Increment."""
    rng = np.random.default_rng(seed)
    W = H = size
    c = rng.uniform(0.0, size, (n_tiny, 2))
    ang = rng.uniform(0.0, 2.0 * math.pi, n_tiny)
    # right isosceles triangle with legs 1 (area 0.5), centroid at the origin
    base = np.array([[-1.0 / 3, -1.0 / 3], [2.0 / 3, -1.0 / 3], [-1.0 / 3, 2.0 / 3]])
    ca, sa = np.cos(ang), np.sin(ang)
    tiny = np.empty((n_tiny, 3, 2))
    for k in range(3):
        tiny[:, k, 0] = c[:, 0] + base[k, 0] * ca - base[k, 1] * sa
        tiny[:, k, 1] = c[:, 1] + base[k, 0] * sa + base[k, 1] * ca
    zt = rng.uniform(0.2, 0.95, n_tiny)
    col = rng.integers(0, 256, (n_tiny, 3))
    rng2 = np.random.default_rng(seed_large)
    large = rng2.uniform(-0.1 * size, 1.1 * size, (n_large, 3, 2))
    zl = np.linspace(0.1, -0.9, n_large)       # later = nearer (back to front)
    coll = rng2.integers(0, 256, (n_large, 3))
    al = np.round(rng2.uniform(0.2, 0.8, n_large) * 255.0)
    n = n_tiny + n_large
    sx = np.concatenate([tiny[:, :, 0], large[:, :, 0]]).reshape(-1)
    sy = np.concatenate([tiny[:, :, 1], large[:, :, 1]]).reshape(-1)
    z = np.repeat(np.concatenate([zt, zl]), 3)
    x, y, zz = _clip_from_screen(sx, sy, z, W, H)
    rgb = np.repeat(np.concatenate([col, coll]), 3, axis=0)
    alpha = np.repeat(np.concatenate([np.full(n_tiny, 255.0), al]), 3)
    packed = _pack_rgba8(rgb[:, 0], rgb[:, 1], rgb[:, 2], alpha)
    planes = [np.ascontiguousarray(x, dtype=np.float32), np.ascontiguousarray(y, dtype=np.float32),
              np.ascontiguousarray(zz, dtype=np.float32), packed.view(np.float32).copy()]
    idx = np.arange(3 * n, dtype=np.uint32)
    sc = Scene(planes=planes, indices=idx, width=W, height=H, color_format=A.SR_COLOR_RGBA8,
               stencil=True, vs="clip_rgba8", fs="vertex_color", blend="over",
               stencil_test=A.SR_STENCIL_ALWAYS, stencil_op=A.SR_STENCIL_INCREMENT,
               stencil_wrap=wrap, clear_color=(0.0, 0.0, 0.0, 1.0),
               name="stress_%d+%d_%d" % (n_tiny, n_large, size))
    for k, val in kw.items():
        setattr(sc, k, val)
    return sc


def sliver_scene(n=4000, size=256, seed=9, **kw):
    """Nearly collinear triangles (perpendicular offsets 1e-7..1e-2 px, lengths
    up to half the frame) in clip space with w = 1: their computed barycentric
    coordinates are dominated by rounding, which exercises the exact handling
    of coverage outside the bounding box."""
    rng = np.random.default_rng(seed)
    W = H = size
    p0 = rng.uniform(-0.1 * size, 1.1 * size, (n, 2))
    ang = rng.uniform(0.0, 2.0 * math.pi, n)
    length = np.exp(rng.uniform(math.log(0.5), math.log(0.5 * size), n))
    d = np.stack([np.cos(ang), np.sin(ang)], 1)
    nrm = np.stack([-d[:, 1], d[:, 0]], 1)
    off = np.exp(rng.uniform(math.log(1e-7), math.log(1e-2), n)) * rng.choice([-1.0, 1.0], n)
    t2 = rng.uniform(0.05, 0.95, n)
    v0 = p0
    v1 = p0 + d * length[:, None]
    v2 = p0 + d * (length * t2)[:, None] + nrm * off[:, None]
    tri = np.stack([v0, v1, v2], 1)
    z = rng.uniform(-0.9, 0.9, (n, 3))
    x, y, zz = _clip_from_screen(tri[:, :, 0].reshape(-1), tri[:, :, 1].reshape(-1), z.reshape(-1), W, H)
    col = rng.integers(0, 256, (3 * n, 3))
    packed = _pack_rgba8(col[:, 0], col[:, 1], col[:, 2], np.full(3 * n, 255))
    planes = [np.ascontiguousarray(x, dtype=np.float32), np.ascontiguousarray(y, dtype=np.float32),
              np.ascontiguousarray(zz, dtype=np.float32), packed.view(np.float32).copy()]
    sc = Scene(planes=planes, indices=np.arange(3 * n, dtype=np.uint32), width=W, height=H,
               color_format=A.SR_COLOR_RGBA8, vs="clip_rgba8", fs="vertex_color", tile=(32, 32),
               name="slivers_%d_%d" % (n, size))
    for k, val in kw.items():
        setattr(sc, k, val)
    return sc


def random_camera(rng, dist_lo=2.0, dist_hi=6.0):
    d = rng.uniform(dist_lo, dist_hi)
    th = rng.uniform(0.2, math.pi - 0.2)
    ph = rng.uniform(0.0, 2.0 * math.pi)
    eye = (d * math.sin(th) * math.cos(ph), d * math.cos(th), d * math.sin(th) * math.sin(ph))
    return eye


def sphere_mesh_for_tris(n_tris, seed):
    """Displaced grid-sphere with about n_tris triangles (n_lon = 2 n_lat)."""
    n_lat = max(2, int(round(math.sqrt(n_tris / 4.0))))
    pos, nrm, uv, tris = grid_sphere(n_lat, 2 * n_lat, seed)
    return _planes(pos, nrm), tris.reshape(-1)


def batch_instances(n=256, seed=4, tri_lo=500, tri_hi=200000,
                    resolutions=(256, 512, 1024, 2048)):
    """Independent render instances: (planes, indices, width, height, uniforms)."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        t = int(round(math.exp(rng.uniform(math.log(tri_lo), math.log(tri_hi)))))
        res = int(resolutions[rng.integers(len(resolutions))])
        planes, idx = sphere_mesh_for_tris(t, seed * 100003 + i)
        eye = random_camera(rng)
        proj = perspective(1.0, math.radians(60.0), 0.1, 100.0)
        view = look_at_rh(eye, (0, 0, 0), (0, 1, 0))
        u = make_uniforms(view=view, projection=proj, camera=eye)
        out.append(Scene(planes=planes, indices=idx, width=res, height=res,
                         color_format=A.SR_COLOR_RGBA8, vs="mvp_pos_nrm", fs="blinn_phong_dir",
                         uniforms=u, name="inst%d" % i))
    return out


def served_workload(rate=2000.0, duration=10.0, seed=5, pool=12, tri_lo=1000, tri_hi=500000,
                    res_lo=(128, 128), res_hi=(1920, 1080)):
    """Request stream of the serving benchmark: a pool of resident seeded
    sphere meshes (triangle counts log-uniform in [tri_lo, tri_hi]) and
    Poisson arrivals at `rate` per second for `duration` seconds; each request
    takes a pool mesh, a random camera and a resolution with width and height
    log-uniform between res_lo and res_hi, RGBA8 + f32 depth, Blinn-Phong.
    Returns (meshes, requests): meshes = [(planes, indices)], requests =
    [(arrival_s, mesh_index, Scene)]."""
    rng = np.random.default_rng(seed)
    meshes = []
    for i in range(pool):
        t = int(round(math.exp(rng.uniform(math.log(tri_lo), math.log(tri_hi)))))
        meshes.append(sphere_mesh_for_tris(t, seed * 1000 + i))
    n = int(rate * duration)
    arrivals = np.cumsum(rng.exponential(1.0 / rate, n))
    reqs = []
    for k in range(n):
        mi = int(rng.integers(pool))
        w = int(round(math.exp(rng.uniform(math.log(res_lo[0]), math.log(res_hi[0])))))
        h = int(round(math.exp(rng.uniform(math.log(res_lo[1]), math.log(res_hi[1])))))
        eye = random_camera(rng)
        u = make_uniforms(view=look_at_rh(eye, (0, 0, 0), (0, 1, 0)),
                          projection=perspective(w / h, math.radians(60.0), 0.1, 100.0), camera=eye)
        planes, idx = meshes[mi]
        reqs.append((float(arrivals[k]), mi, Scene(planes=planes, indices=idx, width=w, height=h,
                                                   color_format=A.SR_COLOR_RGBA8, vs="mvp_pos_nrm",
                                                   fs="blinn_phong_dir", uniforms=u, name="req%d" % k)))
    return meshes, reqs


def lines_scene(n=600, size=200, seed=12, prim=A.SR_PRIM_LINE, outside=0.25, **kw):
    """Lines (or points, prim=SR_PRIM_POINT) with random end points in clip
    space (w = 1; about `outside` of the end points beyond the frustum, so the
    clipping arms have work), depth in (-0.9, 0.9) NDC, RGBA8-packed vertex
    colours; vertex shader clip_rgba8, fragment shader vertex_color."""
    rng = np.random.default_rng(seed)
    W = H = size
    nv = n * (2 if prim == A.SR_PRIM_LINE else 1)
    lo, hi = -outside * size, (1.0 + outside) * size
    sx = rng.uniform(lo, hi, nv)
    sy = rng.uniform(lo, hi, nv)
    if prim == A.SR_PRIM_LINE:
        # mostly short segments, some long ones crossing tiles
        ln = np.exp(rng.uniform(math.log(0.5), math.log(0.6 * size), n))
        ang = rng.uniform(0.0, 2.0 * math.pi, n)
        sx[1::2] = sx[0::2] + np.cos(ang) * ln
        sy[1::2] = sy[0::2] + np.sin(ang) * ln
    z = rng.uniform(-0.9, 0.9, nv)
    x, y, zz = _clip_from_screen(sx, sy, z, W, H)
    col = rng.integers(0, 256, (nv, 4))
    col[:, 3] = rng.integers(128, 256, nv)
    packed = _pack_rgba8(col[:, 0], col[:, 1], col[:, 2], col[:, 3])
    planes = [np.ascontiguousarray(x, dtype=np.float32), np.ascontiguousarray(y, dtype=np.float32),
              np.ascontiguousarray(zz, dtype=np.float32), packed.view(np.float32).copy()]
    sc = Scene(planes=planes, indices=np.arange(nv, dtype=np.uint32), width=W, height=H,
               color_format=A.SR_COLOR_RGBA8, vs="clip_rgba8", fs="vertex_color", prim=prim, tile=(32, 32),
               name="%s_%d_%d" % ("lines" if prim == A.SR_PRIM_LINE else "points", n, size))
    for k, val in kw.items():
        setattr(sc, k, val)
    return sc
