"""ctypes front end of the CPU oracle (oracle/sr_oracle.cpp).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py, never by the product library.
"""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def _load_build():
    import importlib.util
    spec = importlib.util.spec_from_file_location("sr_oracle_build", os.path.join(HERE, "build.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


_build = _load_build()

_lib = None


class OrDraw(C.Structure):
    _fields_ = [
        ("planes", C.POINTER(C.POINTER(C.c_float))), ("n_planes", C.c_uint32),
        ("n_verts", C.c_uint32), ("indices", C.POINTER(C.c_uint32)), ("n_indices", C.c_uint64),
        ("prim", C.c_uint32), ("vs", C.c_char_p), ("gs_mode", C.c_uint32), ("gs", C.c_char_p),
        ("viewport", C.c_float * 6), ("cull", C.c_uint32), ("fs", C.c_char_p),
        ("blend", C.c_char_p), ("aa_lines", C.c_uint32), ("tile_w", C.c_uint32),
        ("tile_h", C.c_uint32), ("stencil_ref", C.c_uint32), ("stencil_test", C.c_uint32),
        ("stencil_op", C.c_uint32), ("stencil_wrap", C.c_uint32),
        ("texture", C.c_void_p), ("tex_w", C.c_uint32), ("tex_h", C.c_uint32),
        ("tex_filter", C.c_uint32), ("tex_edge", C.c_uint32), ("tex_f32", C.c_uint32),
        ("uniforms", C.c_void_p),
    ]


class OrFb(C.Structure):
    _fields_ = [("width", C.c_uint32), ("height", C.c_uint32), ("color_format", C.c_uint32),
                ("color", C.c_void_p), ("depth", C.POINTER(C.c_float)),
                ("stencil", C.POINTER(C.c_uint8))]


class OrStats(C.Structure):
    _fields_ = [("triangles_generated", C.c_uint64), ("fragments", C.c_uint64),
                ("tiles", C.c_uint64), ("nan_bbox", C.c_uint32), ("status", C.c_uint32),
                ("vertex_s", C.c_double), ("geometry_s", C.c_double), ("raster_s", C.c_double)]


def lib():
    global _lib
    if _lib is None:
        path = _build.build()
        L = C.CDLL(path)
        L.or_render.argtypes = [C.POINTER(OrDraw), C.POINTER(OrFb), C.c_int, C.c_uint32,
                                C.c_uint32, C.POINTER(OrStats)]
        L.or_render.restype = C.c_int
        L.or_render_strided.argtypes = [C.POINTER(OrDraw), C.POINTER(OrFb), C.c_int, C.c_uint32, C.c_uint32,
                                        C.c_uint32, C.POINTER(OrStats)]
        L.or_render_strided.restype = C.c_int
        L.or_clear.argtypes = [C.POINTER(OrFb), C.c_void_p]
        L.or_tiles.argtypes = [C.c_uint32] * 4 + [C.POINTER(C.c_uint32), C.c_uint32,
                                                  C.POINTER(C.c_uint32)]
        L.or_normalize.argtypes = [C.POINTER(C.c_float), C.POINTER(C.c_float), C.POINTER(C.c_float)]
        L.or_clip_triangle.argtypes = [C.POINTER(C.c_float)] * 3 + [C.c_uint32, C.POINTER(C.c_float),
                                                                    C.c_uint32]
        L.or_clip_triangle.restype = C.c_uint32
        L.or_raster_tris.argtypes = [C.POINTER(OrDraw), C.c_uint32, C.c_uint32, C.c_void_p, C.c_uint64,
                                     C.POINTER(C.c_uint64)]
        L.or_powf.argtypes = [C.c_float, C.c_float]
        L.or_powf.restype = C.c_float
        L.or_u8_unit.argtypes = [C.c_uint32]
        L.or_u8_unit.restype = C.c_float
        L.or_coordinate_into_index.argtypes = [C.c_uint32, C.c_uint32, C.c_uint32]
        L.or_coordinate_into_index.restype = C.c_uint64
        L.or_coordinate_from_index.argtypes = [C.c_uint64, C.c_uint32, C.POINTER(C.c_uint32),
                                               C.POINTER(C.c_uint32)]
        _lib = L
    return _lib


class Framebuffer:
    """Host SoA planes: colour (H*W*4 f32 or H*W u32), depth (f32), stencil (u8)."""

    def __init__(self, width, height, color_format, depth=True, stencil=False):
        self.width, self.height, self.color_format = width, height, color_format
        n = width * height
        if color_format == 1:
            self.color = np.zeros((height, width, 4), dtype=np.float32)
        elif color_format == 2:
            self.color = np.zeros((height, width), dtype=np.uint32)
        else:
            self.color = None
        self.depth = np.zeros((height, width), dtype=np.float32) if depth else None
        self.stencil = np.zeros((height, width), dtype=np.uint8) if stencil else None
        self._n = n

    def _c(self):
        fb = OrFb()
        fb.width, fb.height, fb.color_format = self.width, self.height, self.color_format
        fb.color = self.color.ctypes.data if self.color is not None else None
        fb.depth = self.depth.ctypes.data_as(C.POINTER(C.c_float)) if self.depth is not None else None
        fb.stencil = self.stencil.ctypes.data_as(C.POINTER(C.c_uint8)) if self.stencil is not None else None
        return fb

    def clear(self, color_bytes):
        buf = C.create_string_buffer(bytes(color_bytes), 16)
        fb = self._c()
        lib().or_clear(C.byref(fb), buf)


def framebuffer_for(scene):
    fb = Framebuffer(scene.width, scene.height, scene.color_format, scene.depth, scene.stencil)
    fb.clear(scene.clear_bytes())
    return fb


def _draw(scene, keep):
    planes = [np.ascontiguousarray(p, dtype=np.float32).reshape(-1) for p in scene.planes]
    if any(p.shape[0] != planes[0].shape[0] for p in planes):
        raise ValueError("every attribute plane must hold one value per vertex")
    keep += planes
    parr = (C.POINTER(C.c_float) * len(planes))(*[p.ctypes.data_as(C.POINTER(C.c_float)) for p in planes])
    keep.append(parr)
    idx = np.ascontiguousarray(scene.indices, dtype=np.uint32)
    keep.append(idx)
    d = OrDraw()
    d.planes = parr
    d.n_planes = len(planes)
    d.n_verts = scene.n_verts
    d.indices = idx.ctypes.data_as(C.POINTER(C.c_uint32))
    d.n_indices = idx.shape[0]
    d.prim = scene.prim
    d.vs = scene.vs.encode()
    d.gs_mode = scene.gs_mode
    d.gs = scene.gs.encode()
    d.viewport[:] = list(scene.viewport)
    d.cull = scene.cull
    d.fs = scene.fs.encode()
    d.blend = scene.blend.encode()
    d.aa_lines = int(scene.aa_lines)
    d.tile_w, d.tile_h = scene.tile
    d.stencil_ref = scene.stencil_ref
    d.stencil_test, d.stencil_op, d.stencil_wrap = scene.stencil_test, scene.stencil_op, scene.stencil_wrap
    if scene.texture is not None:
        if np.asarray(scene.texture).dtype == np.float32:     # RGBA f32 texels, (h, w, 4)
            tex = np.ascontiguousarray(scene.texture, dtype=np.float32)
            d.tex_f32 = 1
        else:                                                  # RGBA8 texels, (h, w) uint32
            tex = np.ascontiguousarray(scene.texture, dtype=np.uint32)
        keep.append(tex)
        d.texture = tex.ctypes.data
        d.tex_h, d.tex_w = tex.shape[:2]
    d.tex_filter, d.tex_edge = scene.tex_filter, scene.tex_edge
    d.uniforms = C.addressof(scene.uniforms)
    return d


def raster_tris(scene):
    """(n, 3, 4) float32 screen positions of the triangles the fragment stage
    rasterises for `scene` (after vertex and geometry stages)."""
    keep = []
    d = _draw(scene, keep)
    n = C.c_uint64()
    lib().or_raster_tris(C.byref(d), scene.width, scene.height, None, 0, C.byref(n))
    out = np.empty((max(1, n.value), 3, 4), dtype=np.float32)
    lib().or_raster_tris(C.byref(d), scene.width, scene.height, out.ctypes.data, n.value, C.byref(n))
    return out[:n.value]


def render(scene, fb=None, n_threads=1, tile_begin=0, tile_end=0xFFFFFFFF, tile_step=1):
    """Renders `scene` (softrender.scenes.Scene) into fb (a new cleared one if
    None); returns (fb, stats dict, status).  Only tiles tile_begin,
    tile_begin + tile_step, ... below tile_end are rasterised (all by default;
    a stride gives timing samples spread over the frame)."""
    if fb is None:
        fb = framebuffer_for(scene)
    keep = []
    d = _draw(scene, keep)
    st = OrStats()
    cfb = fb._c()
    if tile_step == 1:
        status = lib().or_render(C.byref(d), C.byref(cfb), n_threads, tile_begin, tile_end, C.byref(st))
    else:
        n = max(0, -(-(min(tile_end, 0xFFFFFFFF) - tile_begin) // tile_step))
        status = lib().or_render_strided(C.byref(d), C.byref(cfb), n_threads, tile_begin, tile_step,
                                         min(n, 0xFFFFFFFF), C.byref(st))
    stats = dict(triangles_generated=st.triangles_generated, fragments=st.fragments,
                 tiles=st.tiles, nan_bbox=st.nan_bbox, vertex_s=st.vertex_s, geometry_s=st.geometry_s,
                 raster_s=st.raster_s)
    return fb, stats, status


def tiles(width, height, tw, th):
    cap = 1 << 16
    out = (C.c_uint32 * (4 * cap))()
    n = C.c_uint32()
    lib().or_tiles(width, height, tw, th, out, cap, C.byref(n))
    return [tuple(out[4 * i:4 * i + 4]) for i in range(n.value)]


def normalize(clip, viewport):
    a = (C.c_float * 4)(*clip)
    v = (C.c_float * 6)(*viewport)
    o = (C.c_float * 4)()
    lib().or_normalize(a, v, o)
    return np.array(o[:], dtype=np.float32)


def clip_triangle(a, b, c, nk=0):
    stride = 4 + nk
    A_ = (C.c_float * stride)(*a)
    B_ = (C.c_float * stride)(*b)
    C_ = (C.c_float * stride)(*c)
    out = (C.c_float * (stride * 3 * 40))()
    n = lib().or_clip_triangle(A_, B_, C_, nk, out, 120)
    return np.array(out[:n * stride], dtype=np.float32).reshape(n, stride)


def u8_unit(c):
    return np.float32(lib().or_u8_unit(int(c)))


def powf(x, y):
    return np.float32(lib().or_powf(float(x), float(y)))
