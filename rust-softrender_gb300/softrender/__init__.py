"""softrender — Python host mirror of softrender's Pipeline builder API over
the GB300 C ABI (include/sr.h).

The reference chain (src/pipeline/mod.rs, stages/{vertex,geometry,fragment}.rs)

    let mut pipeline = Pipeline::from_framebuffer(framebuffer, uniforms);
    pipeline.render_mesh(Triangle, mesh, Some(stencil))
            .run(vertex_shader)              // or .run_to_fragment(viewport, vs)
            .clip_primitives()
            .finish(viewport)
            .with_blend(blend)
            .run(fragment_shader);

reads here as

    pipeline = Pipeline.from_framebuffer(Framebuffer(w, h, RGBA8), uniforms)
    (pipeline.render_mesh(Triangle, mesh, stencil)
             .run("mvp_pos_nrm_uv")
             .clip_primitives()
             .finish(viewport)
             .with_blend("over")
             .run("textured_blinn_phong"))

with shader stages named device functions compiled into the library.  Every
call goes through the CUDA library; there is no CPU path.
"""
import ctypes as C

import numpy as np

from . import _abi as A
from ._lib import SoftrenderError, check, lib

__all__ = ["Framebuffer", "Pipeline", "Mesh", "Texture", "Viewport", "Point", "Line", "Triangle",
           "SoftrenderError", "render_scene", "shader_id"]

Point, Line, Triangle = A.SR_PRIM_POINT, A.SR_PRIM_LINE, A.SR_PRIM_TRIANGLE


def shader_id(name, stage):
    i = C.c_int()
    check(lib().sr_shader_lookup(name.encode(), stage, C.byref(i)), "sr_shader_lookup(%s)" % name)
    return i.value


class Viewport:
    """Viewport<f32> (src/geometry/clipvertex.rs:28-57)."""

    def __init__(self, x, y, width, height, near=0.0, far=1.0):
        self.x, self.y, self.width, self.height, self.near, self.far = x, y, width, height, near, far

    @classmethod
    def from_dimensions(cls, width, height, near=0.0, far=1.0):
        return cls(0.0, 0.0, float(width), float(height), near, far)

    def c(self):
        return A.SrViewport(self.x, self.y, self.width, self.height, self.near, self.far)


class Framebuffer:
    """RenderBuffer<ColorDepthStencilAttachments<C, D, S>> description."""

    def __init__(self, width, height, color_format=A.SR_COLOR_RGBA32F, depth=True, stencil=False):
        self.width, self.height = width, height
        self.color_format, self.depth, self.stencil = color_format, depth, stencil


class Mesh:
    """Mesh<V> (src/mesh.rs:38-64) uploaded as SoA f32 planes + u32 indices."""

    def __init__(self, planes, indices):
        planes = [np.ascontiguousarray(p, dtype=np.float32).reshape(-1) for p in planes]
        idx = np.ascontiguousarray(indices, dtype=np.uint32)
        n = planes[0].shape[0] if planes else 0
        if any(p.shape[0] != n for p in planes):
            raise ValueError("every attribute plane must hold one value per vertex")
        arr = (C.c_void_p * max(1, len(planes)))(*[p.ctypes.data for p in planes])
        h = C.c_void_p()
        check(lib().sr_mesh_upload(arr, len(planes), n, idx.ctypes.data if idx.size else None, idx.size,
                                   C.byref(h)), "sr_mesh_upload")
        self.handle = h
        self.n_verts = n
        self.n_indices = int(idx.size)

    def update(self, planes, indices, stream_ptr=None):
        """Copies new host data of the same shape into the device mesh."""
        planes = [np.ascontiguousarray(p, dtype=np.float32) for p in planes]
        idx = np.ascontiguousarray(indices, dtype=np.uint32)
        arr = (C.c_void_p * max(1, len(planes)))(*[p.ctypes.data for p in planes])
        check(lib().sr_mesh_update(self.handle, arr, len(planes), planes[0].shape[0] if planes else 0,
                                   idx.ctypes.data if idx.size else None, idx.size,
                                   C.c_void_p(stream_ptr) if stream_ptr else None), "sr_mesh_update")

    @property
    def nbytes(self):
        return int(lib().sr_mesh_bytes(self.handle))

    def free(self):
        if self.handle:
            lib().sr_mesh_free(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


class Texture:
    """A texture read by the textured shaders: (h, w) uint32 RGBA8 texels, or
    (h, w, 4) float32 RGBA texels."""

    def __init__(self, texels):
        h = C.c_void_p()
        if np.asarray(texels).dtype == np.float32:
            t = np.ascontiguousarray(texels, dtype=np.float32)
            if t.ndim != 3 or t.shape[2] != 4:
                raise ValueError("RGBA f32 texels must have shape (h, w, 4)")
            check(lib().sr_texture_upload_rgba32f(t.ctypes.data, t.shape[1], t.shape[0], C.byref(h)),
                  "sr_texture_upload_rgba32f")
        else:
            t = np.ascontiguousarray(texels, dtype=np.uint32)
            check(lib().sr_texture_upload(t.ctypes.data, t.shape[1], t.shape[0], C.byref(h)), "sr_texture_upload")
        self.handle = h
        self.width, self.height = t.shape[1], t.shape[0]

    @classmethod
    def view(cls, pipeline):
        """The pipeline's colour attachment read in place as a texture
        (texture-buffer framebuffers, src/framebuffer/texturebuffer.rs)."""
        h = C.c_void_p()
        check(lib().sr_texture_view_framebuffer(pipeline.handle, C.byref(h)), "sr_texture_view_framebuffer")
        t = cls.__new__(cls)
        t.handle = h
        t.width, t.height = pipeline.framebuffer.width, pipeline.framebuffer.height
        t._pipeline = pipeline   # the plane it reads lives as long as the pipeline
        return t

    def update(self, rgba8, stream_ptr=None):
        t = np.ascontiguousarray(rgba8, dtype=np.uint32)
        check(lib().sr_texture_update(self.handle, t.ctypes.data, t.shape[1], t.shape[0],
                                      C.c_void_p(stream_ptr) if stream_ptr else None), "sr_texture_update")

    def free(self):
        if self.handle:
            lib().sr_texture_free(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


class Pipeline:
    """Pipeline<U, F, S> (src/pipeline/mod.rs:60-155)."""

    def __init__(self, framebuffer, uniforms=None):
        self.framebuffer = framebuffer
        desc = A.SrFbDesc(framebuffer.width, framebuffer.height, framebuffer.color_format,
                          1 if framebuffer.depth else 0, 1 if framebuffer.stencil else 0)
        h = C.c_void_p()
        u = C.byref(uniforms) if uniforms is not None else None
        check(lib().sr_pipeline_create(C.byref(desc), u, C.sizeof(A.SrUniforms) if uniforms is not None else 0,
                                       C.byref(h)), "sr_pipeline_create")
        self.handle = h
        self._uniforms = uniforms
        self._keep = []
        self._last_outputs = None   # stage outputs of the previous draw (duplicate())

    @classmethod
    def from_framebuffer(cls, framebuffer, uniforms=None):
        return cls(framebuffer, uniforms)

    # PipelineObject accessors
    def set_uniforms(self, uniforms):
        check(lib().sr_pipeline_set_uniforms(self.handle, C.byref(uniforms), C.sizeof(A.SrUniforms)),
              "sr_pipeline_set_uniforms")
        self._uniforms = uniforms

    def set_stencil(self, test, op, wrap=True):
        """stencil_config_mut() = GenericStencilConfig { op, test } (src/stencil.rs:182-199)."""
        check(lib().sr_pipeline_set_stencil(self.handle, test, op, 1 if wrap else 0), "sr_pipeline_set_stencil")

    def set_stream(self, stream_ptr):
        check(lib().sr_pipeline_set_stream(self.handle, C.c_void_p(stream_ptr) if stream_ptr else None),
              "sr_pipeline_set_stream")

    def clear(self, color):
        """Framebuffer::clear: colour, depth <- f32::MIN, stencil <- 0."""
        if self.framebuffer.color_format == A.SR_COLOR_RGBA8:
            buf = (C.c_uint8 * 4)(*[int(c) for c in color])
        else:
            buf = (C.c_float * 4)(*[float(c) for c in color])
        check(lib().sr_framebuffer_clear(self.handle, buf), "sr_framebuffer_clear")

    def write(self, color=None, depth=None, stencil=None):
        c = np.ascontiguousarray(color) if color is not None else None
        d = np.ascontiguousarray(depth, dtype=np.float32) if depth is not None else None
        s = np.ascontiguousarray(stencil, dtype=np.uint8) if stencil is not None else None
        check(lib().sr_framebuffer_write(self.handle, c.ctypes.data if c is not None else None,
                                         d.ctypes.data if d is not None else None,
                                         s.ctypes.data if s is not None else None), "sr_framebuffer_write")

    def read(self):
        """Returns (color, depth, stencil) host arrays (None for absent planes)."""
        fb = self.framebuffer
        h, w = fb.height, fb.width
        color = None
        if fb.color_format == A.SR_COLOR_RGBA32F:
            color = np.empty((h, w, 4), dtype=np.float32)
        elif fb.color_format == A.SR_COLOR_RGBA8:
            color = np.empty((h, w), dtype=np.uint32)
        depth = np.empty((h, w), dtype=np.float32) if fb.depth else None
        stencil = np.empty((h, w), dtype=np.uint8) if fb.stencil else None
        st = lib().sr_framebuffer_read(self.handle, color.ctypes.data if color is not None else None,
                                       depth.ctypes.data if depth is not None else None,
                                       stencil.ctypes.data if stencil is not None else None)
        if st not in (A.SR_OK, A.SR_ENAN):
            raise SoftrenderError(st, "sr_framebuffer_read")
        return color, depth, stencil

    def sync(self):
        return lib().sr_sync(self.handle)

    def set_profiling(self, enable=True):
        check(lib().sr_pipeline_set_profiling(self.handle, 1 if enable else 0), "sr_pipeline_set_profiling")

    def stats(self):
        s = A.SrStats()
        check(lib().sr_get_stats(self.handle, C.byref(s)), "sr_get_stats")
        out = {f: getattr(s, f) for f, _ in A.SrStats._fields_ if f != "stage_ms"}
        out["stage_ms"] = dict(zip(A.STAGE_NAMES, list(s.stage_ms))) if s.profiled else {}
        return out

    def render_mesh(self, primitive, mesh, stencil=None):
        """Pipeline::render_mesh (mod.rs:146-155) -> VertexShader."""
        if mesh.n_indices % primitive != 0:
            raise SoftrenderError(A.SR_EINVAL, "render_mesh: indices.len() % num_vertices != 0")
        d = A.SrDraw()
        lib().sr_draw_init(C.byref(d))
        d.mesh = mesh.handle
        d.prim = primitive
        d.stencil_ref = 0 if stencil is None else int(stencil)
        return VertexShader(self, d, [mesh])

    def destroy(self):
        if self.handle:
            lib().sr_pipeline_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.destroy()
        except Exception:
            pass


class _Outputs:
    """The outputs of one vertex (or geometry) stage, shared by a stage object
    and its duplicates: the first of them to render computes them, the
    others render from them (sr_draw.reuse)."""

    def __init__(self):
        self.rendered = False


def _copy_draw(d):
    return A.SrDraw.from_buffer_copy(d)


class VertexShader:
    """stages/vertex.rs: run(vs) -> GeometryShader, run_to_fragment(vp, vs) -> FragmentShader."""

    def __init__(self, pipeline, draw, keep):
        self.pipeline, self.draw, self.keep = pipeline, draw, keep

    def duplicate(self):
        """VertexShader::duplicate (vertex.rs:39-50): nothing is processed yet."""
        return VertexShader(self.pipeline, _copy_draw(self.draw), list(self.keep))

    def run(self, vs):
        self.draw.vs = shader_id(vs, A.SR_STAGE_VERTEX)
        return GeometryShader(self.pipeline, self.draw, self.keep, _Outputs())

    def run_to_fragment(self, viewport, vs):
        self.draw.vs = shader_id(vs, A.SR_STAGE_VERTEX)
        self.draw.gs_mode = A.SR_GS_NONE
        self.draw.viewport = viewport.c()
        return FragmentShader(self.pipeline, self.draw, self.keep, None, _Outputs())


class GeometryShader:
    """stages/geometry.rs: clip_primitives(), run(gs) / replace(gs), finish(viewport), duplicate()."""

    def __init__(self, pipeline, draw, keep, vertices):
        self.pipeline, self.draw, self.keep, self.vertices = pipeline, draw, keep, vertices

    def duplicate(self):
        """GeometryShader::duplicate (geometry.rs:40-54): a copy that renders
        from the same processed vertices (SR_REUSE_VERTICES)."""
        return GeometryShader(self.pipeline, _copy_draw(self.draw), list(self.keep), self.vertices)

    def clip_primitives(self):
        self.draw.gs_mode = A.SR_GS_CLIP
        self.draw.gs = shader_id("clip", A.SR_STAGE_GEOMETRY)
        return self

    def run(self, gs):
        self.draw.gs_mode = A.SR_GS_NAMED
        self.draw.gs = shader_id(gs, A.SR_STAGE_GEOMETRY)
        return self

    replace = run

    def finish(self, viewport):
        self.draw.viewport = viewport.c()
        return FragmentShader(self.pipeline, self.draw, self.keep, self.vertices, _Outputs())


class FragmentShader:
    """stages/fragment.rs: with_blend, cull_faces, antialiased_lines, tile_size, duplicate, run."""

    def __init__(self, pipeline, draw, keep, vertices=None, geometry=None):
        self.pipeline, self.draw, self.keep = pipeline, draw, keep
        self.vertices, self.geometry = vertices, geometry

    def duplicate(self):
        """FragmentShader::duplicate (fragment.rs:118-135): the same geometry
        rasterised again with other settings (SR_REUSE_GEOMETRY)."""
        return FragmentShader(self.pipeline, _copy_draw(self.draw), list(self.keep), self.vertices, self.geometry)

    def with_blend(self, blend):
        self.draw.blend = shader_id(blend, A.SR_STAGE_BLEND)
        return self

    def with_default_blend(self):
        self.draw.blend = 0
        return self

    def cull_faces(self, cull):
        self.draw.cull = cull
        return self

    with_faces_culled = cull_faces

    def antialiased_lines(self, enable):
        self.draw.aa_lines = 1 if enable else 0
        return self

    with_antialiased_lines = antialiased_lines

    def tile_size(self, w, h):
        self.draw.tile_w, self.draw.tile_h = w, h
        return self

    with_tile_size = tile_size

    def with_texture(self, texture, filter=A.SR_SAMPLE_BILINEAR, edge=A.SR_SAMPLE_CLAMP):
        self.draw.texture = texture.handle
        self.draw.tex_filter, self.draw.tex_edge = filter, edge
        self.keep.append(texture)
        return self

    def run(self, fs):
        self.draw.fs = shader_id(fs, A.SR_STAGE_FRAGMENT)
        # reuse what a duplicate rendered, when it was the pipeline's previous
        # draw (the library keeps the outputs of that draw only)
        last = self.pipeline._last_outputs
        reuse = A.SR_REUSE_NONE
        if self.geometry is not None and self.geometry.rendered and last == (self.vertices, self.geometry):
            reuse = A.SR_REUSE_GEOMETRY
        elif (self.vertices is not None and self.vertices.rendered and last is not None and last[0] is self.vertices
              and self.draw.gs_mode != A.SR_GS_NONE):
            reuse = A.SR_REUSE_VERTICES
        self.draw.reuse = reuse
        check(lib().sr_render(self.pipeline.handle, C.byref(self.draw)), "sr_render")
        for o in (self.vertices, self.geometry):
            if o is not None:
                o.rendered = True
        self.pipeline._last_outputs = (self.vertices, self.geometry)
        self.pipeline._keep.extend(self.keep)
        return self.pipeline


def prepare_scene(scene):
    """(pipeline, mesh, texture) for a softrender.scenes.Scene, framebuffer cleared."""
    fb = Framebuffer(scene.width, scene.height, scene.color_format, scene.depth, scene.stencil)
    pl = Pipeline.from_framebuffer(fb, scene.uniforms)
    pl.set_stencil(scene.stencil_test, scene.stencil_op, scene.stencil_wrap)
    if scene.color_format == A.SR_COLOR_RGBA8:
        pl.clear(list(scene.clear_bytes()))
    else:
        pl.clear(scene.clear_color)
    mesh = Mesh(scene.planes, scene.indices)
    tex = Texture(scene.texture) if scene.texture is not None else None
    return pl, mesh, tex


def submit_scene(pl, mesh, tex, scene):
    """Enqueues the draw of `scene` through the builder chain."""
    vp = Viewport(*scene.viewport)
    vs = pl.render_mesh(scene.prim, mesh, scene.stencil_ref if scene.stencil else None)
    if scene.gs_mode == A.SR_GS_NONE:
        fs = vs.run_to_fragment(vp, scene.vs)
    else:
        gs = vs.run(scene.vs)
        gs = gs.clip_primitives() if scene.gs_mode == A.SR_GS_CLIP else gs.run(scene.gs)
        fs = gs.finish(vp)
    fs = fs.with_blend(scene.blend).cull_faces(scene.cull).tile_size(*scene.tile)
    fs = fs.antialiased_lines(scene.aa_lines)
    if tex is not None:
        fs = fs.with_texture(tex, scene.tex_filter, scene.tex_edge)
    fs.run(scene.fs)


def render_scene(scene, initial=None):
    """Renders one Scene on the GPU; returns (color, depth, stencil, stats, status).
    `initial` optionally gives (color, depth, stencil) host planes to start from."""
    pl, mesh, tex = prepare_scene(scene)
    if initial is not None:
        pl.write(*initial)
    submit_scene(pl, mesh, tex, scene)
    status = pl.sync()
    color, depth, stencil = pl.read()
    stats = pl.stats()
    pl.destroy()
    mesh.free()
    if tex is not None:
        tex.free()
    return color, depth, stencil, stats, status


def draw_for_scene(scene, mesh, tex=None):
    """The sr_draw that submit_scene() hands to sr_render, built directly
    (for sr_batch_render, which takes the descriptors of many draws)."""
    d = A.SrDraw()
    lib().sr_draw_init(C.byref(d))
    d.mesh = mesh.handle.value if isinstance(mesh.handle, C.c_void_p) else mesh.handle
    d.prim = scene.prim
    d.vs = shader_id(scene.vs, A.SR_STAGE_VERTEX)
    d.gs_mode = scene.gs_mode
    if scene.gs_mode == A.SR_GS_CLIP:
        d.gs = shader_id("clip", A.SR_STAGE_GEOMETRY)
    elif scene.gs_mode == A.SR_GS_NAMED:
        d.gs = shader_id(scene.gs, A.SR_STAGE_GEOMETRY)
    d.viewport = A.SrViewport(*scene.viewport)
    d.cull = scene.cull
    d.fs = shader_id(scene.fs, A.SR_STAGE_FRAGMENT)
    d.blend = shader_id(scene.blend, A.SR_STAGE_BLEND)
    d.aa_lines = 1 if scene.aa_lines else 0
    d.tile_w, d.tile_h = scene.tile
    d.stencil_ref = scene.stencil_ref
    if tex is not None:
        d.texture = tex.handle.value if isinstance(tex.handle, C.c_void_p) else tex.handle
    d.tex_filter, d.tex_edge = scene.tex_filter, scene.tex_edge
    return d


class Batch:
    """Batched opaque draws (sr_batch_*): one launch per stage renders many
    pipelines' draws; the launch sequence is replayed as a CUDA graph and its
    launch configuration tuned per batch size class."""

    def __init__(self, use_graphs=True, autotune=True):
        h = C.c_void_p()
        check(lib().sr_batch_create(C.byref(h)), "sr_batch_create")
        self.handle = h
        self.set_options(use_graphs, autotune)
        self._keep = None

    def set_options(self, use_graphs=True, autotune=True):
        check(lib().sr_batch_set_options(self.handle, 1 if use_graphs else 0, 1 if autotune else 0),
              "sr_batch_set_options")

    def set_stream(self, stream_ptr):
        check(lib().sr_batch_set_stream(self.handle, C.c_void_p(stream_ptr) if stream_ptr else None),
              "sr_batch_set_stream")

    def set_config(self, bins_per_primitive=0, big_threshold=0, ctas_per_sm=0):
        check(lib().sr_batch_set_config(self.handle, bins_per_primitive, big_threshold, ctas_per_sm),
              "sr_batch_set_config")

    def config(self):
        v = [C.c_uint32() for _ in range(3)]
        check(lib().sr_batch_get_config(self.handle, *[C.byref(x) for x in v]), "sr_batch_get_config")
        return tuple(x.value for x in v)

    @staticmethod
    def items(entries):
        """entries: (pipeline, SrDraw, clear_bytes or None) -> ctypes array."""
        arr = (A.SrBatchItem * len(entries))()
        for i, (pl, d, clear) in enumerate(entries):
            pl._last_outputs = None   # a batched draw leaves nothing for duplicate() to reuse
            arr[i].target = pl.handle.value if isinstance(pl.handle, C.c_void_p) else pl.handle
            arr[i].draw = d
            arr[i].clear = 1 if clear is not None else 0
            if clear is not None:
                b = bytes(clear)
                for k in range(len(b)):
                    arr[i].clear_color[k] = b[k]
        return arr

    def render_items(self, arr):
        """Enqueues a prepared item array (returns the status)."""
        self._keep = arr
        return lib().sr_batch_render(self.handle, arr, len(arr))

    def render(self, entries):
        st = self.render_items(self.items(entries))
        check(st, "sr_batch_render")

    def sync(self):
        return lib().sr_batch_sync(self.handle)

    def stats(self):
        s = A.SrStats()
        check(lib().sr_batch_get_stats(self.handle, C.byref(s)), "sr_batch_get_stats")
        return {f: getattr(s, f) for f, _ in A.SrStats._fields_ if f != "stage_ms"}

    def destroy(self):
        if self.handle:
            lib().sr_batch_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.destroy()
        except Exception:
            pass


class Server:
    """Serving loop (sr_server_*): requests admitted against an HBM budget and
    continuously batched onto the GPU; `plain=True` serves one request at a
    time through sr_render (the per-request pipeline)."""

    def __init__(self, hbm_budget=0, max_inflight=0, max_batch=0, plain=False):
        cfg = A.SrServerConfig(hbm_budget, max_inflight, max_batch, 1 if plain else 0)
        h = C.c_void_p()
        check(lib().sr_server_create(C.byref(cfg), C.byref(h)), "sr_server_create")
        self.handle = h

    @staticmethod
    def request(draw, uniforms, width, height, color_format, clear_bytes):
        r = A.SrRequest()
        r.draw = draw
        r.uniforms = C.cast(C.pointer(uniforms), C.c_void_p)
        r.uniforms_size = C.sizeof(A.SrUniforms)
        r.width, r.height, r.color_format = width, height, color_format
        b = bytes(clear_bytes)
        for k in range(len(b)):
            r.clear_color[k] = b[k]
        r._keep = uniforms
        return r

    def submit(self, req):
        """Queues a prepared SrRequest; returns (status, ticket)."""
        t = C.c_uint64()
        st = lib().sr_server_submit(self.handle, C.byref(req), C.byref(t))
        return st, t.value

    def wait(self, ticket, timeout_ms=60000):
        return lib().sr_server_wait(self.handle, ticket, timeout_ms)

    def read(self, ticket, width, height, color_format):
        color = (np.empty((height, width, 4), dtype=np.float32) if color_format == A.SR_COLOR_RGBA32F
                 else np.empty((height, width), dtype=np.uint32))
        depth = np.empty((height, width), dtype=np.float32)
        check(lib().sr_server_read(self.handle, ticket, color.ctypes.data, depth.ctypes.data), "sr_server_read")
        return color, depth

    def release(self, ticket):
        return lib().sr_server_release(self.handle, ticket)

    def drain(self, timeout_ms=120000):
        return lib().sr_server_drain(self.handle, timeout_ms)

    def stats(self):
        s = A.SrServerStats()
        check(lib().sr_server_get_stats(self.handle, C.byref(s)), "sr_server_get_stats")
        return {f: getattr(s, f) for f, _ in A.SrServerStats._fields_}

    def reset_stats(self):
        check(lib().sr_server_reset_stats(self.handle), "sr_server_reset_stats")

    def destroy(self):
        if self.handle:
            lib().sr_server_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.destroy()
        except Exception:
            pass
