"""sr_render_static: the draw entry point that allocates no device memory.

Some callers cannot let this library allocate: an application whose own
allocator owns all of the GPU's memory, a real-time loop that cannot pay for
cudaMalloc/cudaFree (and the synchronisation they bring) inside a frame, or a
plugin that only receives device pointers.  sr_render_static serves them with
a fixed scratch array inside the library.  These tests call it through the C
ABI on buffers the test owns and check it against sr_render, the pipeline
entry point, for the same draws: bit-exact colour and depth, on two calls in
a row (the second drawing over the first one's output, so the scratch left
behind by the first call must not leak into the second).

The file is named so that pytest collects it last.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

F32_MIN = np.float32(-3.40282347e38)


def _torch():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA GPU")
    return torch


def _scenes(fmt, w, h):
    from softrender import _abi as A
    from softrender import scenes
    a = scenes.icosphere_scene(w, h, color_format=fmt)
    b = scenes.grid_sphere_scene(w, h, n_lat=48, n_lon=96, tex_size=256, gs_mode=A.SR_GS_NONE,
                                 color_format=fmt, camera=dict(eye=(0.4, 0.3, 2.2), target=(0.0, 0.0, 0.0)))
    b.clear_color = a.clear_color
    return a, b


def _draw(sc):
    import softrender as sr
    from softrender import _abi as A
    d = A.SrDraw()
    sr.lib().sr_draw_init(C.byref(d))
    d.prim = A.SR_PRIM_TRIANGLE
    d.vs = sr.shader_id(sc.vs, A.SR_STAGE_VERTEX)
    d.fs = sr.shader_id(sc.fs, A.SR_STAGE_FRAGMENT)
    d.blend = sr.shader_id(sc.blend, A.SR_STAGE_BLEND)
    d.gs_mode = A.SR_GS_NONE
    d.viewport = A.SrViewport(*sc.viewport)
    d.cull = sc.cull
    d.tile_w, d.tile_h = sc.tile
    d.tex_filter, d.tex_edge = sc.tex_filter, sc.tex_edge
    return d


class DeviceMesh:
    """The test's own device copies of a scene's planes, indices and texture."""

    def __init__(self, torch, sc):
        n = sc.n_verts
        self.stride = (n + 3) & ~3
        host = np.zeros((len(sc.planes), self.stride), dtype=np.float32)
        for j, p in enumerate(sc.planes):
            host[j, :n] = p
        self.planes = torch.from_numpy(host).cuda()
        self.indices = torch.from_numpy(np.ascontiguousarray(sc.indices, dtype=np.uint32).view(np.int32)).cuda()
        self.tex = None
        if sc.texture is not None:
            self.tex = torch.from_numpy(np.ascontiguousarray(sc.texture, dtype=np.uint32).view(np.int32)).cuda()
        self.n_planes, self.n_verts, self.n_tris = len(sc.planes), n, sc.n_tris
        self.tex_w = 0 if sc.texture is None else sc.texture.shape[1]
        self.tex_h = 0 if sc.texture is None else sc.texture.shape[0]


def _fb_buffers(torch, sc):
    from softrender import _abi as A
    if sc.color_format == A.SR_COLOR_RGBA8:
        color = torch.from_numpy(np.frombuffer(sc.clear_bytes(), dtype=np.uint8).copy()).cuda()
        color = color.repeat(sc.height * sc.width).view(sc.height, sc.width, 4).contiguous()
    else:
        color = torch.tensor(sc.clear_color, dtype=torch.float32, device="cuda")
        color = color.repeat(sc.height * sc.width).view(sc.height, sc.width, 4).contiguous()
    depth = torch.full((sc.height, sc.width), float(F32_MIN), dtype=torch.float32, device="cuda")
    return color, depth


def _render_static(torch, sc, mesh, color, depth, stream=None):
    import softrender as sr
    from softrender import _abi as A
    fb = A.SrFbDesc(sc.width, sc.height, sc.color_format, 1, 0)
    u = sc.uniforms
    return sr.lib().sr_render_static(
        C.byref(_draw(sc)), C.byref(u), C.sizeof(u),
        mesh.planes.data_ptr(), mesh.n_planes, mesh.stride, mesh.n_verts,
        mesh.indices.data_ptr(), mesh.n_tris,
        mesh.tex.data_ptr() if mesh.tex is not None else None, mesh.tex_w, mesh.tex_h,
        C.byref(fb), color.data_ptr(), depth.data_ptr(), stream)


def _pipeline_frames(first, second):
    """sr_render of `first` alone, then of `first` followed by `second`."""
    import softrender as sr
    out = []
    for draws in ([first], [first, second]):
        pl, mesh, tex = sr.prepare_scene(first)
        keep = []
        for sc in draws:
            if sc is first:
                m, t = mesh, tex
            else:
                m = sr.Mesh(sc.planes, sc.indices)
                t = sr.Texture(sc.texture) if sc.texture is not None else None
            keep += [m, t]
            pl.set_uniforms(sc.uniforms)
            sr.submit_scene(pl, m, t, sc)
        assert pl.sync() == 0
        color, depth, _ = pl.read()
        out.append((color.view(np.uint8).copy(), depth.copy()))
        pl.destroy()
        for k in keep:
            if k is not None:
                k.free()
    return out


def _host(color, depth):
    return color.cpu().numpy().view(np.uint8).reshape(-1), depth.cpu().numpy().copy()


@pytest.mark.parametrize("fmt_name", ["RGBA8", "RGBA32F"])
def test_two_calls_match_sr_render(built_lib, fmt_name):
    torch = _torch()
    from softrender import _abi as A
    fmt = getattr(A, "SR_COLOR_" + fmt_name)
    a, b = _scenes(fmt, 640, 480)
    want_a, want_ab = _pipeline_frames(a, b)

    color, depth = _fb_buffers(torch, a)
    ma, mb = DeviceMesh(torch, a), DeviceMesh(torch, b)
    stream = torch.cuda.current_stream().cuda_stream
    # first call: scene a over the cleared buffers
    assert _render_static(torch, a, ma, color, depth, stream) == A.SR_OK
    torch.cuda.synchronize()
    got_c, got_d = _host(color, depth)
    assert np.array_equal(got_c, want_a[0].reshape(-1)), "colour differs from sr_render (first call)"
    assert np.array_equal(got_d.view(np.uint32), want_a[1].view(np.uint32)), "depth differs (first call)"
    # second call: scene b drawn over the first call's output
    assert _render_static(torch, b, mb, color, depth, stream) == A.SR_OK
    torch.cuda.synchronize()
    got_c, got_d = _host(color, depth)
    assert np.array_equal(got_c, want_ab[0].reshape(-1)), "colour differs from sr_render (second call)"
    assert np.array_equal(got_d.view(np.uint32), want_ab[1].view(np.uint32)), "depth differs (second call)"


def test_same_draw_twice_is_identical(built_lib):
    """The scratch keeps the previous call's contents; a repeat of the same
    draw on freshly cleared buffers must give the same frame."""
    torch = _torch()
    from softrender import _abi as A
    a, _ = _scenes(A.SR_COLOR_RGBA8, 333, 211)
    m = DeviceMesh(torch, a)
    frames = []
    for _ in range(2):
        color, depth = _fb_buffers(torch, a)
        assert _render_static(torch, a, m, color, depth) == A.SR_OK
        torch.cuda.synchronize()
        frames.append(_host(color, depth))
    assert np.array_equal(frames[0][0], frames[1][0])
    assert np.array_equal(frames[0][1].view(np.uint32), frames[1][1].view(np.uint32))
    want, _ = _pipeline_frames(a, a)
    assert np.array_equal(frames[1][0], want[0].reshape(-1))


def test_rejects_sizes_beyond_the_scratch(built_lib):
    torch = _torch()
    import softrender as sr
    from softrender import _abi as A
    a, _ = _scenes(A.SR_COLOR_RGBA8, 64, 64)
    m = DeviceMesh(torch, a)
    color, depth = _fb_buffers(torch, a)
    before = _host(color, depth)
    u = a.uniforms
    L = sr.lib()

    def call(w, h, n_tris, n_verts):
        fb = A.SrFbDesc(w, h, A.SR_COLOR_RGBA8, 1, 0)
        return L.sr_render_static(C.byref(_draw(a)), C.byref(u), C.sizeof(u), m.planes.data_ptr(), m.n_planes,
                                  max(m.stride, (n_verts + 3) & ~3), n_verts, m.indices.data_ptr(), n_tris,
                                  None, 0, 0, C.byref(fb), color.data_ptr(), depth.data_ptr(), None)

    assert call(1025, 1024, m.n_tris, m.n_verts) == A.SR_EOVERFLOW          # pixels
    assert call(64, 64, A.SR_STATIC_MAX_TRIANGLES + 1, m.n_verts) == A.SR_EOVERFLOW
    assert call(64, 64, m.n_tris, A.SR_STATIC_MAX_VERTICES + 1) == A.SR_EOVERFLOW
    torch.cuda.synchronize()
    after = _host(color, depth)
    assert np.array_equal(before[0], after[0]) and np.array_equal(before[1], after[1])
