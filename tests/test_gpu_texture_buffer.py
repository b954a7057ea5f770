"""Texture-buffer framebuffers: a framebuffer's colour attachment read as a
texture in place (src/framebuffer/texturebuffer.rs:13-48, 111-117), RGBA8 or
RGBA f32 (the predefined RGBAf32TextureBuffer, texturebuffer.rs:199-210), and
uploaded RGBA f32 textures, sampled with every filter and edge mode.  Each
result is compared bit for bit with the oracle rendering the same two passes
(the first pass's colour plane handed to the second as its texture)."""
import ctypes as C

import numpy as np
import pytest

from softrender import _abi as A
from softrender import scenes
from util import compare_frame

pytestmark = pytest.mark.gpu


def _second(color_format, filt, edge):
    sc = scenes.grid_sphere_scene(96, 72, n_lat=12, n_lon=24, tex_size=16, tex_filter=filt, tex_edge=edge,
                                  gs_mode=A.SR_GS_NONE, color_format=color_format,
                                  camera=dict(eye=(0.3, 0.2, 2.4), target=(0.0, 0.0, 0.0)))
    sc.planes[6] = (sc.planes[6] * 3.0 - 1.0).astype(np.float32)     # uv beyond [0, 1]
    sc.planes[7] = (sc.planes[7] * 3.0 - 1.0).astype(np.float32)
    return sc


def _render_with(second, tex):
    import softrender as sr
    pl, mesh, own = sr.prepare_scene(second)
    try:
        sr.submit_scene(pl, mesh, tex, second)
        assert pl.sync() == 0
        return pl.read()
    finally:
        pl.destroy()
        mesh.free()
        if own is not None:
            own.free()


@pytest.mark.parametrize("first_fmt", [A.SR_COLOR_RGBA32F, A.SR_COLOR_RGBA8])
@pytest.mark.parametrize("filt,edge", [(A.SR_SAMPLE_BILINEAR, A.SR_SAMPLE_CLAMP),
                                       (A.SR_SAMPLE_BILINEAR, A.SR_SAMPLE_WRAP),
                                       (A.SR_SAMPLE_NEAREST, A.SR_SAMPLE_BORDER)])
def test_colour_attachment_as_texture(built_lib, oracle_mod, first_fmt, filt, edge):
    import softrender as sr
    first = scenes.icosphere_scene(64, 48, color_format=first_fmt)
    second = _second(A.SR_COLOR_RGBA8, filt, edge)
    pl, mesh, _ = sr.prepare_scene(first)
    try:
        sr.submit_scene(pl, mesh, None, first)
        assert pl.sync() == 0
        view = sr.Texture.view(pl)
        got = _render_with(second, view)
        if first_fmt == A.SR_COLOR_RGBA8:
            # the zero-copy view and a copy (render to texture) agree
            copy = sr.Texture(np.zeros((48, 64), np.uint32))
            assert sr.lib().sr_texture_from_framebuffer(pl.handle, copy.handle) == 0
            assert pl.sync() == 0
            again = _render_with(second, copy)
            copy.free()
            for a, b in zip(got, again):
                if a is not None:
                    assert np.array_equal(np.asarray(a).view(np.uint8), np.asarray(b).view(np.uint8))
        view.free()
    finally:
        pl.destroy()
        mesh.free()
    fb1, _, _ = oracle_mod.render(first)
    if first_fmt == A.SR_COLOR_RGBA32F:
        second.texture = fb1.color.reshape(48, 64, 4).copy()
    else:
        second.texture = fb1.color.view(np.uint32).reshape(48, 64).copy()
    fb2, _, _ = oracle_mod.render(second)
    compare_frame(got, fb2)


@pytest.mark.parametrize("out_fmt", [A.SR_COLOR_RGBA8, A.SR_COLOR_RGBA32F])
@pytest.mark.parametrize("filt,edge", [(A.SR_SAMPLE_BILINEAR, A.SR_SAMPLE_CLAMP),
                                       (A.SR_SAMPLE_NEAREST, A.SR_SAMPLE_WRAP),
                                       (A.SR_SAMPLE_BILINEAR, A.SR_SAMPLE_BORDER)])
def test_rgba32f_texture(built_lib, oracle_mod, out_fmt, filt, edge):
    """Uploaded RGBA f32 texels, including values outside [0, 1]."""
    import softrender as sr
    rng = np.random.default_rng(21)
    texels = rng.uniform(-0.2, 1.5, (20, 28, 4)).astype(np.float32)
    second = _second(out_fmt, filt, edge)
    tex = sr.Texture(texels)
    try:
        got = _render_with(second, tex)
    finally:
        tex.free()
    second.texture = texels
    fb, _, _ = oracle_mod.render(second)
    compare_frame(got, fb)


def test_texture_views_rejected(built_lib):
    import softrender as sr
    first = scenes.icosphere_scene(32, 32, subdiv=1, color_format=A.SR_COLOR_RGBA8)
    pl, mesh, _ = sr.prepare_scene(first)
    view = sr.Texture.view(pl)
    L = sr.lib()
    try:
        # a draw may not sample the plane it writes
        sc = scenes.grid_sphere_scene(32, 32, n_lat=4, n_lon=8, tex_size=8, gs_mode=A.SR_GS_NONE,
                                      color_format=A.SR_COLOR_RGBA8)
        m2 = sr.Mesh(sc.planes, sc.indices)
        d = sr.draw_for_scene(sc, m2, view)
        assert L.sr_render(pl.handle, C.byref(d)) == A.SR_EINVAL
        # nor may a batch or a server request sample a view
        b = sr.Batch(use_graphs=False, autotune=False)
        pl2 = sr.Pipeline.from_framebuffer(sr.Framebuffer(32, 32, A.SR_COLOR_RGBA8, True, False), sc.uniforms)
        assert b.render_items(b.items([(pl2, d, None)])) == A.SR_EINVAL
        b.destroy()
        pl2.destroy()
        # views cannot be updated from the host nor be a copy target
        data = np.zeros((32, 32), np.uint32)
        assert L.sr_texture_update(view.handle, data.ctypes.data, 32, 32, None) == A.SR_EINVAL
        assert L.sr_texture_from_framebuffer(pl.handle, view.handle) == A.SR_EINVAL
        # no colour attachment, no view
        pl3 = sr.Pipeline.from_framebuffer(sr.Framebuffer(16, 16, A.SR_COLOR_NONE, True, False), sc.uniforms)
        h = C.c_void_p()
        assert L.sr_texture_view_framebuffer(pl3.handle, C.byref(h)) == A.SR_EINVAL
        pl3.destroy()
        m2.free()
    finally:
        view.free()
        pl.destroy()
        mesh.free()


def test_unknown_sampler_modes_rejected(built_lib):
    """sr_filter has two values and sr_edge three; any other value is refused
    by sr_render, sr_batch_render and sr_render_static alike."""
    import softrender as sr
    sc = scenes.grid_sphere_scene(32, 32, n_lat=4, n_lon=8, tex_size=8, gs_mode=A.SR_GS_NONE,
                                  color_format=A.SR_COLOR_RGBA8)
    pl, mesh, tex = sr.prepare_scene(sc)
    L = sr.lib()
    b = sr.Batch(use_graphs=False, autotune=False)
    try:
        for field, bad in (("tex_filter", A.SR_SAMPLE_BILINEAR + 1), ("tex_edge", A.SR_SAMPLE_BORDER + 1)):
            d = sr.draw_for_scene(sc, mesh, tex)
            setattr(d, field, bad)
            assert L.sr_render(pl.handle, C.byref(d)) == A.SR_EINVAL
            assert b.render_items(b.items([(pl, d, None)])) == A.SR_EINVAL
            ds = A.SrDraw()
            L.sr_draw_init(C.byref(ds))
            setattr(ds, field, bad)
            fb = A.SrFbDesc(32, 32, A.SR_COLOR_RGBA8, 1, 0)
            # refused while checking the draw, before any buffer is looked at
            assert L.sr_render_static(C.byref(ds), C.byref(sc.uniforms), C.sizeof(sc.uniforms), None, 0, 0, 0,
                                      None, 0, None, 0, 0, C.byref(fb), None, None, None) == A.SR_EINVAL
        d = sr.draw_for_scene(sc, mesh, tex)
        assert L.sr_render(pl.handle, C.byref(d)) == A.SR_OK
        assert pl.sync() == A.SR_OK
    finally:
        b.destroy()
        pl.destroy()
        mesh.free()
        if tex is not None:
            tex.free()


def test_view_outlives_its_pipeline(built_lib, oracle_mod):
    """A view holds a reference on the colour plane: the pipeline that drew it
    can be destroyed first, and the view still samples its last frame (the
    plane is freed with the view's last reference)."""
    import softrender as sr
    first = scenes.icosphere_scene(64, 48, color_format=A.SR_COLOR_RGBA8)
    second = _second(A.SR_COLOR_RGBA8, A.SR_SAMPLE_BILINEAR, A.SR_SAMPLE_CLAMP)
    pl, mesh, _ = sr.prepare_scene(first)
    sr.submit_scene(pl, mesh, None, first)
    assert pl.sync() == 0
    view = sr.Texture.view(pl)
    pl.destroy()
    mesh.free()
    got = _render_with(second, view)
    view.free()
    fb1, _, _ = oracle_mod.render(first)
    second.texture = fb1.color.view(np.uint32).reshape(48, 64).copy()
    fb2, _, _ = oracle_mod.render(second)
    compare_frame(got, fb2)
