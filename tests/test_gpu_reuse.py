"""duplicate(): rendering again from the outputs of earlier stages.

GeometryShader::duplicate (src/pipeline/stages/geometry.rs:40-54) keeps the
processed vertices for a second geometry shader (full_example/src/main.rs:
69-92 renders a mesh, then its face normals from the same vertices);
FragmentShader::duplicate (fragment.rs:118-135) rasterises the same geometry
again with other settings.  sr_draw.reuse selects either; the results must
equal the two draws rendered from scratch by the oracle, and a draw that must
recompute the reused stages (an overflow replay) must equal one that skips
them."""
import copy
import ctypes as C

import numpy as np
import pytest

from softrender import _abi as A
from softrender import scenes
from util import compare_frame

pytestmark = pytest.mark.gpu


def _two_draws(first, second, reuse, warm=False, uniforms2=None):
    """`first` through the builder chain, then `second` with sr_draw.reuse on
    the same pipeline; returns ((color, depth, stencil), stats of the second
    draw).  `warm` renders `first` once beforehand so that no buffer grows
    (the reused stages are then skipped rather than recomputed)."""
    import softrender as sr
    pl, mesh, tex = sr.prepare_scene(first)
    try:
        if warm:
            sr.submit_scene(pl, mesh, tex, first)
            assert pl.sync() == 0
            # colour, depth and stencil back to the cleared state
            pl.clear(list(first.clear_bytes()) if first.color_format == A.SR_COLOR_RGBA8 else first.clear_color)
        sr.submit_scene(pl, mesh, tex, first)
        if uniforms2 is not None:
            pl.set_uniforms(uniforms2)
        d = sr.draw_for_scene(second, mesh, tex)
        d.reuse = reuse
        assert sr.lib().sr_render(pl.handle, C.byref(d)) == A.SR_OK
        assert pl.sync() == A.SR_OK
        return pl.read(), pl.stats()
    finally:
        pl.destroy()
        mesh.free()
        if tex is not None:
            tex.free()


def _oracle_two(oracle_mod, first, second):
    fb = oracle_mod.framebuffer_for(first)
    oracle_mod.render(first, fb)
    oracle_mod.render(second, fb)
    return fb


def _variant(sc, **kw):
    s2 = copy.copy(sc)
    for k, v in kw.items():
        setattr(s2, k, v)
    return s2


@pytest.mark.parametrize("gs", ["face_normals", "vertex_normals"])
def test_duplicate_geometry_shader(built_lib, oracle_mod, gs):
    """The mesh through the clip shader, then its normals from the same vertices."""
    first = scenes.icosphere_scene(160, 120, subdiv=2, gs_mode=A.SR_GS_CLIP, tile=(32, 32))
    second = _variant(first, gs_mode=A.SR_GS_NAMED, gs=gs, fs="constant_color", blend="over")
    got, st = _two_draws(first, second, A.SR_REUSE_VERTICES, warm=True)
    compare_frame(got, _oracle_two(oracle_mod, first, second))
    _, full = _two_draws(first, second, A.SR_REUSE_NONE, warm=True)
    assert st["kernel_launches"] < full["kernel_launches"]


@pytest.mark.parametrize("gs_mode", [A.SR_GS_NONE, A.SR_GS_CLIP])
@pytest.mark.parametrize("warm", [True, False])
def test_duplicate_fragment_shader(built_lib, oracle_mod, gs_mode, warm):
    """The same geometry rasterised again with culling, other tiles, another
    fragment shader and the over blend."""
    first = scenes.icosphere_scene(200, 150, subdiv=3, gs_mode=gs_mode, color_format=A.SR_COLOR_RGBA8)
    second = _variant(first, cull=A.SR_CULL_CLOCKWISE, tile=(16, 24), fs="constant_color", blend="over")
    got, st = _two_draws(first, second, A.SR_REUSE_GEOMETRY, warm=warm)
    compare_frame(got, _oracle_two(oracle_mod, first, second))
    if gs_mode == A.SR_GS_CLIP:
        assert st["triangles_generated"] > 0


def test_duplicate_lines(built_lib, oracle_mod):
    first = scenes.lines_scene(n=500, seed=9)
    second = _variant(first, aa_lines=True, blend="over", tile=(24, 40))
    got, _ = _two_draws(first, second, A.SR_REUSE_GEOMETRY, warm=True)
    compare_frame(got, _oracle_two(oracle_mod, first, second))


def test_reuse_keeps_earlier_uniforms(built_lib, oracle_mod):
    """Uniforms changed between the draws: the reused geometry is that of the
    first draw's uniforms, the fragment stage uses the new ones.  The pipeline
    with stencil counting overflows its clip-output buffers on the first use,
    so sync replays both draws and recomputes the reused stages from the saved
    uniforms; a warm pipeline skips them.  Both must agree, and differ from a
    draw that recomputes everything with the new uniforms."""
    first = scenes.icosphere_scene(160, 120, subdiv=3, gs_mode=A.SR_GS_CLIP, stencil=True,
                                   stencil_test=A.SR_STENCIL_ALWAYS, stencil_op=A.SR_STENCIL_INCREMENT)
    second = _variant(first, fs="constant_color", blend="over", tile=(20, 20))
    eye = (0.4, 2.6, 1.1)
    u2_view = scenes.look_at_rh(eye, (0, 0, 0), (0, 1, 0))
    u2 = scenes.make_uniforms(view=u2_view, projection=scenes.perspective(160 / 120, np.radians(60.0), 0.1, 100.0),
                              camera=eye)
    warm, _ = _two_draws(first, second, A.SR_REUSE_GEOMETRY, warm=True, uniforms2=u2)
    cold, _ = _two_draws(first, second, A.SR_REUSE_GEOMETRY, warm=False, uniforms2=u2)
    for a, b in zip(warm, cold):
        assert np.array_equal(np.asarray(a).view(np.uint8), np.asarray(b).view(np.uint8))
    recomputed, _ = _two_draws(first, second, A.SR_REUSE_NONE, warm=True, uniforms2=u2)
    assert not np.array_equal(np.asarray(warm[0]).view(np.uint8), np.asarray(recomputed[0]).view(np.uint8))
    # with unchanged uniforms the reuse equals the oracle's two full draws
    same, _ = _two_draws(first, second, A.SR_REUSE_GEOMETRY, warm=False)
    compare_frame(same, _oracle_two(oracle_mod, first, second))


def test_builder_chain_duplicate(built_lib, oracle_mod):
    """The full_example sequence through the Python mirror of the chain:
    geometry_shader.duplicate().finish(..).run(fs), then
    geometry_shader.replace(gs).finish(..).run(fs2)."""
    import softrender as sr
    first = scenes.icosphere_scene(128, 96, subdiv=2, gs_mode=A.SR_GS_CLIP)
    second = _variant(first, gs_mode=A.SR_GS_NAMED, gs="face_normals", fs="constant_color")
    pl, mesh, _ = sr.prepare_scene(first)
    try:
        vp = sr.Viewport(*first.viewport)
        gs = pl.render_mesh(A.SR_PRIM_TRIANGLE, mesh).run(first.vs)
        gs.duplicate().clip_primitives().finish(vp).tile_size(*first.tile).run(first.fs)
        gs.replace("face_normals").finish(vp).tile_size(*first.tile).run("constant_color")
        assert pl.sync() == 0
        st = pl.stats()
        got = pl.read()
    finally:
        pl.destroy()
        mesh.free()
    compare_frame(got, _oracle_two(oracle_mod, first, second))
    # the normals were drawn without their own vertex stage
    alone = sr.render_scene(second)[3]
    assert st["kernel_launches"] == alone["kernel_launches"] - 1


def test_reuse_rejected(built_lib):
    import softrender as sr
    sc = scenes.icosphere_scene(64, 64, subdiv=1, gs_mode=A.SR_GS_CLIP)
    pl, mesh, _ = sr.prepare_scene(sc)
    other = sr.Mesh(sc.planes, sc.indices)
    L = sr.lib()

    def render(**kw):
        d = sr.draw_for_scene(_variant(sc, **{k: v for k, v in kw.items() if k not in ("reuse", "mesh")}),
                              kw.get("mesh", mesh))
        d.reuse = kw.get("reuse", A.SR_REUSE_NONE)
        return L.sr_render(pl.handle, C.byref(d))

    try:
        assert render(reuse=A.SR_REUSE_GEOMETRY) == A.SR_EINVAL           # nothing rendered yet
        assert render() == A.SR_OK
        assert render(reuse=A.SR_REUSE_GEOMETRY, mesh=other) == A.SR_EINVAL
        assert render(reuse=A.SR_REUSE_GEOMETRY, gs_mode=A.SR_GS_NAMED, gs="face_normals") == A.SR_EINVAL
        assert render(reuse=A.SR_REUSE_VERTICES, gs_mode=A.SR_GS_NONE) == A.SR_EINVAL
        assert render(reuse=A.SR_REUSE_GEOMETRY, viewport=(0.0, 0.0, 32.0, 32.0, 0.0, 1.0)) == A.SR_EINVAL
        assert render(reuse=3) == A.SR_EINVAL
        assert render(reuse=A.SR_REUSE_GEOMETRY, fs="constant_color") == A.SR_OK
        mesh.update(sc.planes, sc.indices)
        assert render(reuse=A.SR_REUSE_GEOMETRY) == A.SR_EINVAL            # the mesh changed since
        assert pl.sync() == 0
        # the batched path has no previous draw to refer to
        b = sr.Batch(use_graphs=False, autotune=False)
        try:
            d = sr.draw_for_scene(_variant(sc, gs_mode=A.SR_GS_NONE), mesh)
            d.reuse = A.SR_REUSE_GEOMETRY
            assert b.render_items(b.items([(pl, d, None)])) == A.SR_EINVAL
        finally:
            b.destroy()
    finally:
        pl.destroy()
        mesh.free()
        other.free()
