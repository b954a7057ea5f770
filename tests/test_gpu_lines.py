"""Lines, points and the named geometry shaders on the GPU versus the oracle.

rasterization/line.rs (Liang-Barsky per tile, Bresenham or Xiaolin Wu),
rasterization/point.rs, the line and point arms of clip_primitives, and the
normal-visualisation geometry shaders of full_example/src/shaders.rs:35-89.
Bit-exact colour, depth and stencil, and equal fragment counts."""
import pytest

from softrender import _abi as A
from softrender import scenes
from test_gpu_parity import check

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("aa", [False, True])
@pytest.mark.parametrize("fmt", [A.SR_COLOR_RGBA8, A.SR_COLOR_RGBA32F])
def test_lines_indexed(built_lib, oracle_mod, aa, fmt):
    check(scenes.lines_scene(aa_lines=aa, color_format=fmt), oracle_mod)


@pytest.mark.parametrize("blend", ["replace", "over"])
def test_lines_clipped_blend(built_lib, oracle_mod, blend):
    check(scenes.lines_scene(n=800, seed=3, gs_mode=A.SR_GS_CLIP, blend=blend, outside=0.6), oracle_mod)


def test_lines_tile_seams_and_stencil(built_lib, oracle_mod):
    sc = scenes.lines_scene(n=500, size=97, seed=8, tile=(7, 13), stencil=True,
                            stencil_test=A.SR_STENCIL_ALWAYS, stencil_op=A.SR_STENCIL_INCREMENT, stencil_wrap=1)
    check(sc, oracle_mod)


def test_lines_wu_over_stencil_gate(built_lib, oracle_mod):
    sc = scenes.lines_scene(n=400, size=120, seed=5, aa_lines=True, blend="over", stencil=True,
                            stencil_test=A.SR_STENCIL_LESS_THAN_EQ, stencil_op=A.SR_STENCIL_INCREMENT, stencil_ref=1)
    check(sc, oracle_mod)


@pytest.mark.parametrize("gs_mode", [A.SR_GS_NONE, A.SR_GS_CLIP])
def test_points(built_lib, oracle_mod, gs_mode):
    check(scenes.lines_scene(n=3000, seed=4, prim=A.SR_PRIM_POINT, gs_mode=gs_mode, tile=(16, 16)), oracle_mod)


@pytest.mark.parametrize("gs", ["vertex_normals", "face_normals"])
def test_normal_geometry_shaders(built_lib, oracle_mod, gs):
    sc = scenes.icosphere_scene(160, 120, subdiv=2, gs_mode=A.SR_GS_NAMED, gs=gs, fs="constant_color",
                                tile=(32, 32))
    check(sc, oracle_mod)


@pytest.mark.parametrize("filt", [A.SR_SAMPLE_NEAREST, A.SR_SAMPLE_BILINEAR])
@pytest.mark.parametrize("edge", [A.SR_SAMPLE_CLAMP, A.SR_SAMPLE_WRAP, A.SR_SAMPLE_BORDER])
def test_sampler_modes(built_lib, oracle_mod, filt, edge):
    sc = scenes.grid_sphere_scene(96, 64, n_lat=12, n_lon=24, tex_size=16, tex_filter=filt, tex_edge=edge,
                                  camera=dict(eye=(0.3, 0.2, 2.4), target=(0.0, 0.0, 0.0)))
    sc.planes[6] = (sc.planes[6] * 3.0 - 1.0).astype("float32")     # uv beyond [0, 1]
    sc.planes[7] = (sc.planes[7] * 3.0 - 1.0).astype("float32")
    check(sc, oracle_mod)


def test_render_to_texture(built_lib, oracle_mod):
    """A frame rendered into an RGBA8 framebuffer becomes the texture of the
    next draw (sr_texture_from_framebuffer)."""
    import numpy as np
    import softrender as sr
    from util import compare_frame
    first = scenes.icosphere_scene(64, 64, color_format=A.SR_COLOR_RGBA8)
    pl, mesh, _ = sr.prepare_scene(first)
    tex = sr.Texture(np.zeros((64, 64), np.uint32))
    try:
        sr.submit_scene(pl, mesh, None, first)
        assert pl.sync() == 0
        assert sr.lib().sr_texture_from_framebuffer(pl.handle, tex.handle) == 0
        assert pl.sync() == 0
        second = scenes.grid_sphere_scene(80, 60, n_lat=10, n_lon=20, tex_size=64, gs_mode=A.SR_GS_NONE,
                                          camera=dict(eye=(0.2, 0.1, 2.6), target=(0.0, 0.0, 0.0)))
        pl2, mesh2, _ = sr.prepare_scene(second)
        try:
            sr.submit_scene(pl2, mesh2, tex, second)
            assert pl2.sync() == 0
            got = pl2.read()
        finally:
            pl2.destroy()
            mesh2.free()
        # the oracle: render the first frame, use its colour as the texture
        fb1, _, _ = oracle_mod.render(first)
        second.texture = fb1.color.view(np.uint32).reshape(64, 64).copy()
        fb2, _, _ = oracle_mod.render(second)
        compare_frame(got, fb2)
    finally:
        pl.destroy()
        mesh.free()
        tex.free()


@pytest.mark.parametrize("tile", [(1, 1), (2, 2), (1, 3), (2, 5)])
def test_wu_lines_tiny_tiles(built_lib, oracle_mod, tile):
    """Xiaolin Wu lines plot one pixel beyond their semantic tile; with tiles
    1 or 2 pixels wide such pixels belong to tiles two columns away, which the
    raster schedule keeps in later phases (over-blend and stencil counting
    make the order visible)."""
    sc = scenes.lines_scene(n=150, size=40, seed=31, aa_lines=True, blend="over", tile=tile, stencil=True,
                            stencil_test=A.SR_STENCIL_ALWAYS, stencil_op=A.SR_STENCIL_INCREMENT)
    check(sc, oracle_mod)
