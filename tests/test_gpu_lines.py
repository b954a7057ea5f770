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
