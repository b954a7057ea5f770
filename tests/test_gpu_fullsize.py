"""Parity at the full benchmark sizes.

The GPU renders the whole frame of the 1,048,576-triangle grid-sphere at
3840x2160 (clip geometry shader, textured Blinn-Phong, RGBA8) and of the
16,777,216-triangle ordering stress frame at 2048x2048 (over-blend, stencil
counting).  The single-threaded oracle (the reference's own order; its
threaded mode reorders like the reference's pool) renders a run of
consecutive semantic tiles of the same frame (fragment.rs:188-216 visits
every primitive in every tile), and every pixel strictly inside that run --
touched by no other tile -- must match bit for bit.  The geometry stage runs
in full on both sides."""
import numpy as np
import pytest

from softrender import _abi as A
from softrender import scenes
from util import assert_bitexact

pytestmark = pytest.mark.gpu


def _window_check(sc, oracle_mod, row, col0, ncols):
    import softrender as sr
    color, depth, stencil, stats, status = sr.render_scene(sc)
    assert status == 0
    tiles = oracle_mod.tiles(sc.width, sc.height, *sc.tile)
    per_row = sum(1 for t in tiles if t[1] == 0)
    first = row * per_row + col0
    fb, ost, ostatus = oracle_mod.render(sc, n_threads=1, tile_begin=first, tile_end=first + ncols)
    assert ostatus == 0
    x0, y0 = tiles[first][0], tiles[first][1]
    x1, y1 = tiles[first + ncols - 1][2], tiles[first + ncols - 1][3]
    ys, xs = slice(y0 + 1, y1), slice(x0 + 1, x1)     # shared edges excluded
    h, w = sc.height, sc.width
    if sc.color_format == A.SR_COLOR_RGBA8:
        want_c = fb.color.view(np.uint32).reshape(h, w)
        assert_bitexact("color", color[ys, xs], want_c[ys, xs])
    else:
        assert_bitexact("color", color[ys, xs], fb.color.reshape(h, w, 4)[ys, xs])
    assert_bitexact("depth", depth[ys, xs], fb.depth.reshape(h, w)[ys, xs])
    if sc.stencil:
        assert_bitexact("stencil", stencil[ys, xs], fb.stencil.reshape(h, w)[ys, xs])
    # the window is not trivially empty
    assert (depth[ys, xs] > np.float32(-3.0e38)).mean() > 0.2
    return stats, ost


def test_gridsphere_full_size(built_lib, oracle_mod):
    """1,048,576 triangles, 3840x2160: the whole tile row through the middle."""
    sc = scenes.grid_sphere_scene()
    stats, ost = _window_check(sc, oracle_mod, row=8, col0=0, ncols=30)
    assert stats["triangles_generated"] == ost["triangles_generated"]


def test_stress_full_size(built_lib, oracle_mod):
    """16,777,216 tiny + 4,096 alpha triangles, 2048x2048, stencil counting:
    8 tiles of the middle tile row."""
    sc = scenes.stress_scene()
    _window_check(sc, oracle_mod, row=8, col0=4, ncols=8)
