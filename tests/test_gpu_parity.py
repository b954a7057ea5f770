"""GPU (through the C ABI) versus the CPU oracle on seeded inputs.

Coverage, depth, stencil and RGBA8 colour must match bit for bit; RGBA f32
colour too (tolerance 0 ULP: the shader arithmetic is the same FP32
operation sequence on both sides, compiled without FMA contraction).
"""
import numpy as np
import pytest

import softrender as sr
from softrender import _abi as A
from softrender import scenes
from util import compare_frame

pytestmark = pytest.mark.gpu

COLOR_ULPS = 0


def run_both(scene, oracle_mod, initial=None):
    gpu = sr.render_scene(scene, initial=initial)
    fb = oracle_mod.framebuffer_for(scene)
    if initial is not None:
        c, d, s = initial
        if c is not None:
            fb.color[...] = c
        if d is not None:
            fb.depth[...] = d
        if s is not None:
            fb.stencil[...] = s
    fb, ostats, ostatus = oracle_mod.render(scene, fb)
    return gpu, fb, ostats, ostatus


def check(scene, oracle_mod, initial=None):
    (color, depth, stencil, stats, status), fb, ostats, ostatus = run_both(scene, oracle_mod, initial)
    compare_frame((color, depth, stencil), fb, COLOR_ULPS)
    assert stats["fragments"] == ostats["fragments"], (stats, ostats)
    assert (status == A.SR_ENAN) == (ostatus == 7)
    return stats, ostats


def test_icosphere_small(built_lib, oracle_mod):
    check(scenes.icosphere_scene(256, 256), oracle_mod)


def test_icosphere_1024(built_lib, oracle_mod):
    check(scenes.icosphere_scene(1024, 1024), oracle_mod)


def test_icosphere_rgba8_nonsquare(built_lib, oracle_mod):
    sc = scenes.icosphere_scene(300, 170, color_format=A.SR_COLOR_RGBA8)
    check(sc, oracle_mod)


@pytest.mark.parametrize("tile", [(128, 128), (16, 16), (7, 13), (1, 1), (1000, 3)])
def test_tile_sizes(built_lib, oracle_mod, tile):
    sc = scenes.icosphere_scene(160, 120, tile=tile)
    check(sc, oracle_mod)


@pytest.mark.parametrize("cull", [A.SR_CULL_CLOCKWISE, A.SR_CULL_COUNTER_CLOCKWISE])
def test_culling(built_lib, oracle_mod, cull):
    check(scenes.icosphere_scene(200, 200, cull=cull), oracle_mod)


def test_clip_gs_icosphere(built_lib, oracle_mod):
    sc = scenes.icosphere_scene(256, 256, gs_mode=A.SR_GS_CLIP)
    check(sc, oracle_mod)


def test_grid_sphere_clip_textured(built_lib, oracle_mod):
    sc = scenes.grid_sphere_scene(width=384, height=216, n_lat=32, n_lon=64, tex_size=64)
    stats, _ = check(sc, oracle_mod)
    assert stats["triangles_generated"] > 0


# ----------------------------------------------------------- ordered paths
@pytest.mark.parametrize("wrap", [1, 0])
def test_stress_blend_stencil_increment(built_lib, oracle_mod, wrap):
    """Tiny triangles + large alpha triangles, over-blend in submission order,
    stencil Always/Increment (wrap and saturate) with 32x24 semantic tiles."""
    sc = scenes.stress_scene(n_tiny=3000, n_large=24, size=160, wrap=wrap, tile=(32, 24))
    check(sc, oracle_mod)


def test_stress_saturates(built_lib, oracle_mod):
    """Enough events on tile edges to saturate / wrap the u8 stencil."""
    sc = scenes.stress_scene(n_tiny=2000, n_large=300, size=96, wrap=0, tile=(8, 8))
    check(sc, oracle_mod)


@pytest.mark.parametrize("test_op", [(A.SR_STENCIL_LESS_THAN, A.SR_STENCIL_KEEP),
                                     (A.SR_STENCIL_EQUAL, A.SR_STENCIL_KEEP),
                                     (A.SR_STENCIL_NEVER, A.SR_STENCIL_INCREMENT),
                                     (A.SR_STENCIL_ALWAYS, A.SR_STENCIL_REPLACE),
                                     (A.SR_STENCIL_ALWAYS, A.SR_STENCIL_INVERT),
                                     (A.SR_STENCIL_ALWAYS, A.SR_STENCIL_DECREMENT)])
def test_stencil_modes_opaque(built_lib, oracle_mod, test_op):
    sc = scenes.icosphere_scene(150, 110, stencil=True, tile=(32, 32), stencil_ref=3,
                                stencil_test=test_op[0], stencil_op=test_op[1])
    rng = np.random.default_rng(11)
    st0 = rng.integers(0, 7, (sc.height, sc.width)).astype(np.uint8)
    check(sc, oracle_mod, initial=(None, None, st0))


@pytest.mark.parametrize("test_op", [(A.SR_STENCIL_LESS_THAN, A.SR_STENCIL_INCREMENT),
                                     (A.SR_STENCIL_GREATER_THAN_EQ, A.SR_STENCIL_ZERO),
                                     (A.SR_STENCIL_NOT_EQUAL, A.SR_STENCIL_REPLACE)])
def test_stencil_exhaustive(built_lib, oracle_mod, test_op):
    """Tests whose outcome changes with the stencil value: the exhaustive path."""
    sc = scenes.icosphere_scene(96, 80, stencil=True, tile=(24, 20), stencil_ref=2, subdiv=2,
                                stencil_test=test_op[0], stencil_op=test_op[1])
    rng = np.random.default_rng(12)
    st0 = rng.integers(0, 5, (sc.height, sc.width)).astype(np.uint8)
    check(sc, oracle_mod, initial=(None, None, st0))


@pytest.mark.parametrize("which", ["icosphere", "gridsphere"])
def test_clip_keeps_degenerate_under_stencil(built_lib, oracle_mod, which):
    """Clip geometry shader with stencil counting: the 15 degenerate fan
    triangles of each inside triangle stay (their bbox pixels are stencil
    events).  The icosphere lies inside every plane; the grid-sphere camera
    makes a share of the triangles cross planes."""
    kw = dict(stencil=True, stencil_test=A.SR_STENCIL_ALWAYS, stencil_op=A.SR_STENCIL_INCREMENT, stencil_wrap=1)
    if which == "icosphere":
        sc = scenes.icosphere_scene(160, 120, subdiv=2, gs_mode=A.SR_GS_CLIP, tile=(40, 32), **kw)
    else:
        sc = scenes.grid_sphere_scene(width=192, height=108, n_lat=16, n_lon=32, tex_size=32, tile=(48, 40), **kw)
    stats, ostats = check(sc, oracle_mod)
    assert stats["triangles_generated"] == ostats["triangles_generated"]


def test_blend_over_f32(built_lib, oracle_mod):
    sc = scenes.stress_scene(n_tiny=1500, n_large=20, size=128, tile=(48, 40))
    sc.color_format = A.SR_COLOR_RGBA32F
    sc.stencil = False
    check(sc, oracle_mod)


# ------------------------------------------------- rounding-dominated slivers
@pytest.mark.parametrize("blend", ["replace", "over"])
def test_slivers(built_lib, oracle_mod, blend):
    """Nearly collinear primitives whose coverage outside the bbox is decided
    by rounding: the unsafe classification and extension pass must reproduce
    the reference's tile-edge fragments exactly."""
    sc = scenes.sliver_scene(n=3000, size=256, blend=blend)
    stats, _ = check(sc, oracle_mod)
    assert stats["unsafe_triangles"] > 0


def test_slivers_stencil(built_lib, oracle_mod):
    sc = scenes.sliver_scene(n=1500, size=160, stencil=True, stencil_test=A.SR_STENCIL_ALWAYS,
                             stencil_op=A.SR_STENCIL_INCREMENT, stencil_wrap=0, tile=(24, 40))
    check(sc, oracle_mod)


@pytest.fixture
def force_unsafe():
    import os
    os.environ["SR_FORCE_UNSAFE"] = "1"
    yield
    del os.environ["SR_FORCE_UNSAFE"]


@pytest.mark.parametrize("make", [
    lambda: scenes.sliver_scene(n=800, size=200, seed=3),
    lambda: scenes.icosphere_scene(180, 140, tile=(32, 24), subdiv=3),
    lambda: scenes.stress_scene(n_tiny=800, n_large=12, size=128, tile=(24, 40)),
    lambda: scenes.grid_sphere_scene(width=256, height=144, n_lat=16, n_lon=32, tex_size=32, tile=(40, 32)),
])
def test_forced_unsafe_path(built_lib, oracle_mod, force_unsafe, make):
    """Every primitive through the unsafe path: bbox bins plus the exact
    evaluation of its clamped tile-edge targets (extension pass)."""
    stats, _ = check(make(), oracle_mod)
    assert stats["unsafe_triangles"] == stats["triangles_raster"] > 0


@pytest.mark.parametrize("size,n", [(64, 20000), (96, 60000)])
def test_dense_overlap(built_lib, oracle_mod, size, n):
    """Thousands of primitives per pixel block: many concurrent 64-bit atomicMax
    reductions on the same pixels must still select the reference's winner."""
    sc = scenes.stress_scene(n_tiny=n, n_large=3, size=size, blend="replace", tile=(20, 24))
    sc.stencil = False
    stats, _ = check(sc, oracle_mod)
    assert stats["fragments"] > n // 4


def test_dense_bins_depth_ties(built_lib, oracle_mod):
    """Equal depths everywhere: the last primitive in submission order wins."""
    sc = scenes.stress_scene(n_tiny=30000, n_large=0, size=64, blend="replace", tile=(16, 16))
    sc.stencil = False
    z = sc.planes[2]
    z[:] = np.float32(0.25)
    check(sc, oracle_mod)


def test_read_async_matches_read(built_lib):
    """sr_framebuffer_read_async enqueues the copies; after sr_sync the host
    buffers equal a synchronous read."""
    import numpy as np
    from softrender._lib import lib
    sc = scenes.icosphere_scene(160, 120, color_format=A.SR_COLOR_RGBA8)
    pl, mesh, tex = sr.prepare_scene(sc)
    try:
        sr.submit_scene(pl, mesh, tex, sc)
        hc = np.zeros((sc.height, sc.width), np.uint32)
        hd = np.zeros((sc.height, sc.width), np.float32)
        assert lib().sr_framebuffer_read_async(pl.handle, hc.ctypes.data, hd.ctypes.data, None) == 0
        assert pl.sync() == 0
        c, d, _ = pl.read()
        assert np.array_equal(hc, c) and np.array_equal(hd.view(np.uint32), d.view(np.uint32))
    finally:
        pl.destroy()
        mesh.free()


def test_ordered_bins_longer_than_16k(built_lib, oracle_mod):
    """Blended draws whose bins hold more than 16,384 primitives (every bin
    of a 64x64 frame is covered by some 22,000 of 40,000 large alpha triangles)."""
    sc = scenes.stress_scene(n_tiny=64, n_large=40000, size=64, seed=3, seed_large=5)
    stats, _ = check(sc, oracle_mod)
    assert stats["bin_entries"] > 16 * 16384


@pytest.mark.parametrize("fmt", [A.SR_COLOR_RGBA32F, A.SR_COLOR_RGBA8])
@pytest.mark.parametrize("gs_mode", [A.SR_GS_NONE, A.SR_GS_CLIP])
def test_aces_lights(built_lib, oracle_mod, fmt, gs_mode):
    """The 4-point-light Blinn-Phong with the ACES tonemap
    (full_example/src/shaders.rs:108-163)."""
    sc = scenes.icosphere_scene(200, 150, subdiv=3, fs="aces_lights", color_format=fmt, gs_mode=gs_mode,
                                tile=(64, 48))
    stats, _ = check(sc, oracle_mod)
    assert stats["fragments"] > 0
