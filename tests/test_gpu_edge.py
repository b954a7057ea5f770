"""Edge cases of the inputs, against the oracle where the reference defines
the outcome.

- A vertex with a NaN position: the reference's clamp_as_int panics on the
  all-NaN bbox (triangle.rs:66-78); here the primitive is skipped and the draw
  reports SR_ENAN, the oracle likewise (status 7).
- A clip-space vertex with w = 0 (ClipVertex::normalize computes 1/w,
  clipvertex.rs:121), through run_to_fragment and through the clip shader.
- Zero-area triangles, triangles far outside the frame (their clamped bbox
  collapses onto tile edges) and coordinates near the f32 range.
- Frames one pixel wide or high (no semantic tile: fragment.rs:188-216 never
  enters its loop), an empty index buffer.
- An index past the vertex count: the reference indexes out of bounds
  (a panic); the library skips that primitive, renders the rest and sync
  returns SR_EINVAL; the pipeline stays usable."""
import ctypes as C

import numpy as np
import pytest

from softrender import _abi as A
from softrender import scenes
from test_gpu_parity import check

pytestmark = pytest.mark.gpu

F = np.float32


def _clip_scene(W, H, verts, tile=(8, 8), **kw):
    """Triangles given directly in clip space: verts is (n, 4) x, y, z, w;
    colours vary per vertex (vertex shader clip_color, fragment shader
    vertex_color)."""
    v = np.asarray(verts, dtype=np.float64).reshape(-1, 4)
    n = v.shape[0]
    rng = np.random.default_rng(n)
    col = rng.uniform(0.1, 1.0, (n, 4))
    planes = [np.asarray(v[:, j], F) for j in range(4)] + [np.asarray(col[:, j], F) for j in range(4)]
    sc = scenes.Scene(planes=planes, indices=np.arange(n, dtype=np.uint32), width=W, height=H,
                      color_format=A.SR_COLOR_RGBA8, vs="clip_color", fs="vertex_color", tile=tile,
                      clear_color=(0, 0, 0, 0))
    for k, val in kw.items():
        setattr(sc, k, val)
    return sc


GOOD = [(-0.8, -0.7, 0.3, 1.0), (0.7, -0.6, 0.4, 1.0), (0.0, 0.8, 0.5, 1.0),
        (-0.5, 0.5, 0.2, 1.0), (0.9, 0.9, 0.6, 1.0), (-0.9, 0.1, 0.7, 1.0)]


@pytest.mark.parametrize("cull", [A.SR_CULL_CLOCKWISE, A.SR_CULL_COUNTER_CLOCKWISE])
def test_nan_shoelace_area_culling(built_lib, oracle_mod, cull):
    """A NaN shoelace sum (triangle.rs:53-61) winds counter-clockwise on the
    GPU as in the oracle: the stencil shows whether the triangle was culled."""
    nan = float("nan")
    sc = _clip_scene(24, 20, [(-0.6, nan, 0.5, 1.0), (0.6, -0.5, 0.5, 1.0), (0.0, 0.7, 0.5, 1.0)] + GOOD[:3],
                     stencil=True, stencil_test=A.SR_STENCIL_ALWAYS, stencil_op=A.SR_STENCIL_INCREMENT, cull=cull)
    check(sc, oracle_mod)


@pytest.mark.parametrize("gs_mode", [A.SR_GS_NONE, A.SR_GS_CLIP])
def test_nan_vertex(built_lib, oracle_mod, gs_mode):
    nan = float("nan")
    sc = _clip_scene(40, 30, GOOD + [(0.1, 0.1, 0.5, 1.0), (nan, 0.2, 0.5, 1.0), (0.3, -0.4, 0.5, 1.0)],
                     gs_mode=gs_mode)
    stats, ostats = check(sc, oracle_mod)
    assert stats["fragments"] > 0


@pytest.mark.parametrize("gs_mode", [A.SR_GS_NONE, A.SR_GS_CLIP])
def test_w_zero_vertex(built_lib, oracle_mod, gs_mode):
    sc = _clip_scene(40, 30, GOOD + [(0.2, 0.1, 0.0, 0.0), (0.6, 0.3, 0.5, 1.0), (0.1, 0.7, 0.4, 1.0)],
                     gs_mode=gs_mode)
    check(sc, oracle_mod)


def test_zero_area_and_far_outside(built_lib, oracle_mod):
    tris = GOOD + [
        (-0.5, -0.5, 0.5, 1.0), (0.0, 0.0, 0.5, 1.0), (0.5, 0.5, 0.5, 1.0),        # collinear
        (0.2, 0.2, 0.5, 1.0), (0.2, 0.2, 0.5, 1.0), (0.2, 0.2, 0.5, 1.0),          # a point
        (30.0, 30.0, 0.5, 1.0), (40.0, 30.0, 0.5, 1.0), (30.0, 45.0, 0.5, 1.0),    # far outside
        (-1e30, -1e30, 0.5, 1.0), (1e30, -1e30, 0.5, 1.0), (0.0, 1e30, 0.5, 1.0),  # near the f32 range
        (-3.0, -0.2, 0.5, 1.0), (3.0, -0.1, 0.5, 1.0), (0.0, 0.05, 0.5, 1.0),      # sliver across the frame
    ]
    import os
    for force in (False, True):
        # SR_FORCE_UNSAFE=1: every primitive through the exact clamped-edge path
        if force:
            os.environ["SR_FORCE_UNSAFE"] = "1"
        try:
            check(_clip_scene(48, 36, tris), oracle_mod)
        finally:
            os.environ.pop("SR_FORCE_UNSAFE", None)


@pytest.mark.parametrize("wh", [(1, 9), (9, 1), (1, 1), (2, 2)])
def test_tiny_frames(built_lib, oracle_mod, wh):
    sc = _clip_scene(wh[0], wh[1], GOOD)
    check(sc, oracle_mod)


def test_empty_mesh(built_lib, oracle_mod):
    sc = _clip_scene(16, 16, GOOD)
    sc.indices = np.zeros(0, dtype=np.uint32)
    stats, _ = check(sc, oracle_mod)
    assert stats["fragments"] == 0


def test_index_out_of_range(built_lib, oracle_mod):
    import softrender as sr
    sc = _clip_scene(32, 32, GOOD)
    # an upload is checked on the host
    with pytest.raises(sr.SoftrenderError):
        sr.Mesh(sc.planes, np.array([0, 1, 2, 3, 4, 99], dtype=np.uint32))
    pl, mesh, _ = sr.prepare_scene(sc)
    bad = sr.Mesh(sc.planes, sc.indices)
    try:
        # an update is copied asynchronously and checked on the device
        bad.update(sc.planes, np.array([0, 1, 2, 3, 4, 99], dtype=np.uint32))
        d = sr.draw_for_scene(sc, bad)
        assert sr.lib().sr_render(pl.handle, C.byref(d)) == A.SR_OK
        assert pl.sync() == A.SR_EINVAL
        # the pipeline stays usable: a clean draw afterwards matches the oracle
        pl.clear([0, 0, 0, 0])
        sr.submit_scene(pl, mesh, None, sc)
        assert pl.sync() == A.SR_OK
        color, depth, _ = pl.read()
    finally:
        pl.destroy()
        mesh.free()
        bad.free()
    fb, _, _ = oracle_mod.render(sc)
    assert np.array_equal(color, fb.color.view(np.uint32).reshape(32, 32))
    assert np.array_equal(depth.view(np.uint32), fb.depth.view(np.uint32))


def test_mesh_and_texture_freed_before_sync(built_lib, oracle_mod):
    """Meshes and textures are shared like the reference's Arc<Mesh>
    (src/pipeline/mod.rs:146): freeing the caller's handles right after
    sr_render leaves them alive for the pending draw.  The first clipped draw
    on a fresh pipeline outgrows its clip-output buffers (sized 2 x inputs +
    4096; with stencil counting every inside triangle keeps its 16 fan
    outputs), so sr_sync replays it from its descriptor after the handles are
    gone; the frame still equals the oracle's."""
    import softrender as sr
    from util import compare_frame
    sc = scenes.grid_sphere_scene(64, 48, n_lat=16, n_lon=32, tex_size=16, color_format=A.SR_COLOR_RGBA8,
                                  stencil=True, stencil_test=A.SR_STENCIL_ALWAYS,
                                  stencil_op=A.SR_STENCIL_INCREMENT, stencil_wrap=1)
    assert sc.gs_mode == A.SR_GS_CLIP
    pl, mesh, tex = sr.prepare_scene(sc)
    try:
        d = sr.draw_for_scene(sc, mesh, tex)
        assert sr.lib().sr_render(pl.handle, C.byref(d)) == A.SR_OK
        mesh.free()
        tex.free()
        assert pl.sync() == A.SR_OK
        n_in = sc.indices.shape[0] // 3
        assert pl.stats()["triangles_generated"] > 2 * n_in + 4096       # the draw was replayed
        got = pl.read()
    finally:
        pl.destroy()
    fb, _, _ = oracle_mod.render(sc)
    compare_frame(got, fb)


@pytest.mark.parametrize("aa", [False, True])
def test_nan_line_end_point(built_lib, oracle_mod, aa):
    """A line with a NaN vertex under stencil counting, Bresenham and Xiaolin
    Wu: skipped with SR_ENAN where the reference's cast to i64 panics or is
    undefined (line.rs:111-116, 163); the rest of the frame equals the
    oracle's."""
    sc = scenes.lines_scene(n=60, size=64, seed=21, tile=(16, 16), stencil=True, stencil_test=A.SR_STENCIL_ALWAYS,
                            stencil_op=A.SR_STENCIL_INCREMENT, aa_lines=aa)
    sc.planes[0] = sc.planes[0].copy()
    sc.planes[0][2 * 7] = np.float32("nan")
    stats, ostats = check(sc, oracle_mod)
    assert stats["fragments"] > 0


def test_clear_between_draws_survives_replay(built_lib, oracle_mod):
    """Draw A, clear, draw B, sync: A outgrows its clip-output buffers on the
    fresh pipeline, so sync replays from A -- and must clear again before B,
    as the sequence did (Framebuffer::clear between render_mesh calls).
    The frame equals B alone on the cleared framebuffer, stencil included,
    and an asynchronous read enqueued right after A holds A alone (the
    replay repeats the copy in its place)."""
    import softrender as sr
    from util import compare_frame
    kw = dict(color_format=A.SR_COLOR_RGBA8, stencil=True, stencil_test=A.SR_STENCIL_ALWAYS,
              stencil_op=A.SR_STENCIL_INCREMENT, stencil_wrap=1)
    a = scenes.grid_sphere_scene(64, 48, n_lat=16, n_lon=32, tex_size=16, **kw)
    b = scenes.icosphere_scene(64, 48, subdiv=2, **kw)
    b.clear_color = (0.2, 0.4, 0.6, 1.0)
    pl, mesh_a, tex_a = sr.prepare_scene(a)
    mesh_b = sr.Mesh(b.planes, b.indices)
    try:
        L = sr.lib()
        da = sr.draw_for_scene(a, mesh_a, tex_a)
        assert L.sr_render(pl.handle, C.byref(da)) == A.SR_OK
        hc = np.zeros((a.height, a.width), np.uint32)
        hd = np.zeros((a.height, a.width), np.float32)
        hs = np.zeros((a.height, a.width), np.uint8)
        assert L.sr_framebuffer_read_async(pl.handle, hc.ctypes.data, hd.ctypes.data, hs.ctypes.data) == A.SR_OK
        pl.clear(list(b.clear_bytes()))
        pl.set_uniforms(b.uniforms)
        db = sr.draw_for_scene(b, mesh_b)
        assert L.sr_render(pl.handle, C.byref(db)) == A.SR_OK
        assert pl.sync() == A.SR_OK
        got = pl.read()
    finally:
        pl.destroy()
        mesh_a.free()
        mesh_b.free()
        tex_a.free()
    fb, _, _ = oracle_mod.render(b)
    compare_frame(got, fb)
    fa, _, _ = oracle_mod.render(a)
    compare_frame((hc, hd, hs), fa)
