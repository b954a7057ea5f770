"""Known-answer tests that pin the CPU oracle (oracle/) to the reference.

The reference's own tests hold one value-pinning test, coordinate_index
(src/geometry/coordinate.rs:66-87); it is restated first.  The others are
hand-derived from the reference's formulas (file:line in each test) and are
computed here independently of the oracle's code: tile walks from the loop
in fragment.rs:188-216, viewport products from clipvertex.rs:89-127, the
clip push order of geometry.rs:264-299, coverage from triangle.rs:104-126
evaluated with numpy float32 (IEEE single, no contraction), the f32::MIN
depth clear, ties passing `>=`, stencil events per tile pass (clamped onto
tile edges, counted behind the depth test), the NaN coverage of a
zero-area triangle, seam pixels blended once per tile pass, and the
accuracy of the pow used by the shaders.  No GPU needed."""
import ctypes as C
import math

import numpy as np
import pytest

from softrender import _abi as A
from softrender import scenes

F = np.float32


def test_coordinate_index(oracle_mod):
    """coordinate.rs:66-87: index = x + y * width and back, on a 10 x 20 grid."""
    L = oracle_mod.lib()
    i = 0
    for y in range(20):
        for x in range(10):
            assert L.or_coordinate_into_index(x, y, 10) == i
            ox, oy = C.c_uint32(), C.c_uint32()
            L.or_coordinate_from_index(i, 10, C.byref(ox), C.byref(oy))
            assert (ox.value, oy.value) == (x, y)
            i += 1


def _tiles_by_hand(W, H, tw, th):
    # fragment.rs:188-216, written out independently
    out = []
    y = 0
    while y < H - 1:
        ny = min(y + th, H - 1)
        x = 0
        while x < W - 1:
            nx = min(x + tw, W - 1)
            out.append((x, y, nx, ny))
            x = nx
        y = ny
    return out


@pytest.mark.parametrize("W,H,tw,th,n", [(5, 4, 2, 2, 4), (1024, 1024, 128, 128, 64), (3840, 2160, 128, 128, 510),
                                         (2048, 2048, 128, 128, 256), (97, 61, 7, 13, None), (2, 2, 128, 128, 1),
                                         (1, 9, 4, 4, 0)])
def test_tiles(oracle_mod, W, H, tw, th, n):
    t = oracle_mod.tiles(W, H, tw, th)
    assert t == _tiles_by_hand(W, H, tw, th)
    if n is not None:
        assert len(t) == n
    # adjacent tiles share a column / row (inclusive corners)
    if len(t) > 1 and t[0][1] == t[1][1]:
        assert t[0][2] == t[1][0]


def test_tiles_small_known_answer(oracle_mod):
    assert oracle_mod.tiles(5, 4, 2, 2) == [(0, 0, 2, 2), (2, 0, 4, 2), (0, 2, 2, 3), (2, 2, 4, 3)]


def test_normalize_known_answers(oracle_mod):
    """clipvertex.rs:89-127 with viewport (0, 0, W, H, near 0, far 1): x' = W/2 x
    + W/2, y' = -H/2 y + H/2, z' = -z/2 - 1/2 (nearer is larger), w' = 1/w."""
    vp = (0.0, 0.0, 640.0, 480.0, 0.0, 1.0)
    assert np.array_equal(oracle_mod.normalize((0, 0, 0, 1), vp), np.array([320, 240, -0.5, 1], F))
    assert np.array_equal(oracle_mod.normalize((2, 2, 2, 2), vp), np.array([640, 0, -1, 0.5], F))
    assert np.array_equal(oracle_mod.normalize((-4, -4, 4, 4), vp), np.array([0, 480, -1, 0.25], F))


def test_clip_inside_triangle_structure(oracle_mod):
    """geometry.rs:264-299: a triangle inside every plane pushes each vertex 6
    times (poly = b*6, c*6, a*6) and the fan from the last entry yields 16
    triangles: (a, b, c) at index 5, the other 15 exactly degenerate."""
    a = (0.1, 0.2, 0.3, 1.0)
    b = (0.5, -0.2, 0.4, 1.0)
    c = (-0.3, 0.6, 0.5, 1.0)
    out = oracle_mod.clip_triangle(a, b, c).reshape(-1, 3, 4)
    assert out.shape[0] == 16
    assert np.array_equal(out[5], np.array([a, b, c], F))
    for k in range(16):
        if k == 5:
            continue
        t = out[k]
        assert (np.array_equal(t[0], t[1]) or np.array_equal(t[1], t[2]) or np.array_equal(t[0], t[2])), k


def test_clip_near_plane(oracle_mod):
    """Near plane is z >= 0 (clip.rs:33-44).  The push loop of geometry.rs:
    270-284 tests each plane independently, so with a (z < 0) outside only the
    near plane the polygon is [b b b b I_ab b b | c*6 | a a a a I_ca a]
    (19 entries -> 17 fan triangles): the near-plane intersections lie
    exactly on z = 0 (t = 0.5 here), and a itself is still emitted."""
    a = (0.0, 0.0, -0.5, 1.0)
    b = (0.5, 0.0, 0.5, 1.0)
    c = (0.0, 0.5, 0.5, 1.0)
    out = oracle_mod.clip_triangle(a, b, c).reshape(-1, 3, 4)
    assert out.shape[0] == 17
    verts = {tuple(v) for v in out.reshape(-1, 4).tolist()}
    assert (0.25, 0.0, 0.0, 1.0) in verts            # I_ab = lerp(0.5, a, b)
    assert (0.0, 0.25, 0.0, 1.0) in verts            # I_ca = lerp(0.5, c, a)
    assert a in verts
    assert sorted(v for v in verts if v[2] == 0.0) == [(0.0, 0.25, 0.0, 1.0), (0.25, 0.0, 0.0, 1.0)]


def _one_triangle_scene(tri_screen, W, H, z=-0.5, rgba=(255, 0, 0, 255), **kw):
    """Triangles given in screen space (every vertex at screen depth z)."""
    tri = np.asarray(tri_screen, dtype=np.float64)
    z_ndc = np.full(len(tri), z * -2.0 - 1.0)
    x, y, zz = scenes._clip_from_screen(tri[:, 0], tri[:, 1], z_ndc, W, H)
    col = np.array([rgba] * len(tri))
    packed = scenes._pack_rgba8(col[:, 0], col[:, 1], col[:, 2], col[:, 3])
    planes = [np.asarray(x, F), np.asarray(y, F), np.asarray(zz, F), packed.view(np.float32).copy()]
    sc = scenes.Scene(planes=planes, indices=np.arange(len(tri), dtype=np.uint32), width=W, height=H,
                      color_format=A.SR_COLOR_RGBA8, vs="clip_rgba8", fs="vertex_color", tile=(4, 4),
                      clear_color=(0, 0, 0, 0))
    for k, v in kw.items():
        setattr(sc, k, v)
    return sc


def _coverage_by_hand(v, W, H):
    """triangle.rs:64,104-113 in float32: inclusive, NaN counts as covered."""
    (x1, y1), (x2, y2), (x3, y3) = [(F(p[0]), F(p[1])) for p in v]
    det = (y2 - y3) * (x1 - x3) + (x3 - x2) * (y1 - y3)
    m = np.zeros((H, W), bool)
    for py in range(H):
        for px in range(W):
            x, y = F(px) + F(0.5), F(py) + F(0.5)
            u = ((y2 - y3) * (x - x3) + (x3 - x2) * (y - y3)) / det
            vv = ((y3 - y1) * (x - x3) + (x1 - x3) * (y - y3)) / det
            w = (F(1) - u) - vv
            m[py, px] = not (u < 0 or vv < 0 or w < 0)
    return m


def test_single_triangle_mask(oracle_mod):
    W = H = 12
    scr = [(1.25, 1.5), (10.5, 3.0), (4.0, 10.75)]
    sc = _one_triangle_scene(scr, W, H)
    fb, st, status = oracle_mod.render(sc)
    assert status == 0
    # the oracle's screen positions come from the same clip -> normalize path
    tri = oracle_mod.raster_tris(sc)[0]
    want = _coverage_by_hand([(tri[0][0], tri[0][1]), (tri[1][0], tri[1][1]), (tri[2][0], tri[2][1])], W, H)
    got = fb.color.view(np.uint32).reshape(H, W) != 0
    assert np.array_equal(got, want)
    assert st["fragments"] == int(want.sum())


def test_shared_edge_is_inclusive_and_ties_pass(oracle_mod):
    """Two triangles sharing an edge at equal depth: the edge pixels are
    covered by both (no top-left rule) and the later one wins (>=)."""
    W = H = 10
    quad = [(1.0, 1.0), (9.0, 1.0), (1.0, 9.0), (9.0, 1.0), (9.0, 9.0), (1.0, 9.0)]
    sc = _one_triangle_scene(quad, W, H)
    col = np.array([(255, 0, 0, 255)] * 3 + [(0, 255, 0, 255)] * 3)
    sc.planes[3] = scenes._pack_rgba8(col[:, 0], col[:, 1], col[:, 2], col[:, 3]).view(np.float32).copy()
    fb, _, _ = oracle_mod.render(sc)
    tris = oracle_mod.raster_tris(sc)
    m1 = _coverage_by_hand([tris[0][j][:2] for j in range(3)], W, H)
    m2 = _coverage_by_hand([tris[1][j][:2] for j in range(3)], W, H)
    both = m1 & m2
    assert both.any()                                  # inclusive edges: the diagonal is in both
    c = fb.color.view(np.uint32).reshape(H, W)
    green = scenes._pack_rgba8(np.array([0]), np.array([255]), np.array([0]), np.array([255]))[0]
    assert (c[both] == green).all()                    # the later triangle passes the >= test


def test_depth_clear_is_f32_min(oracle_mod):
    sc = _one_triangle_scene([(0, 0), (1, 0), (0, 1)], 4, 4)
    fb = oracle_mod.framebuffer_for(sc)
    assert (fb.depth == np.float32(-3.4028235e38)).all()


def test_stencil_counts_every_tile_pass(oracle_mod):
    """stencil.rs:112-158 applied per clamped-bbox pixel per tile pass
    (triangle.rs:90-99): a triangle whose bbox covers the frame increments
    each pixel once per semantic tile containing it (1, 2 or 4)."""
    W, H = 9, 9
    sc = _one_triangle_scene([(-5.0, -5.0), (30.0, -5.0), (-5.0, 30.0)], W, H, stencil=True,
                             stencil_test=A.SR_STENCIL_ALWAYS, stencil_op=A.SR_STENCIL_INCREMENT)
    fb, _, _ = oracle_mod.render(sc)
    want = np.zeros((H, W), np.uint8)
    for (x0, y0, x1, y1) in _tiles_by_hand(W, H, 4, 4):
        want[y0:y1 + 1, x0:x1 + 1] += 1
    assert np.array_equal(fb.stencil, want)
    assert want.max() == 4 and want.min() == 1


def test_pow_accuracy(oracle_mod):
    """The shaders' powf (own table-driven log2/exp2) is within 1 ULP of the
    exact power (float64 reference) over the ranges the shaders use."""
    rng = np.random.default_rng(0)
    xs = np.concatenate([rng.uniform(0, 1, 3000), np.exp(rng.uniform(-80, 5, 2000))]).astype(F)
    ys = np.array([2.2, 1 / 2.2, 64.0, 5.0, 0.5, 3.7, -1.3], F)
    worst = 0.0
    for y in ys:
        for x in xs[::7]:
            got = oracle_mod.powf(x, y)
            exact = float(x) ** float(y)
            if exact == 0.0 or not math.isfinite(exact) or exact < 1.2e-38 or exact > 3.0e38:
                continue
            ulp = float(np.spacing(np.float32(exact)))
            worst = max(worst, abs(float(got) - exact) / ulp)
    assert worst <= 1.0, worst


def test_pow_special_cases(oracle_mod):
    p = oracle_mod.powf
    assert p(0.0, 2.2) == 0.0 and p(1.0, 123.0) == 1.0 and p(3.0, 0.0) == 1.0
    assert p(2.0, 10.0) == 1024.0 and p(0.25, 0.5) == 0.5
    assert np.isnan(p(-2.0, 0.5))


def test_byte_to_unit_exact(oracle_mod):
    for c in range(256):
        assert oracle_mod.u8_unit(c) == F(c) / F(255)


def _clamp_as_int(v, lo, hi):
    # triangle.rs:66-78: below the tile -> its low edge, above -> its high edge, else trunc
    return lo if v < lo else hi if v > hi else int(math.trunc(v))


def _stencil_events_by_hand(tri_xy, W, H, tw, th):
    """Stencil events of one triangle (triangle.rs:82-99): every pixel of its
    bbox clamped to each semantic tile, once per tile, covered or not."""
    xs, ys = [float(p[0]) for p in tri_xy], [float(p[1]) for p in tri_xy]
    want = np.zeros((H, W), np.uint8)
    for (x0, y0, x1, y1) in _tiles_by_hand(W, H, tw, th):
        mnx, mxx = _clamp_as_int(min(xs), x0, x1), _clamp_as_int(max(xs), x0, x1)
        mny, mxy = _clamp_as_int(min(ys), y0, y1), _clamp_as_int(max(ys), y0, y1)
        want[mny:mxy + 1, mnx:mxx + 1] += 1
    return want


def test_degenerate_triangle_nan_path(oracle_mod):
    """A triangle with det = 0 (triangle.rs:64): at a pixel centre on its line
    both numerators are 0, so u = v = w = NaN and the pixel counts as covered
    (triangle.rs:113); the interpolated depth is NaN too, so `pos.z < 0`
    fails (triangle.rs:120) and nothing is shaded.  The stencil, applied per
    bbox pixel before the coverage test (triangle.rs:90-99), still counts, and
    its bbox clamped onto a tile it misses collapses onto that tile's edge row."""
    W = H = 8
    sc = _one_triangle_scene([(1.5, 2.5), (5.5, 2.5), (3.5, 2.5)], W, H, stencil=True,
                             stencil_test=A.SR_STENCIL_ALWAYS, stencil_op=A.SR_STENCIL_INCREMENT)
    tri = oracle_mod.raster_tris(sc)[0]
    xy = [(tri[j][0], tri[j][1]) for j in range(3)]
    assert all(p[1] == F(2.5) for p in xy)            # the line runs exactly through row 2's centres
    with np.errstate(divide="ignore", invalid="ignore"):
        m = _coverage_by_hand(xy, W, H)
    # covered through NaN: every centre of row 2 lies on the line (the bbox
    # limits the visited ones to x = 1..5)
    assert m.sum() == W and m[2].all()
    fb, st, status = oracle_mod.render(sc)
    assert status == 0 and st["fragments"] == 0
    assert (fb.color == 0).all()
    assert (fb.depth == F(-3.4028235e38)).all()
    want = _stencil_events_by_hand(xy, W, H, 4, 4)
    assert want[4].any()                              # events on the edge row of the tiles below
    assert np.array_equal(fb.stencil, want)


def test_seam_pixels_blend_once_per_tile_pass(oracle_mod):
    """Adjacent semantic tiles share a row or column (fragment.rs:188-216) and
    every primitive is visited in every tile (fragment.rs:240-318), so with a
    blend a seam pixel is blended once per tile holding it, and ties pass the
    depth test (`>=`, triangle.rs:120-126) each time.  Checked per pixel: one
    draw with 4x4 tiles equals the same triangle drawn, with one tile over the
    whole frame, as many times as 4x4 tiles hold that pixel (1, 2 or 4)."""
    W = H = 9
    kw = dict(rgba=(200, 100, 50, 128), blend="over", clear_color=(0.0, 0.0, 1.0, 1.0))
    tri = [(-5.0, -5.0), (30.0, -5.0), (-5.0, 30.0)]
    tiled, _, status = oracle_mod.render(_one_triangle_scene(tri, W, H, **kw))
    assert status == 0
    whole = _one_triangle_scene(tri, W, H, tile=(128, 128), **kw)
    assert len(_tiles_by_hand(W, H, 128, 128)) == 1
    fb = oracle_mod.framebuffer_for(whole)
    after = {}
    for k in range(1, 5):
        fb, _, _ = oracle_mod.render(whole, fb=fb)
        after[k] = fb.color.view(np.uint32).reshape(H, W).copy()
    count = np.zeros((H, W), int)
    for (x0, y0, x1, y1) in _tiles_by_hand(W, H, 4, 4):
        count[y0:y1 + 1, x0:x1 + 1] += 1
    assert sorted(set(count.ravel().tolist())) == [1, 2, 4]
    want = np.choose(count - 1, [after[1], after[2], after[3], after[4]])
    got = tiled.color.view(np.uint32).reshape(H, W)
    assert np.array_equal(got, want)
    assert (after[2] != after[1]).all()              # each extra blend changes the pixel


def test_stencil_counts_pixels_failing_depth(oracle_mod):
    """The stencil op runs before the depth test (triangle.rs:90-99 then
    :120-126): a triangle behind the depth already written still counts its
    events, and leaves colour and depth as they were."""
    W = H = 9
    tri = [(-5.0, -5.0), (30.0, -5.0), (-5.0, 30.0)]
    front = _one_triangle_scene(tri, W, H, z=-0.25, stencil=True,
                                stencil_test=A.SR_STENCIL_ALWAYS, stencil_op=A.SR_STENCIL_INCREMENT)
    back = _one_triangle_scene(tri, W, H, z=-0.75, rgba=(0, 255, 0, 255), stencil=True,
                               stencil_test=A.SR_STENCIL_ALWAYS, stencil_op=A.SR_STENCIL_INCREMENT)
    fb, _, _ = oracle_mod.render(front)
    color, depth = fb.color.copy(), fb.depth.copy()
    fb, st, status = oracle_mod.render(back, fb=fb)
    assert status == 0 and st["fragments"] > 0                     # covered, reaching the depth test
    assert np.array_equal(fb.color, color) and np.array_equal(fb.depth, depth)
    xy = [(v[0], v[1]) for v in oracle_mod.raster_tris(front)[0]]
    assert np.array_equal(fb.stencil, 2 * _stencil_events_by_hand(xy, W, H, 4, 4))


def test_strided_tiles_partition_the_frame(oracle_mod):
    """The tile stride used for timing samples selects exactly every k-th tile:
    for an opaque draw with a counting stencil (neither depends on the order
    of tile passes) the even tiles then the odd tiles into one framebuffer
    give the full frame, colour, depth and stencil, and their fragment
    counts add up."""
    sc = scenes.icosphere_scene(40, 30, subdiv=2, color_format=A.SR_COLOR_RGBA8)
    sc.tile = (8, 8)
    sc.stencil = True
    sc.stencil_test, sc.stencil_op = A.SR_STENCIL_ALWAYS, A.SR_STENCIL_INCREMENT
    full, st_full, s0 = oracle_mod.render(sc)
    n = int(st_full["tiles"])
    assert s0 == 0 and n == 20
    fb = oracle_mod.framebuffer_for(sc)
    frags = 0
    for first in (0, 1):
        fb, st, s = oracle_mod.render(sc, fb=fb, tile_begin=first, tile_step=2)
        assert s == 0
        frags += st["fragments"]
    assert np.array_equal(fb.color, full.color)
    assert np.array_equal(fb.depth.view(np.uint32), full.depth.view(np.uint32))
    assert np.array_equal(fb.stencil, full.stencil)
    assert frags == st_full["fragments"] > 0
    # a window of 3 tiles with stride 7 rasterises tiles 2, 9, 16 only
    _, st3, _ = oracle_mod.render(sc, tile_begin=2, tile_end=2 + 7 * 3, tile_step=7)
    one = sum(oracle_mod.render(sc, tile_begin=t, tile_end=t + 1)[1]["fragments"] for t in (2, 9, 16))
    assert st3["fragments"] == one


@pytest.mark.parametrize("aa", [False, True])
def test_nan_line_end_point(oracle_mod, aa):
    """A line with a NaN vertex: Liang-Barsky (line.rs:22-52) passes NaN end
    points through; Bresenham's cast to i64 then panics in the reference
    (line.rs:111-116) and Xiaolin Wu's `as i64` of NaN (line.rs:163) was
    undefined when it was written, so the oracle skips the line and reports
    status 7 -- the frame equals the scene without that line, stencil events
    included."""
    kw = dict(stencil=True, stencil_test=A.SR_STENCIL_ALWAYS, stencil_op=A.SR_STENCIL_INCREMENT, aa_lines=aa)
    sc = scenes.lines_scene(n=60, size=64, seed=21, tile=(16, 16), **kw)
    sc.planes[0] = sc.planes[0].copy()
    sc.planes[0][2 * 7] = np.float32("nan")                      # line 7's first vertex
    fb, st, status = oracle_mod.render(sc)
    assert status == 7
    keep = np.ones(sc.indices.shape[0], bool)
    keep[14:16] = False
    dropped = scenes.lines_scene(n=60, size=64, seed=21, tile=(16, 16), **kw)
    dropped.indices = sc.indices[keep]
    fb2, st2, status2 = oracle_mod.render(dropped)
    assert status2 == 0
    assert np.array_equal(fb.color, fb2.color)
    assert np.array_equal(fb.depth.view(np.uint32), fb2.depth.view(np.uint32))
    assert np.array_equal(fb.stencil, fb2.stencil)
    assert st["fragments"] == st2["fragments"] > 0


@pytest.mark.parametrize("cull", [A.SR_CULL_CLOCKWISE, A.SR_CULL_COUNTER_CLOCKWISE])
def test_nan_shoelace_area_winds_counter_clockwise(oracle_mod, cull):
    """triangle.rs:53-61 culls by `a.is_sign_negative()` of the shoelace sum.
    A vertex with a NaN coordinate makes that sum NaN, whose sign bit IEEE
    754 leaves to the platform (x86's default NaN has it set, AArch64's and
    CUDA's do not, and an input NaN's sign propagates).  Here a NaN sum is
    read as not negative -- counter-clockwise -- on every platform: with
    back faces counter-clockwise the triangle is culled and leaves the
    stencil untouched; with clockwise culling it is kept, and its (finite,
    NaN-ignoring) bbox counts stencil events in every tile pass though no
    pixel is covered with a finite depth."""
    W = H = 12
    sc = _one_triangle_scene([(2.0, 2.0), (9.0, 3.0), (4.0, 9.0)], W, H, stencil=True,
                             stencil_test=A.SR_STENCIL_ALWAYS, stencil_op=A.SR_STENCIL_INCREMENT, cull=cull)
    sc.planes[1] = sc.planes[1].copy()
    sc.planes[1][0] = np.float32(np.nan)          # vertex 1: y = NaN
    fb, st, status = oracle_mod.render(sc)
    assert status == 0 and st["fragments"] == 0
    if cull == A.SR_CULL_COUNTER_CLOCKWISE:
        assert (fb.stencil == 0).all()
    else:
        assert fb.stencil.max() >= 1
