"""Batched rendering (sr_batch_*) against the plain per-draw path.

Every target's framebuffer after a batch must equal, bit for bit, what
sr_render produces for the same draw on the same starting framebuffer — for
every launch configuration, with and without CUDA graphs, and over two
consecutive batches (the second drawing over the first's output)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _mix(n=10, seed=11):
    """Uneven instances: small and large meshes, several resolutions, both
    colour formats, culling, a textured shader and a non-square frame."""
    from softrender import _abi as A
    from softrender import scenes
    out = []
    for i, sc in enumerate(scenes.batch_instances(n=n, seed=seed, tri_lo=200, tri_hi=40000,
                                                  resolutions=(64, 128, 256, 300))):
        if i % 3 == 1:
            sc.color_format = A.SR_COLOR_RGBA32F
        if i % 4 == 2:
            sc.cull = A.SR_CULL_CLOCKWISE
        if i % 5 == 3:
            sc.width, sc.height = sc.width, max(2, sc.height // 2 + 7)
            sc.viewport = (0.0, 0.0, float(sc.width), float(sc.height), 0.0, 1.0)
        out.append(sc)
    tex_sc = scenes.grid_sphere_scene(200, 150, n_lat=24, n_lon=48, tex_size=64, gs_mode=A.SR_GS_NONE,
                                      camera=dict(eye=(0.3, 0.2, 2.5), target=(0.0, 0.0, 0.0)))
    out.append(tex_sc)
    return out


def _clear_bytes(sc):
    return sc.clear_bytes()


def _plain(scenes_, initial=None):
    """sr_render per draw (reference for the batch)."""
    import softrender as sr
    res = []
    for k, sc in enumerate(scenes_):
        init = None if initial is None else initial[k]
        color, depth, _, _, status = sr.render_scene(sc, init)
        assert status == 0
        res.append((color.copy(), depth.copy()))
    return res


class Targets:
    def __init__(self, scenes_):
        import softrender as sr
        self.pls, self.meshes, self.texs, self.draws = [], [], [], []
        for sc in scenes_:
            fb = sr.Framebuffer(sc.width, sc.height, sc.color_format, sc.depth, sc.stencil)
            pl = sr.Pipeline.from_framebuffer(fb, sc.uniforms)
            m = sr.Mesh(sc.planes, sc.indices)
            t = sr.Texture(sc.texture) if sc.texture is not None else None
            self.pls.append(pl)
            self.meshes.append(m)
            self.texs.append(t)
            self.draws.append(sr.draw_for_scene(sc, m, t))

    def read(self):
        return [tuple(x.copy() for x in pl.read()[:2]) for pl in self.pls]

    def free(self):
        for pl in self.pls:
            pl.destroy()
        for m in self.meshes:
            m.free()
        for t in self.texs:
            if t is not None:
                t.free()


def _same(got, want):
    for k, ((gc, gd), (wc, wd)) in enumerate(zip(got, want)):
        assert np.array_equal(gc.view(np.uint8), wc.view(np.uint8)), "colour differs for draw %d" % k
        assert np.array_equal(gd.view(np.uint32), wd.view(np.uint32)), "depth differs for draw %d" % k


@pytest.mark.parametrize("graphs", [True, False])
def test_batch_matches_plain(built_lib, graphs):
    import softrender as sr
    scs = _mix()
    want = _plain(scs)
    T = Targets(scs)
    b = sr.Batch(use_graphs=graphs, autotune=False)
    try:
        b.render([(T.pls[k], T.draws[k], _clear_bytes(sc)) for k, sc in enumerate(scs)])
        assert b.sync() == 0
        _same(T.read(), want)
        st = b.stats()
        assert st["triangles_in"] == sum(sc.n_tris for sc in scs)
        assert st["fragments"] > 0
    finally:
        b.destroy()
        T.free()


def test_batch_every_config_identical(built_lib):
    import softrender as sr
    scs = _mix(n=6, seed=5)
    want = _plain(scs)
    T = Targets(scs)
    b = sr.Batch(use_graphs=True, autotune=False)
    try:
        for cfg in [(1, 64, 1), (4, 512, 4), (8, 2048, 8), (32, 8192, 2), (16, 1 << 30, 8)]:
            b.set_config(*cfg)
            b.render([(T.pls[k], T.draws[k], _clear_bytes(sc)) for k, sc in enumerate(scs)])
            assert b.sync() == 0
            assert b.config() == cfg
            _same(T.read(), want)
    finally:
        b.destroy()
        T.free()


def test_batch_autotune_and_two_batches_in_a_row(built_lib):
    """Second batch draws new cameras over the first batch's output, without
    clearing: must equal sr_render of the second draw on that framebuffer."""
    import copy
    import softrender as sr
    from softrender import scenes
    scs = _mix(n=8, seed=7)
    first = _plain(scs)
    second_scs = []
    rng = np.random.default_rng(3)
    for sc in scs:
        s2 = copy.copy(sc)
        eye = scenes.random_camera(rng)
        view = scenes.look_at_rh(eye, (0, 0, 0), (0, 1, 0))
        s2.uniforms = scenes.make_uniforms(view=view, projection=scenes.perspective(
            sc.width / sc.height, np.radians(60.0), 0.1, 100.0), camera=eye)
        second_scs.append(s2)
    want2 = _plain(second_scs, initial=[(c, d, None) for c, d in first])
    T = Targets(scs)
    b = sr.Batch(use_graphs=True, autotune=True)
    try:
        b.render([(T.pls[k], T.draws[k], _clear_bytes(sc)) for k, sc in enumerate(scs)])
        assert b.sync() == 0
        _same(T.read(), first)
        for k, s2 in enumerate(second_scs):
            T.pls[k].set_uniforms(s2.uniforms)
        b.render([(T.pls[k], T.draws[k], None) for k in range(len(scs))])
        assert b.sync() == 0
        _same(T.read(), want2)
        g, big, ctas = b.config()
        assert g in (4, 8, 16, 32) and ctas in (4, 8)
    finally:
        b.destroy()
        T.free()


def test_batch_mixed_clears(built_lib):
    """One batch where only the even items clear (the clear is deferred past
    the raster passes and merged into resolve): even targets must equal a
    draw on a cleared framebuffer, odd ones a draw over the previous output;
    a target one pixel high renders nothing and is only cleared."""
    import copy
    import softrender as sr
    from softrender import scenes
    scs = _mix(n=7, seed=13)
    flat = copy.copy(scs[0])
    flat.width, flat.height = 50, 1
    flat.viewport = (0.0, 0.0, 50.0, 1.0, 0.0, 1.0)
    scs.append(flat)
    first = _plain(scs)
    rng = np.random.default_rng(8)
    second_scs = []
    for sc in scs:
        s2 = copy.copy(sc)
        eye = scenes.random_camera(rng)
        view = scenes.look_at_rh(eye, (0, 0, 0), (0, 1, 0))
        s2.uniforms = scenes.make_uniforms(view=view, projection=scenes.perspective(
            sc.width / sc.height, np.radians(60.0), 0.1, 100.0), camera=eye)
        second_scs.append(s2)
    want = []
    for k, s2 in enumerate(second_scs):
        if k % 2 == 0:
            want += _plain([s2])
        else:
            want += _plain([s2], initial=[(first[k][0], first[k][1], None)])
    T = Targets(scs)
    b = sr.Batch(use_graphs=True, autotune=False)
    try:
        b.render([(T.pls[k], T.draws[k], _clear_bytes(sc)) for k, sc in enumerate(scs)])
        assert b.sync() == 0
        _same(T.read(), first)
        for k, s2 in enumerate(second_scs):
            T.pls[k].set_uniforms(s2.uniforms)
        b.render([(T.pls[k], T.draws[k], _clear_bytes(s2) if k % 2 == 0 else None)
                  for k, s2 in enumerate(second_scs)])
        assert b.sync() == 0
        _same(T.read(), want)
    finally:
        b.destroy()
        T.free()


def test_batch_rejects_ineligible(built_lib):
    import softrender as sr
    from softrender import _abi as A
    scs = _mix(n=3, seed=9)
    T = Targets(scs)
    b = sr.Batch(autotune=False)
    try:
        # the same target twice
        st = b.render_items(b.items([(T.pls[0], T.draws[0], None), (T.pls[0], T.draws[1], None)]))
        assert st == A.SR_EINVAL
        # a clipping geometry shader
        d = T.draws[1]
        d2 = type(d).from_buffer_copy(d)
        d2.gs_mode = A.SR_GS_CLIP
        assert b.render_items(b.items([(T.pls[1], d2, None)])) == A.SR_EINVAL
        # blending
        d3 = type(d).from_buffer_copy(d)
        d3.blend = sr.shader_id("over", A.SR_STAGE_BLEND)
        assert b.render_items(b.items([(T.pls[1], d3, None)])) == A.SR_EINVAL
    finally:
        b.destroy()
        T.free()
