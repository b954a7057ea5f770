"""Serving loop (sr_server_*): continuous batching under an HBM budget.

Each request's result, whether it was served in a mix of requests arriving
while others run on the GPU, under a budget that forces admission to wait,
or by the plain one-at-a-time mode, must equal rendering it alone with
sr_render (bit-exact colour and depth)."""
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _requests(n=24, seed=21):
    import softrender as sr
    from softrender import _abi as A
    from softrender import scenes
    scs = scenes.batch_instances(n=n, seed=seed, tri_lo=300, tri_hi=30000, resolutions=(64, 96, 128, 200))
    for i, sc in enumerate(scs):
        if i % 4 == 3:
            sc.color_format = A.SR_COLOR_RGBA32F
        if i % 5 == 1:
            sc.width = max(2, sc.width // 2 + 5)
            sc.viewport = (0.0, 0.0, float(sc.width), float(sc.height), 0.0, 1.0)
    meshes = [sr.Mesh(sc.planes, sc.indices) for sc in scs]
    draws = [sr.draw_for_scene(sc, m) for sc, m in zip(scs, meshes)]
    reqs = [sr.Server.request(d, sc.uniforms, sc.width, sc.height, sc.color_format, sc.clear_bytes())
            for d, sc in zip(draws, scs)]
    return scs, meshes, reqs


def _alone(scs):
    import softrender as sr
    out = []
    for sc in scs:
        c, d, _, _, st = sr.render_scene(sc)
        assert st == 0
        out.append((c.copy(), d.copy()))
    return out


def _check(got, want, k):
    gc, gd = got
    wc, wd = want
    assert np.array_equal(gc.view(np.uint8), wc.view(np.uint8)), "colour differs for request %d" % k
    assert np.array_equal(gd.view(np.uint32), wd.view(np.uint32)), "depth differs for request %d" % k


@pytest.mark.parametrize("plain", [False, True])
def test_server_results_equal_alone(built_lib, plain):
    import softrender as sr
    scs, meshes, reqs = _requests()
    want = _alone(scs)
    srv = sr.Server(max_inflight=3, max_batch=8, plain=plain)
    try:
        tickets = []
        rng = np.random.default_rng(1)
        for r in reqs:       # staggered arrivals: later requests join while earlier batches run
            st, t = srv.submit(r)
            assert st == 0
            tickets.append(t)
            time.sleep(float(rng.uniform(0.0, 0.002)))
        for k, (t, sc) in enumerate(zip(tickets, scs)):
            assert srv.wait(t) == 0
            _check(srv.read(t, sc.width, sc.height, sc.color_format), want[k], k)
        st = srv.stats()
        assert st["completed"] == len(reqs) and st["submitted"] == len(reqs)
        assert 0 < st["p50_ms"] <= st["p99_ms"] <= st["max_ms"]
        if not plain:
            assert st["batches"] <= len(reqs)
    finally:
        srv.destroy()
        for m in meshes:
            m.free()


def test_server_budget_admission(built_lib):
    """A budget that holds about two requests: admission waits for results to
    be released, and every result still equals the request rendered alone."""
    import softrender as sr
    from softrender import _abi as A
    scs, meshes, reqs = _requests(n=6, seed=4)
    want = _alone(scs)
    biggest = max(sc.width * sc.height * 28 + sc.n_tris * 96 + sc.n_verts * 64 + 65536 for sc in scs)
    srv = sr.Server(hbm_budget=2 * biggest, max_inflight=2, max_batch=4)
    try:
        tickets = [srv.submit(r)[1] for r in reqs]
        for k, (t, sc) in enumerate(zip(tickets, scs)):
            assert srv.wait(t) == 0
            _check(srv.read(t, sc.width, sc.height, sc.color_format), want[k], k)
        assert srv.stats()["peak_bytes"] <= 2 * biggest
        # a request larger than the whole budget is refused
        big = sr.Server.request(reqs[0].draw, scs[0].uniforms, 4000, 4000, A.SR_COLOR_RGBA8, scs[0].clear_bytes())
        st, _ = srv.submit(big)
        assert st == A.SR_EBUDGET
    finally:
        srv.destroy()
        for m in meshes:
            m.free()


def test_server_refuses_ineligible_request_alone(built_lib):
    """A request sr_batch_render would refuse (a zero semantic tile width, an
    unknown cull or texture edge mode) is refused when it is submitted, so it
    cannot fail the batch it would have been folded into; the requests
    around it are served and equal their renders alone."""
    import softrender as sr
    from softrender import _abi as A
    scs, meshes, reqs = _requests(n=8, seed=23)
    want = _alone(scs)
    srv = sr.Server(max_inflight=1, max_batch=8)
    try:
        tickets = []
        for k, r in enumerate(reqs):
            if k == 4:
                for field, val in (("tile_w", 0), ("cull", 9), ("tex_edge", 7)):
                    bad = A.SrRequest.from_buffer_copy(reqs[0])
                    setattr(bad.draw, field, val)
                    st, _ = srv.submit(bad)
                    assert st == A.SR_EINVAL, field
            st, t = srv.submit(r)
            assert st == 0
            tickets.append(t)
        for k, (t, sc) in enumerate(zip(tickets, scs)):
            assert srv.wait(t) == 0
            _check(srv.read(t, sc.width, sc.height, sc.color_format), want[k], k)
        assert srv.stats()["submitted"] == len(reqs)
    finally:
        srv.destroy()
        for m in meshes:
            m.free()
