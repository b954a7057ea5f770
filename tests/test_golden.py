"""Golden frames (tests/golden/*.npz, made by tests/golden/make_golden.py
with the oracle): the oracle must still reproduce them (CPU), and the GPU
library must match them bit for bit (GPU)."""
import importlib.util
import os

import numpy as np
import pytest

from util import assert_bitexact

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _gen():
    spec = importlib.util.spec_from_file_location("make_golden", os.path.join(HERE, "make_golden.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


GEN = _gen()
NAMES = sorted(GEN.golden_scenes().keys())


def _load(name):
    return dict(np.load(os.path.join(HERE, name + ".npz")))


def test_every_golden_scene_has_a_fixture():
    for name in NAMES:
        assert os.path.exists(os.path.join(HERE, name + ".npz")), name


@pytest.mark.parametrize("name", NAMES)
def test_oracle_reproduces_golden(oracle_mod, name):
    sc = GEN.golden_scenes()[name]
    want = _load(name)
    got = GEN.render_golden(sc)
    for k in ("color", "depth", "stencil"):
        assert (k in got) == (k in want), k
        if k in want:
            assert_bitexact(k, got[k], want[k])
    assert int(got["fragments"]) == int(want["fragments"])


@pytest.mark.parametrize("name", NAMES)
def test_oracle_phased_threads_equal_one_thread(oracle_mod, name):
    """The oracle's deterministic multi-threaded mode (order-preserving
    geometry, tiles in phases) reproduces the 1-thread frame: the full-frame
    digests of the benchmark scenes are made with it."""
    sc = GEN.golden_scenes()[name]
    want = _load(name)
    fb, stats, status = oracle_mod.render(sc, n_threads=-3)
    for k in ("color", "depth", "stencil"):
        if k in want:
            assert_bitexact(k, getattr(fb, k), want[k])
    assert int(stats["fragments"]) == int(want["fragments"])
    assert status == int(want["status"])


@pytest.mark.gpu
@pytest.mark.parametrize("name", NAMES)
def test_gpu_matches_golden(built_lib, name):
    import softrender as sr
    sc = GEN.golden_scenes()[name]
    want = _load(name)
    color, depth, stencil, stats, status = sr.render_scene(sc)
    if "color" in want:
        assert_bitexact("color", color, want["color"])
    if "depth" in want:
        assert_bitexact("depth", depth, want["depth"])
    if "stencil" in want:
        assert_bitexact("stencil", stencil, want["stencil"])
    assert stats["fragments"] == int(want["fragments"])


@pytest.mark.parametrize("tile", [(1, 1), (2, 3), (3, 2), (7, 5)])
@pytest.mark.parametrize("kind", ["wu_lines", "stencil_blend"])
def test_oracle_phased_threads_small_tiles(oracle_mod, tile, kind):
    """The phased mode on semantic tiles of 1-7 pixels, where seams are
    everywhere: Xiaolin Wu lines (which plot one pixel past their tile) and
    blended triangles with stencil counting, against the 1-thread order."""
    from softrender import scenes
    import softrender._abi as A
    if kind == "wu_lines":
        sc = scenes.lines_scene(n=150, size=40, seed=21, aa_lines=True, blend="over", tile=tile)
    else:
        sc = scenes.sliver_scene(n=300, size=40, seed=22, color_format=A.SR_COLOR_RGBA8, stencil=True,
                                 stencil_test=A.SR_STENCIL_ALWAYS, stencil_op=A.SR_STENCIL_INCREMENT, blend="over", tile=tile)
    want, wstats, wst = oracle_mod.render(sc, n_threads=1)
    got, gstats, gst = oracle_mod.render(sc, n_threads=-4)
    for k in ("color", "depth", "stencil"):
        assert_bitexact(k, getattr(got, k), getattr(want, k))
    assert gstats["fragments"] == wstats["fragments"] and gst == wst


def test_fullframe_digest_inputs_match_scene_generators():
    """The stored full-frame digests (tests/golden/fullframe_digests.npz) were
    made from the scenes the generators build today: a generator change must
    come with regenerated digests."""
    spec = importlib.util.spec_from_file_location("make_fullframe_digests",
                                                  os.path.join(HERE, "make_fullframe_digests.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    stored = dict(np.load(mod.OUT))
    for name, make in mod.fullframe_scenes().items():
        sc = make()
        assert np.array_equal(mod.input_digest(sc), stored[name + "__input"]), name
        assert stored[name + "__rows"].shape[0] == sc.height


def _suzanne():
    spec = importlib.util.spec_from_file_location("make_suzanne_golden", os.path.join(HERE, "make_suzanne_golden.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    z = dict(np.load(mod.OUT))
    return mod.suzanne_scene(z["pos"], z["nrm"], z["idx"]), z


def test_oracle_reproduces_suzanne_golden(oracle_mod):
    """The reference example's mesh (examples/assets/suzanne.obj, loaded as
    examples/suzanne.rs:24-47 does, fixture made by make_suzanne_golden.py)
    rendered with the example's shading: the oracle still gives the stored
    frame."""
    sc, z = _suzanne()
    fb, st, status = oracle_mod.render(sc)
    assert status == 0 and st["fragments"] == int(z["fragments"]) > 1000
    assert_bitexact("color", fb.color, z["color"])
    assert_bitexact("depth", fb.depth, z["depth"])


@pytest.mark.gpu
def test_gpu_renders_suzanne_like_the_oracle(built_lib):
    """The OBJ mesh through sr_render matches the oracle's frame bit for bit."""
    import softrender as sr
    sc, z = _suzanne()
    color, depth, stencil, stats, status = sr.render_scene(sc)
    assert status == 0
    assert_bitexact("color", color, z["color"])
    assert_bitexact("depth", depth, z["depth"])
    assert stats["fragments"] == int(z["fragments"])
