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
