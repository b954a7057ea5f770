"""Whole-frame parity at the full benchmark sizes.

The GPU renders every benchmark frame in full -- the 5,120-triangle icosphere
at 1024x1024 RGBA f32, the 1,048,576-triangle clipped, textured grid-sphere at
3840x2160 RGBA8, and the 16,777,216-triangle ordering stress frame at
2048x2048 (over-blend, stencil Increment wrapping and saturating) -- and every
pixel row must match, bit for bit, the row digest of the same frame rendered
in full by the oracle (tests/golden/make_fullframe_digests.py; the oracle's
deterministic mode, whose frames equal the reference's 1-thread order:
fragment.rs:188-216 visits every primitive in every semantic tile,
fragment.rs:268-311 in submission order).  The digest file also holds a
digest of each scene's inputs, checked first, so that a scene generated
differently on this machine is reported as such rather than as a raster
difference."""
import os

import numpy as np
import pytest

from softrender import scenes  # noqa: F401  (the generator builds the scenes)

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))


def _gen():
    import importlib.util
    path = os.path.join(HERE, "golden", "make_fullframe_digests.py")
    spec = importlib.util.spec_from_file_location("make_fullframe_digests", path)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


GEN = _gen()
DIGESTS = dict(np.load(GEN.OUT)) if os.path.exists(GEN.OUT) else {}


@pytest.mark.parametrize("name", sorted(GEN.fullframe_scenes().keys()))
def test_full_frame_rows_match_oracle(built_lib, name):
    import softrender as sr
    assert name + "__rows" in DIGESTS, "no stored digests for " + name
    sc = GEN.fullframe_scenes()[name]()
    assert np.array_equal(GEN.input_digest(sc), DIGESTS[name + "__input"]), \
        "the scene's inputs differ from those the digests were made from"
    color, depth, stencil, stats, status = sr.render_scene(sc)
    assert status == int(DIGESTS[name + "__status"])
    got = GEN.row_digests(sc.height, color, depth if sc.depth else None, stencil if sc.stencil else None)
    want = DIGESTS[name + "__rows"]
    bad = np.nonzero(got != want)[0]
    assert bad.size == 0, "%d of %d rows differ, first %s" % (bad.size, sc.height, bad[:10].tolist())
    assert stats["fragments"] == int(DIGESTS[name + "__fragments"])
    if sc.gs_mode != 0:
        assert stats["triangles_generated"] == int(DIGESTS[name + "__generated"])
