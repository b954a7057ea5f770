"""Host-side I/O (softrender.io): OBJ loading with fan triangulation, PNG
write / read round trip.  No GPU needed."""
import numpy as np

from softrender import io as sio

OBJ = """# a unit quad and a pentagon
v 0 0 0
v 1 0 0
v 1 1 0
v 0 1 0
v 2 0 0
vt 0 0
vt 1 0
vt 1 1
vt 0 1
vn 0 0 1
f 1/1/1 2/2/1 3/3/1 4/4/1
f 2/2/1 5/1/1 3/3/1
f -1/-1/1 -2/-2/1 -5/-4/1
"""


def test_obj_fan_triangulation_and_corners():
    pos, nrm, uv, idx = sio.load_obj(OBJ)
    # quad -> 2 triangles, triangle -> 1, relative-index triangle -> 1
    assert idx.shape == (12,)
    assert idx[:6].tolist() == [0, 1, 2, 0, 2, 3]
    assert pos.shape[1] == 3 and nrm.shape[1] == 3 and uv.shape[1] == 2
    assert (nrm == np.array([0, 0, 1], np.float32)).all()
    # every index points at a vertex whose position is the referenced v
    assert np.array_equal(pos[idx[6:9]], np.array([[1, 0, 0], [2, 0, 0], [1, 1, 0]], np.float32))
    assert idx.max() < pos.shape[0]


def test_png_round_trip(tmp_path):
    rng = np.random.default_rng(0)
    img = rng.integers(0, 2 ** 32, (37, 53), dtype=np.uint64).astype(np.uint32)
    p = tmp_path / "x.png"
    sio.save_png(str(p), img)
    back = sio.load_png(str(p))
    assert back.dtype == np.uint32 and np.array_equal(back, img)


def _reference_asset(rel):
    """A file of the reference checkout named by SOFTRENDER_REFERENCE; None
    when that variable is unset or the file is absent."""
    import os
    base = os.environ.get("SOFTRENDER_REFERENCE")
    if not base:
        return None
    p = os.path.join(base, rel)
    return p if os.path.exists(p) else None


def test_obj_reference_suzanne(oracle_mod):
    """The reference example's mesh (examples/assets/suzanne.obj, loaded by
    tobj in examples/suzanne.rs:24-47): 468 quads and 32 triangles become 968
    triangles; every corner carries the position and normal its face names;
    the mesh renders through the oracle with the example's shading."""
    import math
    import pytest
    from softrender import _abi as A
    from softrender import scenes
    path = _reference_asset("examples/assets/suzanne.obj")
    if path is None:
        pytest.skip("SOFTRENDER_REFERENCE does not name a reference checkout")
    text = open(path).read()
    pos, nrm, uv, idx = sio.load_obj(path)
    assert idx.shape == (3 * 968,) and idx.max() < pos.shape[0]
    assert nrm is not None and uv is not None and nrm.shape == pos.shape
    # an independent reading of the corners, face by face, fan-triangulated
    v = [tuple(map(float, l.split()[1:4])) for l in text.splitlines() if l.startswith("v ")]
    vn = [tuple(map(float, l.split()[1:4])) for l in text.splitlines() if l.startswith("vn ")]
    want_p, want_n = [], []
    for l in text.splitlines():
        if l.startswith("f "):
            c = [tuple(int(x) for x in tok.split("/")) for tok in l.split()[1:]]
            for i in range(1, len(c) - 1):
                for k in (c[0], c[i], c[i + 1]):
                    want_p.append(v[k[0] - 1])
                    want_n.append(vn[k[2] - 1])
    assert np.array_equal(pos[idx], np.asarray(want_p, np.float32))
    assert np.array_equal(nrm[idx], np.asarray(want_n, np.float32))
    # Blinn-Phong with one directional light, camera at distance 3 (examples/suzanne.rs)
    W = H = 96
    cam = (0.0, 0.0, 3.0)
    u = scenes.make_uniforms(view=scenes.look_at_rh(cam, (0, 0, 0), (0, 1, 0)),
                             projection=scenes.perspective(1.0, math.radians(60.0), 0.1, 100.0), camera=cam)
    sc = scenes.Scene(planes=scenes._planes(pos, nrm), indices=idx, width=W, height=H,
                      color_format=A.SR_COLOR_RGBA8, vs="mvp_pos_nrm", fs="blinn_phong_dir", uniforms=u,
                      tile=(32, 32))
    fb, st, status = oracle_mod.render(sc)
    assert status == 0 and st["fragments"] > 1000
