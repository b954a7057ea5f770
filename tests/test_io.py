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
