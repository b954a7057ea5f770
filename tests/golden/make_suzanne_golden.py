"""Golden fixture of the reference example's mesh rendered by the oracle.

    SOFTRENDER_REFERENCE=<reference checkout> python tests/golden/make_suzanne_golden.py

Reads examples/assets/suzanne.obj of the reference checkout (the mesh
examples/suzanne.rs:24-47 loads with tobj), fan-triangulates it with the
package's OBJ loader (rust-softrender_gb300/softrender/io.py), renders it with
the example's shading -- Blinn-Phong with one directional light, camera at
distance 3, 96x96 RGBA8 + f32 depth, 32x32 semantic tiles -- through the
oracle, and stores the loaded mesh (positions, normals, u32 indices) and the
frame in tests/golden/suzanne_96.npz, so that the GPU test can render the
same mesh where the reference checkout is absent.
"""
import math
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "rust-softrender_gb300"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

OUT = os.path.join(HERE, "suzanne_96.npz")
SIZE = 96


def suzanne_scene(pos, nrm, idx):
    from softrender import _abi as A
    from softrender import scenes
    cam = (0.0, 0.0, 3.0)
    u = scenes.make_uniforms(view=scenes.look_at_rh(cam, (0, 0, 0), (0, 1, 0)),
                             projection=scenes.perspective(1.0, math.radians(60.0), 0.1, 100.0), camera=cam)
    return scenes.Scene(planes=scenes._planes(pos, nrm), indices=np.asarray(idx, np.uint32), width=SIZE,
                        height=SIZE, color_format=A.SR_COLOR_RGBA8, vs="mvp_pos_nrm", fs="blinn_phong_dir",
                        uniforms=u, tile=(32, 32), name="suzanne_%d" % SIZE)


def main():
    base = os.environ.get("SOFTRENDER_REFERENCE")
    if not base:
        sys.exit("set SOFTRENDER_REFERENCE to the reference checkout")
    from softrender import io as sio
    import oracle
    pos, nrm, uv, idx = sio.load_obj(os.path.join(base, "examples", "assets", "suzanne.obj"))
    sc = suzanne_scene(pos, nrm, idx)
    fb, st, status = oracle.render(sc)
    assert status == 0
    np.savez_compressed(OUT, pos=np.asarray(pos, np.float32), nrm=np.asarray(nrm, np.float32),
                        idx=np.asarray(idx, np.uint32), color=fb.color, depth=fb.depth,
                        fragments=np.array(st["fragments"], np.uint64))
    print(OUT, os.path.getsize(OUT), st["fragments"])


if __name__ == "__main__":
    main()
