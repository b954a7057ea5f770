"""Per-row digests of the benchmark frames, rendered in full by the oracle.

    python tests/golden/make_fullframe_digests.py [--threads N]

The frames are those the benchmark measures, at their full sizes:
  * icosphere_5120tri_1024x1024_rgba32f: 5,120-triangle icosphere, 1024x1024
    RGBA f32 + f32 depth, Blinn-Phong;
  * gridsphere_1M_3840x2160: 1,048,576-triangle clipped, textured, displaced
    grid-sphere at 3840x2160 RGBA8 + f32 depth;
  * stress_16M_2048_wrap / stress_16M_2048_sat: 16,777,216 tiny triangles and
    4,096 large alpha-blended ones at 2048x2048 RGBA8 + f32 depth + u8
    stencil, stencil Increment wrapping / saturating.
Each is rendered by the oracle in its deterministic multi-threaded mode
(equal to the 1-thread order; tests/test_golden.py checks that), and every
pixel row is reduced to a 64-bit digest of its colour, depth and stencil
bytes (any NaN of an f32 plane written as the canonical quiet NaN first,
since IEEE 754 leaves a produced NaN's payload open).  A digest of the scene's
inputs (attribute planes, indices, texture, uniforms and draw state) is kept
beside them, so that a test can tell a differing frame from a differing scene.
The GPU test tests/test_gpu_fullsize.py renders the same frames and compares
every row.  Output: tests/golden/fullframe_digests.npz (a few tens of KB).
"""
import argparse
import hashlib
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "rust-softrender_gb300"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

OUT = os.path.join(HERE, "fullframe_digests.npz")


def fullframe_scenes():
    from softrender import scenes
    return {
        "icosphere_5120tri_1024x1024_rgba32f": lambda: scenes.icosphere_scene(1024, 1024),
        "gridsphere_1M_3840x2160": lambda: scenes.grid_sphere_scene(),
        "stress_16M_2048_wrap": lambda: scenes.stress_scene(wrap=1),
        "stress_16M_2048_sat": lambda: scenes.stress_scene(wrap=0),
    }


def _canon_f32(a):
    a = np.ascontiguousarray(a, dtype=np.float32).copy()
    a.view(np.uint32)[np.isnan(a)] = np.uint32(0x7FC00000)
    return a


def row_digests(height, color, depth, stencil):
    """uint64 digest of each of the `height` pixel rows of the row-major
    planes (any may be None)."""
    parts = []
    for p in (color, depth, stencil):
        if p is None:
            continue
        p = np.asarray(p)
        if p.dtype == np.float32:
            p = _canon_f32(p)
        parts.append(np.ascontiguousarray(p).view(np.uint8).reshape(height, -1))
    rows = np.concatenate(parts, axis=1)
    out = np.empty(rows.shape[0], dtype=np.uint64)
    for y in range(rows.shape[0]):
        out[y] = np.frombuffer(hashlib.blake2b(rows[y].tobytes(), digest_size=8).digest(), dtype=np.uint64)[0]
    return out


def input_digest(sc):
    """Digest of everything the frame depends on."""
    h = hashlib.blake2b(digest_size=16)
    for p in sc.planes:
        h.update(np.ascontiguousarray(p).tobytes())
    h.update(np.ascontiguousarray(sc.indices).tobytes())
    if sc.texture is not None:
        h.update(np.ascontiguousarray(sc.texture).tobytes())
    h.update(bytes(sc.uniforms))
    state = (sc.width, sc.height, sc.color_format, sc.depth, sc.stencil, sc.prim, sc.vs, sc.gs_mode, sc.gs, sc.fs,
             sc.blend, sc.cull, sc.aa_lines, tuple(sc.tile), sc.stencil_ref, sc.stencil_test, sc.stencil_op,
             sc.stencil_wrap, tuple(float(v) for v in sc.viewport), sc.tex_filter, sc.tex_edge,
             tuple(float(c) for c in sc.clear_color))
    h.update(repr(state).encode())
    return np.frombuffer(h.digest(), dtype=np.uint8).copy()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--threads", type=int, default=os.cpu_count() or 1)
    ap.add_argument("--only", default=None, help="one scene name (the others keep their stored digests)")
    args = ap.parse_args()
    import oracle
    out = dict(np.load(OUT)) if os.path.exists(OUT) else {}
    for name, make in fullframe_scenes().items():
        if args.only and name != args.only:
            continue
        sc = make()
        t = time.time()
        fb, stats, status = oracle.render(sc, n_threads=-max(1, args.threads))
        out[name + "__rows"] = row_digests(sc.height, fb.color, fb.depth, fb.stencil)
        out[name + "__input"] = input_digest(sc)
        out[name + "__fragments"] = np.array(stats["fragments"], np.uint64)
        out[name + "__generated"] = np.array(stats["triangles_generated"], np.uint64)
        out[name + "__status"] = np.array(status, np.int32)
        print("%s: %.1f s, %d fragments, status %d" % (name, time.time() - t, stats["fragments"], status), flush=True)
        np.savez_compressed(OUT, **out)
    print(OUT, os.path.getsize(OUT))


if __name__ == "__main__":
    main()
