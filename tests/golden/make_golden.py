"""Generates the golden frames under tests/golden/ with the CPU oracle.

    python tests/golden/make_golden.py

Each fixture is a small seeded scene (softrender.scenes) rendered by the
oracle (oracle/), the CPU restatement of the reference's rendering path;
the .npz holds the colour, depth and stencil planes and the fragment count.
tests/test_golden.py checks that the oracle still reproduces them (CPU) and
that the GPU library matches them bit for bit (GPU)."""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "rust-softrender_gb300"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

from softrender import _abi as A  # noqa: E402
from softrender import scenes  # noqa: E402


def golden_scenes():
    """name -> Scene; small enough for the oracle to render in well under a second."""
    return {
        "icosphere_blinn_rgba32f_96x72": scenes.icosphere_scene(96, 72, subdiv=3),
        "icosphere_clip_cull_rgba8_80x64": scenes.icosphere_scene(80, 64, subdiv=2, gs_mode=A.SR_GS_CLIP,
                                                                   color_format=A.SR_COLOR_RGBA8,
                                                                   cull=A.SR_CULL_CLOCKWISE, tile=(16, 16)),
        "gridsphere_clip_textured_128x72": scenes.grid_sphere_scene(128, 72, n_lat=16, n_lon=32, tex_size=32),
        "stress_over_stencil_wrap_96": scenes.stress_scene(n_tiny=6000, n_large=24, size=96, wrap=1),
        "stress_over_stencil_sat_64": scenes.stress_scene(n_tiny=3000, n_large=300, size=64, wrap=0),
        "slivers_stencil_64": scenes.sliver_scene(n=300, size=64, stencil=True,
                                                  stencil_test=A.SR_STENCIL_ALWAYS,
                                                  stencil_op=A.SR_STENCIL_INCREMENT),
        "lines_wu_over_90": scenes.lines_scene(n=200, size=90, seed=2, aa_lines=True, blend="over"),
        "lines_clip_bresenham_90": scenes.lines_scene(n=300, size=90, seed=6, gs_mode=A.SR_GS_CLIP, outside=0.5),
        "points_70": scenes.lines_scene(n=800, size=70, seed=7, prim=A.SR_PRIM_POINT),
        "face_normals_96x64": scenes.icosphere_scene(96, 64, subdiv=2, gs_mode=A.SR_GS_NAMED, gs="face_normals",
                                                     fs="constant_color", tile=(32, 32)),
        "vertex_normals_96x64": scenes.icosphere_scene(96, 64, subdiv=2, gs_mode=A.SR_GS_NAMED,
                                                       gs="vertex_normals", fs="constant_color", tile=(32, 32)),
        "icosphere_aces_rgba32f_96x72": scenes.icosphere_scene(96, 72, subdiv=3, fs="aces_lights"),
        "icosphere_clip_aces_rgba8_80x64": scenes.icosphere_scene(80, 64, subdiv=2, gs_mode=A.SR_GS_CLIP,
                                                                  color_format=A.SR_COLOR_RGBA8, fs="aces_lights",
                                                                  cull=A.SR_CULL_COUNTER_CLOCKWISE, tile=(16, 16)),
    }


def render_golden(sc):
    import oracle
    fb, stats, status = oracle.render(sc)
    out = {"fragments": np.array(stats["fragments"], np.uint64), "status": np.array(status, np.int32)}
    if fb.color is not None:
        out["color"] = fb.color
    if fb.depth is not None:
        out["depth"] = fb.depth
    if fb.stencil is not None:
        out["stencil"] = fb.stencil
    return out


def main():
    for name, sc in golden_scenes().items():
        path = os.path.join(HERE, name + ".npz")
        np.savez_compressed(path, **render_golden(sc))
        print(path, os.path.getsize(path))


if __name__ == "__main__":
    main()
