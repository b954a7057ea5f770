"""The sign tests that skip pixels unevaluated are sound.

segment_cleared (the extension pass of unsafe primitives) and rect_cleared
(bins of the ordered path a large primitive cannot touch) must never declare
cleared a rectangle holding a pixel the reference's coverage test covers.
tests/rect_clear_check.cu calls the same header functions the kernels use,
compiled by nvcc as host code, on random, sliver, sub-pixel and
far-from-origin triangles, and evaluates every pixel of each cleared
rectangle in f32 without contraction.  Needs nvcc, no GPU."""
import re
import subprocess

import pytest

from util import build_host_check


@pytest.fixture(scope="module")
def checker(tmp_path_factory):
    exe = build_host_check("rect_clear_check.cu", tmp_path_factory.mktemp("rect_clear"))
    if exe is None:
        pytest.skip("nvcc not available")
    return exe


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_cleared_rectangles_hold_no_covered_pixel(checker, seed):
    out = subprocess.run([checker, "200000", str(seed)], capture_output=True, text=True)
    f = {k: int(v) for k, v in re.findall(r"(\w+)=(\d+)", out.stdout)}
    assert out.returncode == 0 and f["violations"] == 0, out.stdout
    # the test is not vacuous: many rectangles and segments were cleared
    assert f["cleared"] > 100000 and f["seg_cleared"] > 10000, out.stdout
