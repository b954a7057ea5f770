"""The sign tests that skip pixels unevaluated are sound.

segment_cleared (the extension pass of unsafe primitives) and rect_cleared
(bins of the ordered path a large primitive cannot touch) must never declare
cleared a rectangle holding a pixel the reference's coverage test covers.
tests/rect_clear_check.cu calls the same header functions the kernels use,
compiled by nvcc as host code, on random, sliver, sub-pixel and
far-from-origin triangles, and evaluates every pixel of each cleared
rectangle in f32 without contraction.  Needs nvcc, no GPU."""
import os
import re
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc")


@pytest.fixture(scope="module")
def checker(tmp_path_factory):
    if not (os.path.exists(NVCC) or shutil.which("nvcc")):
        pytest.skip("nvcc not available")
    nvcc = NVCC if os.path.exists(NVCC) else shutil.which("nvcc")
    exe = str(tmp_path_factory.mktemp("rect_clear") / "check")
    subprocess.check_call([nvcc, "-std=c++17", "-O2", "-fmad=false", "-gencode", "arch=compute_103a,code=sm_103a",
                           "-Xcompiler", "-ffp-contract=off,-fno-fast-math",
                           "-I", os.path.join(ROOT, "include"), "-I", os.path.join(ROOT, "rust-softrender_gb300", "csrc"),
                           os.path.join(HERE, "rect_clear_check.cu"), "-o", exe])
    return exe


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_cleared_rectangles_hold_no_covered_pixel(checker, seed):
    out = subprocess.run([checker, "200000", str(seed)], capture_output=True, text=True)
    f = {k: int(v) for k, v in re.findall(r"(\w+)=(\d+)", out.stdout)}
    assert out.returncode == 0 and f["violations"] == 0, out.stdout
    # the test is not vacuous: many rectangles and segments were cleared
    assert f["cleared"] > 100000 and f["seg_cleared"] > 10000, out.stdout
