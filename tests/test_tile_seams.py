"""Semantic-tile pass ranks: the number of tiles containing a pixel
(seam_count with its division magic, used for the opaque path's per-pixel
keys) and the first such tile (tiles_of, used by the extension pass and the
ordered path) agree with the reference's tile walk (fragment.rs:188-216) for
every tile size 1..65535, every coordinate of frames up to 4097 pixels and a
sample of tile sizes at 32767; the magic division equals floor(p / t).
tests/tile_seam_check.cu, compiled by nvcc as host code.  Needs nvcc, no GPU."""
import re
import subprocess

import pytest

from util import build_host_check


def test_tile_seams_match_the_reference_walk(tmp_path):
    exe = build_host_check("tile_seam_check.cu", tmp_path)
    if exe is None:
        pytest.skip("nvcc not available")
    out = subprocess.run([exe], capture_output=True, text=True)
    f = {k: int(v) for k, v in re.findall(r"(\w+)=(\d+)", out.stdout)}
    assert out.returncode == 0 and f["bad"] == 0, out.stdout
    assert f["checked"] > 500_000_000 and f["magic"] > 2_000_000, out.stdout
