"""Schedule of the line / point raster (tiles of one phase run concurrently):
the phases cover every semantic tile once, and any two tiles that can write
a common pixel -- seams, and the pixel beyond the tile that Xiaolin Wu lines
plot -- run in distinct phases in the reference's row-major order, for
frames and tiles from 1 pixel up (tests/lp_phase_check.cu, compiled by nvcc
as host code; needs nvcc, no GPU)."""
import re
import subprocess

import pytest

from util import build_host_check


def test_line_raster_phases(tmp_path):
    exe = build_host_check("lp_phase_check.cu", tmp_path)
    if exe is None:
        pytest.skip("nvcc not available")
    out = subprocess.run([exe], capture_output=True, text=True)
    f = {k: int(v) for k, v in re.findall(r"(\w+)=(\d+)", out.stdout)}
    assert out.returncode == 0 and f["bad"] == 0, out.stdout
    assert f["configs"] > 5000 and f["pairs"] > 300000, out.stdout
