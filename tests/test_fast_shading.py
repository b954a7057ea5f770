"""The RGBA8 fast shading path (bounded-error powers, exact fallback) of
include/sr_shaders.h reproduces the exact shader's bytes.

tests/fast_shading_check.cpp is compiled with the oracle's flags and run on
the CPU; the same header is what the resolve kernels compile, and the GPU
parity tests compare whole frames against the oracle on top of this."""
import os
import re
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def checker(tmp_path_factory):
    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    exe = str(tmp_path_factory.mktemp("fast_shading") / "check")
    subprocess.check_call(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fno-fast-math",
                           "-fno-finite-math-only", os.path.join(HERE, "fast_shading_check.cpp"), "-o", exe])
    return exe


def _run(exe, n_pow, n_shade, seed):
    out = subprocess.run([exe, str(n_pow), str(n_shade), str(seed)], capture_output=True, text=True)
    fields = dict(re.findall(r"(\w+)=([0-9.]+)", out.stdout))
    return out.returncode, fields, out.stdout


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_fast_shading_matches_exact(checker, seed):
    rc, f, text = _run(checker, 300000, 300000, seed)
    assert rc == 0 and int(f["mismatches"]) == 0, text
    # the fast power stays well inside its stated bound, and so do the
    # squarings for power-of-two exponents
    assert float(f["pow_max_ratio"]) < 0.5, text
    assert float(f["sq_max_ratio"]) < 0.6, text
    # and decides almost every pixel of a random scene (fallback is rare)
    assert int(f["shade_fallbacks"]) < 0.01 * int(f["shade_cases"]), text
    # near a byte boundary most cases fall back, and none is decided wrongly
    assert int(f["near_fallbacks"]) > 0.5 * int(f["near_cases"]), text
