"""The RGBA8 byte arithmetic the kernels compute in a cheaper form than the
reference's (the device form of the saturating `as u8` cast, c/255 by one
fused operation, the over operator's three quotients from one reciprocal)
equals the reference's form on every input it can see.

tests/byte_ops_check.cpp enumerates the inputs exhaustively on the CPU with
the oracle's flags; the kernels compile the same header, and the GPU parity
tests compare whole blended frames against the oracle on top of this."""
import os
import re
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


def test_byte_ops_exhaustive(tmp_path):
    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    exe = str(tmp_path / "byte_ops_check")
    subprocess.check_call(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fno-fast-math",
                           "-fno-finite-math-only", "-pthread", os.path.join(HERE, "byte_ops_check.cpp"),
                           "-o", exe])
    out = subprocess.run([exe], capture_output=True, text=True, timeout=600)
    fields = {k: int(v) for k, v in re.findall(r"(\w+)=([0-9]+)", out.stdout)}
    assert set(fields) == {"cast_mismatches", "unit_mismatches", "over_mismatches", "word_mismatches"}, out.stdout
    assert out.returncode == 0 and not any(fields.values()), out.stdout
