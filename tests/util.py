"""Comparison helpers shared by the parity tests, and the build of the host
programs that check device helpers on the CPU."""
import os
import shutil
import subprocess

import numpy as np

TESTS = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(TESTS)


def build_host_check(src, out_dir):
    """Compiles tests/<src> (a .cu file that calls __host__ __device__ helpers
    of the library's headers) with nvcc as a host program and returns its path;
    None when nvcc is not available."""
    nvcc = "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        nvcc = shutil.which("nvcc")
    if not nvcc:
        return None
    exe = os.path.join(str(out_dir), os.path.splitext(src)[0])
    subprocess.check_call([nvcc, "-std=c++17", "-O2", "-fmad=false", "-gencode", "arch=compute_103a,code=sm_103a",
                           "-Xcompiler", "-ffp-contract=off,-fno-fast-math",
                           "-I", os.path.join(ROOT, "include"), "-I", os.path.join(ROOT, "rust-softrender_gb300", "csrc"),
                           os.path.join(TESTS, src), "-o", exe])
    return exe


def ulp_diff_f32(a, b):
    """Per-element distance in units in the last place between two f32 arrays
    (NaN == NaN counts as 0; mixed NaN as a huge distance)."""
    a = np.ascontiguousarray(a, dtype=np.float32)
    b = np.ascontiguousarray(b, dtype=np.float32)
    ia = a.view(np.int32).astype(np.int64)
    ib = b.view(np.int32).astype(np.int64)
    ia = np.where(ia < 0, -(ia & 0x7fffffff), ia)
    ib = np.where(ib < 0, -(ib & 0x7fffffff), ib)
    d = np.abs(ia - ib)
    na, nb = np.isnan(a), np.isnan(b)
    d = np.where(na & nb, 0, d)
    d = np.where(na ^ nb, 1 << 40, d)
    return d


def assert_bitexact(name, got, want):
    """Bit for bit, except that for f32 data any NaN matches any NaN: IEEE 754
    leaves the payload of a produced NaN open (the GPU writes the canonical
    NaN, x86 keeps the sign and quiet bit of its default NaN)."""
    if got is None and want is None:
        return
    got = np.asarray(got)
    want = np.asarray(want)
    assert got.shape == want.shape, (name, got.shape, want.shape)
    if got.dtype == np.float32 and want.dtype == np.float32:
        got = np.ascontiguousarray(got)
        want = np.ascontiguousarray(want)
        differ = (got.view(np.uint32) != want.view(np.uint32)) & ~(np.isnan(got) & np.isnan(want))
    else:
        gb = got.view(np.uint8) if got.dtype != np.uint8 else got
        wb = want.view(np.uint8) if want.dtype != np.uint8 else want
        differ = None if np.array_equal(gb, wb) else (got != want)
    if differ is not None and differ.any():
        bad = np.argwhere(differ)
        first = tuple(bad[0]) if len(bad) else None
        raise AssertionError("%s differs at %d positions; first %s got %r want %r" % (
            name, len(bad), first, got[first] if first else None, want[first] if first else None))


def compare_frame(gpu, ref, color_ulps=0):
    """gpu = (color, depth, stencil) from the library, ref = oracle Framebuffer.
    Depth, stencil and RGBA8 colour must match bit for bit; RGBA f32 colour
    within `color_ulps` ULP (0: bit-exact)."""
    color, depth, stencil = gpu
    if ref.color is not None:
        if ref.color.dtype == np.float32 and color_ulps:
            d = ulp_diff_f32(color, ref.color)
            assert d.max() <= color_ulps, "colour differs by %d ULP" % d.max()
        else:
            assert_bitexact("color", color, ref.color)
    if ref.depth is not None:
        assert_bitexact("depth", depth, ref.depth)
    if ref.stencil is not None:
        assert_bitexact("stencil", stencil, ref.stencil)
