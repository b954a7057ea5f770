"""ctypes mirrors of the POD types declared in include/sr.h and include/sr_shaders.h."""
import ctypes as C

# sr_status
SR_OK, SR_EINVAL, SR_ENOMEM, SR_EBUDGET, SR_EOVERFLOW, SR_ETIMEOUT, SR_ECUDA, SR_ENAN, \
    SR_ENOTFOUND, SR_EBUSY = range(10)
STATUS_NAMES = {0: "SR_OK", 1: "SR_EINVAL", 2: "SR_ENOMEM", 3: "SR_EBUDGET", 4: "SR_EOVERFLOW",
                5: "SR_ETIMEOUT", 6: "SR_ECUDA", 7: "SR_ENAN", 8: "SR_ENOTFOUND", 9: "SR_EBUSY"}

# sr_color_format
SR_COLOR_NONE, SR_COLOR_RGBA32F, SR_COLOR_RGBA8 = 0, 1, 2
# sr_prim
SR_PRIM_POINT, SR_PRIM_LINE, SR_PRIM_TRIANGLE = 1, 2, 3
# sr_gs_mode
SR_GS_NONE, SR_GS_CLIP, SR_GS_NAMED = 0, 1, 2
SR_REUSE_NONE, SR_REUSE_VERTICES, SR_REUSE_GEOMETRY = 0, 1, 2   # sr_draw.reuse (duplicate())
# limits of sr_render_static (its fixed scratch)
SR_STATIC_MAX_PIXELS, SR_STATIC_MAX_TRIANGLES, SR_STATIC_MAX_VERTICES = 1 << 20, 1 << 16, 1 << 16
# sr_cull
SR_CULL_NONE, SR_CULL_CLOCKWISE, SR_CULL_COUNTER_CLOCKWISE = 0, 1, 2
# sr_stencil_test
(SR_STENCIL_ALWAYS, SR_STENCIL_NEVER, SR_STENCIL_LESS_THAN, SR_STENCIL_GREATER_THAN,
 SR_STENCIL_LESS_THAN_EQ, SR_STENCIL_GREATER_THAN_EQ, SR_STENCIL_EQUAL,
 SR_STENCIL_NOT_EQUAL) = range(8)
# sr_stencil_op
(SR_STENCIL_KEEP, SR_STENCIL_INVERT, SR_STENCIL_ZERO, SR_STENCIL_REPLACE,
 SR_STENCIL_INCREMENT, SR_STENCIL_DECREMENT) = range(6)
# sr_stage
SR_STAGE_VERTEX, SR_STAGE_GEOMETRY, SR_STAGE_FRAGMENT, SR_STAGE_BLEND = range(4)
# sampling
SR_SAMPLE_NEAREST, SR_SAMPLE_BILINEAR = 0, 1
SR_SAMPLE_CLAMP, SR_SAMPLE_WRAP, SR_SAMPLE_BORDER = 0, 1, 2

F32_MIN = -3.4028234663852886e38   # f32::MIN, the cleared depth

_f16 = C.c_float * 16
_f4 = C.c_float * 4


class SrUniforms(C.Structure):
    """sr_uniforms (include/sr_shaders.h); matrices row-major."""
    _fields_ = [
        ("model", _f16), ("mit", _f16), ("view", _f16), ("projection", _f16),
        ("camera", _f4), ("light_dir", _f4), ("light_pos", _f4), ("color", _f4),
        ("intensity", C.c_float), ("shininess", C.c_float), ("ior", C.c_float),
        ("gamma", C.c_float),
        ("light_color", _f4 * 4), ("light_pos4", _f4 * 4), ("light_int4", _f4),
        ("pv", _f16), ("mvp", _f16),
    ]


class SrFbDesc(C.Structure):
    _fields_ = [("width", C.c_uint32), ("height", C.c_uint32), ("color_format", C.c_uint32),
                ("depth", C.c_uint32), ("stencil", C.c_uint32)]


class SrViewport(C.Structure):
    _fields_ = [("x", C.c_float), ("y", C.c_float), ("width", C.c_float),
                ("height", C.c_float), ("near", C.c_float), ("far", C.c_float)]


class SrDraw(C.Structure):
    _fields_ = [
        ("mesh", C.c_void_p), ("prim", C.c_uint32), ("vs", C.c_int32),
        ("gs_mode", C.c_uint32), ("gs", C.c_int32), ("viewport", SrViewport),
        ("cull", C.c_uint32), ("fs", C.c_int32), ("blend", C.c_int32),
        ("aa_lines", C.c_uint32), ("tile_w", C.c_uint32), ("tile_h", C.c_uint32),
        ("stencil_ref", C.c_uint32), ("texture", C.c_void_p),
        ("tex_filter", C.c_uint32), ("tex_edge", C.c_uint32), ("reuse", C.c_uint32),
    ]


class SrBatchItem(C.Structure):
    _fields_ = [("target", C.c_void_p), ("draw", SrDraw), ("clear", C.c_uint32), ("clear_color", C.c_uint8 * 16)]


class SrServerConfig(C.Structure):
    _fields_ = [("hbm_budget", C.c_uint64), ("max_inflight", C.c_uint32), ("max_batch", C.c_uint32),
                ("plain", C.c_uint32)]


class SrRequest(C.Structure):
    _fields_ = [("draw", SrDraw), ("uniforms", C.c_void_p), ("uniforms_size", C.c_size_t),
                ("width", C.c_uint32), ("height", C.c_uint32), ("color_format", C.c_uint32),
                ("clear_color", C.c_uint8 * 16)]


class SrServerStats(C.Structure):
    _fields_ = [("submitted", C.c_uint64), ("completed", C.c_uint64), ("batches", C.c_uint64),
                ("mean_batch", C.c_double), ("p50_ms", C.c_double), ("p99_ms", C.c_double),
                ("mean_ms", C.c_double), ("max_ms", C.c_double), ("throughput_rps", C.c_double),
                ("peak_bytes", C.c_uint64)]


class SrStats(C.Structure):
    _fields_ = [
        ("triangles_in", C.c_uint64), ("triangles_generated", C.c_uint64),
        ("triangles_raster", C.c_uint64), ("unsafe_triangles", C.c_uint64),
        ("bin_entries", C.c_uint64), ("fragments", C.c_uint64),
        ("nan_bbox", C.c_uint32), ("overflow", C.c_uint32),
        ("kernel_launches", C.c_uint32), ("profiled", C.c_uint32), ("stage_ms", C.c_float * 6),
    ]

STAGE_NAMES = ("vertex", "geometry", "setup_bin", "raster", "stencil", "total")
