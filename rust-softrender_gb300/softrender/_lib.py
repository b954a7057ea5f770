"""Loads libsoftrender_gb300.so and declares the C ABI of include/sr.h.

There is no CPU fallback: if the library is missing or fails to load, every
entry point of this package raises.
"""
import ctypes as C
import os

from . import _abi as A

PKG_ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB_PATH = os.path.join(PKG_ROOT, "lib", "libsoftrender_gb300.so")

# every function exported by the library, with (restype, argtypes)
SIGNATURES = {
    "sr_pipeline_create": (C.c_int, [C.POINTER(A.SrFbDesc), C.c_void_p, C.c_size_t, C.POINTER(C.c_void_p)]),
    "sr_pipeline_set_uniforms": (C.c_int, [C.c_void_p, C.c_void_p, C.c_size_t]),
    "sr_pipeline_set_stencil": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_int]),
    "sr_pipeline_set_stream": (C.c_int, [C.c_void_p, C.c_void_p]),
    "sr_pipeline_destroy": (C.c_int, [C.c_void_p]),
    "sr_pipeline_set_profiling": (C.c_int, [C.c_void_p, C.c_int]),
    "sr_framebuffer_clear": (C.c_int, [C.c_void_p, C.c_void_p]),
    "sr_framebuffer_read": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "sr_framebuffer_read_async": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "sr_framebuffer_write": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "sr_framebuffer_device_ptrs": (C.c_int, [C.c_void_p, C.POINTER(C.c_void_p), C.POINTER(C.c_void_p),
                                             C.POINTER(C.c_void_p)]),
    "sr_mesh_upload": (C.c_int, [C.POINTER(C.c_void_p), C.c_uint32, C.c_uint32, C.c_void_p, C.c_uint64,
                                 C.POINTER(C.c_void_p)]),
    "sr_mesh_update": (C.c_int, [C.c_void_p, C.POINTER(C.c_void_p), C.c_uint32, C.c_uint32, C.c_void_p,
                                 C.c_uint64, C.c_void_p]),
    "sr_mesh_free": (C.c_int, [C.c_void_p]),
    "sr_mesh_bytes": (C.c_uint64, [C.c_void_p]),
    "sr_texture_upload": (C.c_int, [C.c_void_p, C.c_uint32, C.c_uint32, C.POINTER(C.c_void_p)]),
    "sr_texture_update": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint32, C.c_uint32, C.c_void_p]),
    "sr_texture_free": (C.c_int, [C.c_void_p]),
    "sr_texture_from_framebuffer": (C.c_int, [C.c_void_p, C.c_void_p]),
    "sr_texture_upload_rgba32f": (C.c_int, [C.c_void_p, C.c_uint32, C.c_uint32, C.POINTER(C.c_void_p)]),
    "sr_texture_view_framebuffer": (C.c_int, [C.c_void_p, C.POINTER(C.c_void_p)]),
    "sr_shader_lookup": (C.c_int, [C.c_char_p, C.c_int, C.POINTER(C.c_int)]),
    "sr_draw_init": (None, [C.POINTER(A.SrDraw)]),
    "sr_render": (C.c_int, [C.c_void_p, C.POINTER(A.SrDraw)]),
    "sr_sync": (C.c_int, [C.c_void_p]),
    "sr_get_stats": (C.c_int, [C.c_void_p, C.POINTER(A.SrStats)]),
    "sr_batch_create": (C.c_int, [C.POINTER(C.c_void_p)]),
    "sr_batch_destroy": (C.c_int, [C.c_void_p]),
    "sr_batch_set_stream": (C.c_int, [C.c_void_p, C.c_void_p]),
    "sr_batch_set_options": (C.c_int, [C.c_void_p, C.c_int, C.c_int]),
    "sr_batch_set_config": (C.c_int, [C.c_void_p, C.c_uint32, C.c_uint32, C.c_uint32]),
    "sr_batch_get_config": (C.c_int, [C.c_void_p, C.POINTER(C.c_uint32), C.POINTER(C.c_uint32),
                                      C.POINTER(C.c_uint32)]),
    "sr_batch_render": (C.c_int, [C.c_void_p, C.POINTER(A.SrBatchItem), C.c_uint32]),
    "sr_batch_sync": (C.c_int, [C.c_void_p]),
    "sr_batch_get_stats": (C.c_int, [C.c_void_p, C.POINTER(A.SrStats)]),
    "sr_server_create": (C.c_int, [C.POINTER(A.SrServerConfig), C.POINTER(C.c_void_p)]),
    "sr_server_submit": (C.c_int, [C.c_void_p, C.POINTER(A.SrRequest), C.POINTER(C.c_uint64)]),
    "sr_server_wait": (C.c_int, [C.c_void_p, C.c_uint64, C.c_uint32]),
    "sr_server_read": (C.c_int, [C.c_void_p, C.c_uint64, C.c_void_p, C.c_void_p]),
    "sr_server_release": (C.c_int, [C.c_void_p, C.c_uint64]),
    "sr_server_drain": (C.c_int, [C.c_void_p, C.c_uint32]),
    "sr_server_get_stats": (C.c_int, [C.c_void_p, C.POINTER(A.SrServerStats)]),
    "sr_server_reset_stats": (C.c_int, [C.c_void_p]),
    "sr_server_destroy": (C.c_int, [C.c_void_p]),
    "sr_render_static": (C.c_int, [C.POINTER(A.SrDraw), C.c_void_p, C.c_size_t, C.c_void_p, C.c_uint32, C.c_uint32,
                                   C.c_uint32, C.c_void_p, C.c_uint32, C.c_void_p, C.c_uint32, C.c_uint32,
                                   C.POINTER(A.SrFbDesc), C.c_void_p, C.c_void_p, C.c_void_p]),
    "sr_status_string": (C.c_char_p, [C.c_int]),
    "sr_version": (C.c_char_p, []),
}

_lib = None


class SoftrenderError(RuntimeError):
    def __init__(self, status, what=""):
        self.status = status
        super().__init__("%s failed: %s" % (what, A.STATUS_NAMES.get(status, status)))


def lib():
    """The loaded library (raises OSError when it is not built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise OSError("libsoftrender_gb300.so is not built (%s); run __graft_entry__.build()" % LIB_PATH)
        L = C.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def check(status, what):
    if status != A.SR_OK:
        raise SoftrenderError(status, what)
    return status
