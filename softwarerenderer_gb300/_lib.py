"""ctypes binding of libswr_gb300.so (the C ABI declared in include/swr_gb300.h).

The library is built in-tree by softwarerenderer_gb300.build; importing this module
without it raises, so no caller can silently fall back to a CPU path.
"""
import ctypes
import os

from .abi import SwrUniforms

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libswr_gb300.so")

SWR_OK, SWR_EINVAL, SWR_ENOMEM, SWR_EOVERFLOW, SWR_ECUDA, SWR_EINDEX = range(6)


class SwrStats(ctypes.Structure):
    _fields_ = [("fragments", ctypes.c_uint64), ("primitives", ctypes.c_uint64),
                ("bin_pairs", ctypes.c_uint64), ("clip_polygons", ctypes.c_uint32),
                ("flags", ctypes.c_uint32), ("launches", ctypes.c_uint64),
                ("passes", ctypes.c_uint64)]


class SwrError(RuntimeError):
    def __init__(self, code, what):
        super().__init__(f"{what}: {status_string(code)} ({code})")
        self.code = code


_lib = None


def lib():
    """The loaded CUDA library; raises if it has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"CUDA library missing: {LIB_PATH} (run softwarerenderer_gb300.build)")
        L = ctypes.CDLL(LIB_PATH)
        vp = ctypes.c_void_p
        i, u64, f = ctypes.c_int, ctypes.c_uint64, ctypes.c_float
        sig = {
            "swr_create": [ctypes.POINTER(vp)],
            "swr_destroy": [vp],
            "swr_set_viewport": [vp, i, i, i, i],
            "swr_set_depth_range": [vp, f, f],
            "swr_set_cull_mode": [vp, i],
            "swr_set_vertex_shader": [vp, i],
            "swr_set_vertex_attrib_pointer": [vp, i, i, vp, u64],
            "swr_draw_elements": [vp, i, u64, vp, vp],
            "swr_set_raster_mode": [vp, i],
            "swr_set_scissor_rect": [vp, i, i, i, i],
            "swr_set_pixel_shader": [vp, i],
            "swr_set_uniforms": [vp, ctypes.POINTER(SwrUniforms)],
            "swr_draw_list": [vp, i, vp, u64, vp, u64, vp],
            "swr_finish": [vp, vp, ctypes.POINTER(SwrStats)],
            "swr_set_tile_size": [vp, i],
            "swr_set_profiling": [vp, i],
            "swr_stage_times": [vp, ctypes.POINTER(ctypes.c_float)],
        }
        for name, args in sig.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = ctypes.c_int
        L.swr_status_string.argtypes = [ctypes.c_int]
        L.swr_status_string.restype = ctypes.c_char_p
        _lib = L
    return _lib


def status_string(code):
    try:
        return lib().swr_status_string(code).decode()
    except Exception:  # pragma: no cover - library absent
        return "status"


def check(code, what):
    if code != SWR_OK:
        raise SwrError(code, what)
    return code
