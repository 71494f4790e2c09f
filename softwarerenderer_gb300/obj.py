"""OBJ ingestion through the C-ABI (swr_obj_*): the reference examples' ObjData loader
(ObjData::loadFromFile + toVertexArray, src/examples/ObjData.cpp:46-199).

    vdata, idata = load_obj("mesh.obj")          # (N, 8) float32, (3T,) int32 on the host
    v, i = to_device(vdata, idata)               # torch CUDA tensors for drawElements
"""
import ctypes
import os

import numpy as np

from . import _lib


def _bind(L):
    if getattr(L, "_swr_obj_bound", False):
        return
    vp = ctypes.c_void_p
    L.swr_obj_parse.argtypes = [ctypes.c_char_p, ctypes.c_uint64, ctypes.POINTER(vp)]
    L.swr_obj_load.argtypes = [ctypes.c_char_p, ctypes.POINTER(vp)]
    L.swr_obj_counts.argtypes = [vp, ctypes.POINTER(ctypes.c_uint64), ctypes.POINTER(ctypes.c_uint64)]
    L.swr_obj_read.argtypes = [vp, vp, vp]
    L.swr_obj_upload.argtypes = [vp, vp, vp, vp]
    L.swr_obj_free.argtypes = [vp]
    for f in ("swr_obj_parse", "swr_obj_load", "swr_obj_counts", "swr_obj_read", "swr_obj_upload", "swr_obj_free"):
        getattr(L, f).restype = ctypes.c_int
    L._swr_obj_bound = True


class ObjMesh:
    """A parsed OBJ file (owns the native swr_obj_mesh)."""

    def __init__(self, source):
        L = _lib.lib()
        _bind(L)
        self.L, self.h = L, ctypes.c_void_p()
        if isinstance(source, (bytes, bytearray)):
            rc = L.swr_obj_parse(bytes(source), len(source), ctypes.byref(self.h))
        else:
            rc = L.swr_obj_load(os.fsencode(source), ctypes.byref(self.h))
        _lib.check(rc, "swr_obj")
        nv, ni = ctypes.c_uint64(), ctypes.c_uint64()
        _lib.check(L.swr_obj_counts(self.h, ctypes.byref(nv), ctypes.byref(ni)), "swr_obj_counts")
        self.n_vertices, self.n_indices = nv.value, ni.value

    def __del__(self):
        if getattr(self, "h", None) and self.h.value:
            self.L.swr_obj_free(self.h)
            self.h = None

    def arrays(self):
        vdata = np.zeros((self.n_vertices, 8), np.float32)
        idata = np.zeros(self.n_indices, np.int32)
        _lib.check(self.L.swr_obj_read(self.h, vdata.ctypes.data, idata.ctypes.data), "swr_obj_read")
        return vdata, idata

    def upload(self):
        """Device tensors (vdata (N, 8) float32, idata (3T,) int32) filled by swr_obj_upload."""
        import torch
        v = torch.empty((self.n_vertices, 8), dtype=torch.float32, device="cuda")
        i = torch.empty(self.n_indices, dtype=torch.int32, device="cuda")
        stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
        _lib.check(self.L.swr_obj_upload(self.h, v.data_ptr() if v.numel() else None,
                                         i.data_ptr() if i.numel() else None, stream), "swr_obj_upload")
        return v, i


def load_obj(source):
    """(vdata (N, 8) float32: position, normal, texcoord; idata (3T,) int32) of an OBJ file
    path or of OBJ text given as bytes."""
    return ObjMesh(source).arrays()
