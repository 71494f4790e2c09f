"""Test infrastructure: ctypes front-end of the CPU oracle.

`load("port")` opens the CPU restatement (oracle/_build/liboracle_port.so, built by
`make -C oracle port`); `load("ref")` opens the reference library itself compiled with
oracle/ref_harness.cpp (oracle/_ref/liboracle_ref.so, built only where the reference
sources exist).  Both expose oracle_draw(); `Oracle.draw(scene, target)` renders a
softwarerenderer_gb300.scenes.Scene into a host Target exactly as the reference's
VertexProcessor::drawElements / Rasterizer::draw*List would.

Only tests, the smoke check and bench.py's CPU-baseline leg import this module.
"""
import ctypes
import os
import subprocess

import numpy as np

from softwarerenderer_gb300.abi import SwrUniforms, make_uniforms

HERE = os.path.dirname(os.path.abspath(__file__))
PATHS = {"port": os.path.join(HERE, "_build", "liboracle_port.so"),
         "ref": os.path.join(HERE, "_ref", "liboracle_ref.so")}


class OracleDraw(ctypes.Structure):
    _fields_ = [
        ("vs_id", ctypes.c_int32), ("ps_id", ctypes.c_int32),
        ("draw_mode", ctypes.c_int32), ("cull_mode", ctypes.c_int32),
        ("raster_mode", ctypes.c_int32),
        ("viewport", ctypes.c_int32 * 4),
        ("depth_range", ctypes.c_float * 2),
        ("scissor", ctypes.c_int32 * 4),
        ("attrib_stride", ctypes.c_int32 * 8),
        ("attrib", ctypes.c_void_p * 8),
        ("indices", ctypes.c_void_p),
        ("count", ctypes.c_uint64),
        ("raster_vertices", ctypes.c_void_p),
        ("uniforms", ctypes.POINTER(SwrUniforms)),
        ("threads", ctypes.c_int32),
        ("_pad", ctypes.c_int32),
    ]


class OracleStats(ctypes.Structure):
    _fields_ = [("fragments", ctypes.c_uint64), ("outside", ctypes.c_uint64),
                ("primitives", ctypes.c_uint64), ("batches", ctypes.c_uint64)]


def build(which="port"):
    """Compile the oracle library (`port` anywhere, `ref` only with the reference checkout)."""
    target = {"port": "port", "ref": "ref"}[which]
    subprocess.run(["make", "-s", "-C", HERE, target], check=True)
    return PATHS[which]


_LIBS = {}


def load(which="port"):
    if which not in _LIBS:
        path = PATHS[which]
        if not os.path.exists(path):
            build(which)
        lib = ctypes.CDLL(path)
        lib.oracle_draw.argtypes = [ctypes.POINTER(OracleDraw), ctypes.POINTER(OracleStats)]
        lib.oracle_draw.restype = ctypes.c_int
        lib.oracle_fold.argtypes = [ctypes.c_float, ctypes.c_float, ctypes.c_int]
        lib.oracle_fold.restype = ctypes.c_float
        if hasattr(lib, "oracle_fold_selftest"):
            lib.oracle_fold_selftest.argtypes = [ctypes.c_uint64, ctypes.c_uint64]
            lib.oracle_fold_selftest.restype = ctypes.c_uint64
        _LIBS[which] = Oracle(lib, which)
    return _LIBS[which]


def _ptr(a):
    return a.ctypes.data if a is not None else 0


class Oracle:
    def __init__(self, lib, which):
        self.lib = lib
        self.which = which

    def fold(self, v, a, k):
        return self.lib.oracle_fold(v, a, k)

    def draw(self, scene, target, threads=0):
        """Render `scene` into `target` (numpy buffers, modified in place); returns stats."""
        keep = []
        tex = scene.texture
        if tex is not None:
            tex = np.ascontiguousarray(tex)
            keep.append(tex)
        u = make_uniforms(scene.mvp, scene.light, scene.checker, scene.width, scene.height,
                          tex_ptr=_ptr(tex), tex_w=tex.shape[1] if tex is not None else 0,
                          tex_h=tex.shape[0] if tex is not None else 0,
                          color=_ptr(target.color), depth=_ptr(target.depth),
                          frag_count=_ptr(target.frag_count), winner=_ptr(target.winner))
        d = OracleDraw()
        d.vs_id, d.ps_id = int(scene.vs), int(scene.ps)
        d.draw_mode, d.cull_mode, d.raster_mode = int(scene.draw_mode), int(scene.cull), int(scene.raster)
        for i in range(4):
            d.viewport[i] = int(scene.viewport[i])
            d.scissor[i] = int(scene.scissor[i])
        d.depth_range[0], d.depth_range[1] = float(scene.depth_range[0]), float(scene.depth_range[1])
        for i, (arr, stride) in enumerate(scene.attribs):
            arr = np.ascontiguousarray(arr)
            keep.append(arr)
            d.attrib[i] = arr.ctypes.data
            d.attrib_stride[i] = int(stride)
        idx = np.ascontiguousarray(scene.indices, dtype=np.int32)
        keep.append(idx)
        d.indices = idx.ctypes.data
        d.count = int(idx.shape[0])
        if scene.raster_vertices is not None:
            rv = np.ascontiguousarray(scene.raster_vertices, dtype=np.float32)
            keep.append(rv)
            d.raster_vertices = rv.ctypes.data
        d.uniforms = ctypes.pointer(u)
        d.threads = int(threads)
        st = OracleStats()
        rc = self.lib.oracle_draw(ctypes.byref(d), ctypes.byref(st))
        if rc != 0:
            raise ValueError(f"oracle_draw rejected the draw (status {rc})")
        return {"fragments": st.fragments, "outside": st.outside,
                "primitives": st.primitives, "batches": st.batches}
