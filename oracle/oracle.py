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
        ("prim_src", ctypes.c_void_p),
        ("prim_src_cap", ctypes.c_uint64),
    ]


class OracleDiffScene(ctypes.Structure):
    _fields_ = [("vertices", ctypes.c_void_p), ("nverts", ctypes.c_uint64),
                ("indices", ctypes.c_void_p), ("count", ctypes.c_uint64),
                ("texture", ctypes.c_void_p), ("tex_w", ctypes.c_int32), ("tex_h", ctypes.c_int32)]


class OracleDiffView(ctypes.Structure):
    _fields_ = [("mvp", ctypes.c_float * 16), ("viewport", ctypes.c_int32 * 4),
                ("width", ctypes.c_int32), ("height", ctypes.c_int32),
                ("winner", ctypes.c_void_p), ("prim_src", ctypes.c_void_p), ("nprims", ctypes.c_uint64),
                ("grad_color", ctypes.c_void_p), ("target", ctypes.c_void_p)]


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
        if hasattr(lib, "oracle_diff_eval"):
            lib.oracle_diff_eval.argtypes = [ctypes.POINTER(OracleDiffScene), ctypes.POINTER(OracleDiffView),
                                             ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
            lib.oracle_diff_eval.restype = ctypes.c_int
            lib.oracle_diff_fd.argtypes = [ctypes.POINTER(OracleDiffScene), ctypes.POINTER(OracleDiffView),
                                           ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int,
                                           ctypes.c_double, ctypes.c_void_p, ctypes.c_int]
            lib.oracle_diff_fd.restype = ctypes.c_int
        if hasattr(lib, "oracle_ref_obj"):
            lib.oracle_ref_obj.argtypes = [ctypes.c_char_p, ctypes.c_void_p, ctypes.c_uint64, ctypes.c_void_p,
                                           ctypes.c_uint64, ctypes.POINTER(ctypes.c_uint64),
                                           ctypes.POINTER(ctypes.c_uint64)]
            lib.oracle_ref_obj.restype = ctypes.c_int
            lib.oracle_ref_random.argtypes = [ctypes.c_int, ctypes.c_uint64, ctypes.c_void_p]
            lib.oracle_ref_random.restype = None
        if hasattr(lib, "oracle_tex_sample"):
            lib.oracle_tex_sample.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                              ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint64]
            lib.oracle_tex_sample.restype = None
        if hasattr(lib, "oracle_ref_tex_sample"):
            lib.oracle_ref_tex_sample.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                                  ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint64,
                                                  ctypes.c_void_p]
            lib.oracle_ref_tex_sample.restype = ctypes.c_int
        if hasattr(lib, "oracle_log2"):
            lib.oracle_log2.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint64]
            lib.oracle_log2.restype = None
        if hasattr(lib, "oracle_fold_selftest"):
            lib.oracle_fold_selftest.argtypes = [ctypes.c_uint64, ctypes.c_uint64]
            lib.oracle_fold_selftest.restype = ctypes.c_uint64
        _LIBS[which] = Oracle(lib, which)
    return _LIBS[which]


def scenes_chain_size(w, h):
    n = w * h
    while w > 1 or h > 1:
        w, h = max(1, w // 2), max(1, h // 2)
        n += w * h
    return n


def _ptr(a):
    return a.ctypes.data if a is not None else 0


class Oracle:
    def __init__(self, lib, which):
        self.lib = lib
        self.which = which

    def fold(self, v, a, k):
        return self.lib.oracle_fold(v, a, k)

    def ref_obj(self, path):
        """The reference's ObjData::loadFromFile(path).toVertexArray (ref library only)."""
        nv, ni = ctypes.c_uint64(), ctypes.c_uint64()
        self.lib.oracle_ref_obj(os.fsencode(path), None, 0, None, 0, ctypes.byref(nv), ctypes.byref(ni))
        v = np.zeros((nv.value, 8), np.float32)
        i = np.zeros(ni.value, np.int32)
        self.lib.oracle_ref_obj(os.fsencode(path), v.ctypes.data, nv.value, i.ctypes.data, ni.value,
                                ctypes.byref(nv), ctypes.byref(ni))
        return v, i

    def ref_random(self, seed, n):
        """n values of the reference examples' Random(seed).NextDouble() (ref library only)."""
        out = np.zeros(n, np.float64)
        self.lib.oracle_ref_random(int(seed), int(n), out.ctypes.data)
        return out

    def tex_sample(self, texture, q, max_aniso=0):
        """Sampled 0x00RRGGBB colours for records q (n x 6: u, v, dudx, dvdx, dudy, dvdy) of a
        w x h texture.  The port samples the mip chain `texture` with swr_tex_sample
        (texture = scenes.mip_chain of the level-0 image); the reference builds its own chain
        from the level-0 image and samples it with Texture::sample, and then also returns
        that chain."""
        q = np.ascontiguousarray(q, np.float32)
        out = np.zeros(q.shape[0], np.uint32)
        h, w = texture.shape[:2] if texture.ndim == 2 else (None, None)
        if self.which == "ref":
            base = np.ascontiguousarray(texture, np.uint32)
            chain = np.zeros(scenes_chain_size(w, h), np.uint32)
            self.lib.oracle_ref_tex_sample(base.ctypes.data, w, h, max_aniso, q.ctypes.data, out.ctypes.data,
                                           q.shape[0], chain.ctypes.data)
            return out, chain
        raise TypeError("the port samples a chain: use tex_sample_chain")

    def tex_sample_chain(self, chain, w, h, q, max_aniso=0):
        q = np.ascontiguousarray(q, np.float32)
        chain = np.ascontiguousarray(chain, np.uint32)
        out = np.zeros(q.shape[0], np.uint32)
        self.lib.oracle_tex_sample(chain.ctypes.data, w, h, max_aniso, q.ctypes.data, out.ctypes.data, q.shape[0])
        return out

    def log2(self, x):
        """swr_log2 (the texture sampler's level-of-detail logarithm) of a float32 array."""
        x = np.ascontiguousarray(x, dtype=np.float32)
        out = np.empty_like(x)
        self.lib.oracle_log2(x.ctypes.data, out.ctypes.data, x.size)
        return out

    def draw(self, scene, target, threads=0, prim_src=None):
        """Render `scene` into `target` (numpy buffers, modified in place); returns stats.
        `prim_src` (int32 array, port only) receives the source triangle of every primitive."""
        keep = []
        tex = scene.texture
        if tex is not None:
            tex = np.ascontiguousarray(tex)
            keep.append(tex)
        tw, th = scene.texture_wh()
        u = make_uniforms(scene.mvp, scene.light, scene.checker, scene.width, scene.height,
                          tex_ptr=_ptr(tex), tex_w=tw, tex_h=th,
                          color=_ptr(target.color), depth=_ptr(target.depth),
                          frag_count=_ptr(target.frag_count), winner=_ptr(target.winner),
                          max_aniso=scene.max_aniso)
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
        if prim_src is not None:
            assert prim_src.dtype == np.int32 and prim_src.flags.c_contiguous
            d.prim_src = prim_src.ctypes.data
            d.prim_src_cap = int(prim_src.size)
        st = OracleStats()
        rc = self.lib.oracle_draw(ctypes.byref(d), ctypes.byref(st))
        if rc != 0:
            raise ValueError(f"oracle_draw rejected the draw (status {rc})")
        return {"fragments": st.fragments, "outside": st.outside,
                "primitives": st.primitives, "batches": st.batches}

    # --- differentiable rendering reference (port only) -------------------------------

    def _diff_args(self, problem, views):
        """problem: softwarerenderer_gb300.scenes.DiffProblem; views: list of dicts with
        mvp, winner, prim_src, and grad_color and/or target (numpy)."""
        keep = []
        vd = np.ascontiguousarray(problem.vertices, dtype=np.float64)
        td = np.ascontiguousarray(problem.texture, dtype=np.float64)
        idx = np.ascontiguousarray(problem.indices, dtype=np.int32)
        keep += [vd, td, idx]
        sc = OracleDiffScene(vd.ctypes.data, vd.shape[0], idx.ctypes.data, idx.size, td.ctypes.data,
                             td.shape[1], td.shape[0])
        arr = (OracleDiffView * len(views))()
        for k, v in enumerate(views):
            o = arr[k]
            m = np.ascontiguousarray(v["mvp"], dtype=np.float32).reshape(16)
            for i in range(16):
                o.mvp[i] = float(m[i])
            for i in range(4):
                o.viewport[i] = int(problem.viewport[i])
            o.width, o.height = problem.width, problem.height
            w = np.ascontiguousarray(v["winner"], dtype=np.int32)
            ps = np.ascontiguousarray(v["prim_src"], dtype=np.int32)
            keep += [w, ps]
            o.winner, o.prim_src, o.nprims = w.ctypes.data, ps.ctypes.data, ps.size
            for name in ("grad_color", "target"):
                a = v.get(name)
                if a is not None:
                    a = np.ascontiguousarray(a, dtype=np.float32)
                    keep.append(a)
                    setattr(o, name, a.ctypes.data)
        return sc, arr, keep

    def diff_eval(self, problem, views, grads=True):
        """(loss, grad_vertices (V, 8), grad_texture (T, T, 4)) in double."""
        sc, arr, keep = self._diff_args(problem, views)
        loss = ctypes.c_double(0.0)
        gv = np.zeros(problem.vertices.shape, np.float64) if grads else None
        gt = np.zeros(problem.texture.shape, np.float64) if grads else None
        rc = self.lib.oracle_diff_eval(ctypes.byref(sc), arr, len(views), ctypes.addressof(loss),
                                       _ptr(gv), _ptr(gt))
        if rc != 0:
            raise ValueError(f"oracle_diff_eval failed (status {rc})")
        return loss.value, gv, gt

    def diff_fd(self, problem, views, kind, index, h=1e-3, threads=0):
        """Central differences of the fixed-visibility L2 loss for parameters (kind, index):
        kind 0 = vertex-record component (8 * vertex + c), 1 = texel component (4 * texel + c)."""
        sc, arr, keep = self._diff_args(problem, views)
        kind = np.ascontiguousarray(kind, dtype=np.int32)
        index = np.ascontiguousarray(index, dtype=np.uint64)
        out = np.zeros(kind.size, np.float64)
        rc = self.lib.oracle_diff_fd(ctypes.byref(sc), arr, len(views), kind.ctypes.data, index.ctypes.data,
                                     kind.size, float(h), out.ctypes.data, int(threads))
        if rc != 0:
            raise ValueError(f"oracle_diff_fd failed (status {rc})")
        return out
