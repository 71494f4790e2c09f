"""ctypes mirrors of the plain-C structures shared by the CUDA library and the CPU oracle.

`SwrUniforms` matches `struct SwrUniforms` in csrc/swr_programs.h byte for byte; the
enums carry the reference's values (DrawMode/CullMode in VertexProcessor.h:42-53,
RasterMode in Rasterizer.h:45-49).
"""
import ctypes
import enum

import numpy as np


class DrawMode(enum.IntEnum):
    """swr::DrawMode (VertexProcessor.h:42-46)."""
    Point = 0
    Line = 1
    Triangle = 2


class CullMode(enum.IntEnum):
    """swr::CullMode (VertexProcessor.h:49-53); the reference's default is CW."""
    None_ = 0
    CCW = 1
    CW = 2


class RasterMode(enum.IntEnum):
    """swr::RasterMode (Rasterizer.h:45-49); the reference's default is Span."""
    Span = 0
    Block = 1
    Adaptive = 2


class VS(enum.IntEnum):
    """Built-in vertex shaders (SwrVsId in csrc/swr_programs.h)."""
    POS_UV = 1
    POS_NRM_UV = 2
    POS_RGB = 3
    POS_RGB_AFFINE = 4
    POS_RGB_UV = 5


class PS(enum.IntEnum):
    """Built-in pixel shaders (SwrPsId in csrc/swr_programs.h)."""
    TEX_NEAREST = 1
    LAMBERT = 2
    VCOLOR = 3
    VCOLOR_AFFINE = 4
    LAMBERT_TEX = 5
    DIFF = 6
    TEX_MIP = 7
    PERSP_DERIV = 8


# (AttribCount, AVarCount, PVarCount) of each vertex shader, and
# (AVarCount, PVarCount, InterpolateZ, InterpolateW, HasDepth, rgba32f) of each pixel shader.
VS_INFO = {VS.POS_UV: (1, 0, 2), VS.POS_NRM_UV: (2, 3, 2), VS.POS_RGB: (1, 0, 3),
           VS.POS_RGB_AFFINE: (1, 3, 0), VS.POS_RGB_UV: (1, 0, 5)}
PS_INFO = {PS.TEX_NEAREST: (0, 2, 1, 1, 1, 0), PS.LAMBERT: (3, 2, 1, 1, 1, 0),
           PS.VCOLOR: (0, 3, 1, 1, 1, 0), PS.VCOLOR_AFFINE: (3, 0, 0, 0, 0, 0),
           PS.LAMBERT_TEX: (3, 2, 1, 1, 1, 0), PS.DIFF: (0, 5, 1, 1, 1, 1),
           PS.TEX_MIP: (0, 2, 0, 1, 0, 0), PS.PERSP_DERIV: (0, 2, 1, 1, 1, 1)}
# Pixel shaders that read the triangle equations (triangles only).
PS_NEEDS_EQUATIONS = {PS.TEX_MIP, PS.PERSP_DERIV}

# Floats per RasterizerVertex (IRasterizer.h:42-53): x, y, z, w, avar[16], pvar[16].
RASTER_VERTEX_FLOATS = 36


class SwrUniforms(ctypes.Structure):
    _fields_ = [
        ("mvp", ctypes.c_float * 16),
        ("light", ctypes.c_float * 4),
        ("tex", ctypes.c_void_p),
        ("tex_w", ctypes.c_int32),
        ("tex_h", ctypes.c_int32),
        ("color", ctypes.c_void_p),
        ("depth", ctypes.c_void_p),
        ("frag_count", ctypes.c_void_p),
        ("winner", ctypes.c_void_p),
        ("width", ctypes.c_int32),
        ("height", ctypes.c_int32),
        ("checker", ctypes.c_int32),
        ("max_aniso", ctypes.c_int32),
    ]


assert ctypes.sizeof(SwrUniforms) == 144


def make_uniforms(mvp, light, checker, width, height, tex_ptr=0, tex_w=0, tex_h=0,
                  color=0, depth=0, frag_count=0, winner=0, max_aniso=0):
    u = SwrUniforms()
    m = np.asarray(mvp, dtype=np.float32).reshape(16)
    for i in range(16):
        u.mvp[i] = float(m[i])
    lt = np.asarray(light, dtype=np.float32).reshape(4)
    for i in range(4):
        u.light[i] = float(lt[i])
    u.tex = tex_ptr or None
    u.tex_w, u.tex_h = int(tex_w), int(tex_h)
    u.color = color or None
    u.depth = depth or None
    u.frag_count = frag_count or None
    u.winner = winner or None
    u.width, u.height = int(width), int(height)
    u.checker = int(checker)
    u.max_aniso = int(max_aniso)
    return u
