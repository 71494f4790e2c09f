"""Headless presentation: write a render target (device tensor or host array) to a PPM or
PNG file through swr_write_image.

    save_image("frame.png", target.color)                 # RGBA8 shaders (R in the low byte)
    save_image("box.ppm", target.color, fmt=XRGB8)        # the Box example's 0x00RRGGBB
    save_image("diff.png", renderer.color[0])             # RGBA32F, clamped to [0, 1]
"""
import ctypes
import os

import numpy as np

from . import _lib

RGBA8, XRGB8, RGBA32F = 0, 1, 2


def save_image(path, pixels, fmt=None):
    """pixels: (H, W) uint32/int32 (RGBA8 unless fmt says XRGB8) or (H, W, 4) float32,
    as a numpy array or a (CUDA or CPU) torch tensor, row-contiguous."""
    L = _lib.lib()
    L.swr_write_image.argtypes = [ctypes.c_char_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int]
    L.swr_write_image.restype = ctypes.c_int
    keep = pixels
    if hasattr(pixels, "data_ptr"):  # torch tensor
        if not pixels.is_contiguous():
            raise ValueError("pixels must be contiguous")
        ptr, shape, is_float = pixels.data_ptr(), tuple(pixels.shape), pixels.is_floating_point()
    else:
        keep = np.ascontiguousarray(pixels)
        ptr, shape, is_float = keep.ctypes.data, keep.shape, keep.dtype.kind == "f"
    if is_float:
        if len(shape) != 3 or shape[2] != 4:
            raise ValueError("float pixels must be (H, W, 4)")
        fmt = RGBA32F
    elif len(shape) != 2:
        raise ValueError("packed pixels must be (H, W)")
    elif fmt is None:
        fmt = RGBA8
    _lib.check(L.swr_write_image(os.fsencode(path), ptr, shape[1], shape[0], int(fmt)), "swr_write_image")
    del keep
    return path


def read_image(path):
    """(H, W, 3) uint8 of a file written by save_image (test helper; binary PPM or the
    stored-deflate PNG the writer produces, decoded with zlib)."""
    import struct
    import zlib
    data = open(path, "rb").read()
    if data[:2] == b"P6":
        parts = data.split(b"\n", 3)
        w, h = (int(x) for x in parts[1].split())
        return np.frombuffer(parts[3], np.uint8).reshape(h, w, 3)
    assert data[:8] == b"\x89PNG\r\n\x1a\n"
    off, idat, w, h = 8, b"", 0, 0
    while off < len(data):
        n, typ = struct.unpack(">I4s", data[off:off + 8])
        body = data[off + 8:off + 8 + n]
        if zlib.crc32(typ + body) != struct.unpack(">I", data[off + 8 + n:off + 12 + n])[0]:
            raise ValueError("bad CRC")
        if typ == b"IHDR":
            w, h = struct.unpack(">II", body[:8])
        elif typ == b"IDAT":
            idat += body
        off += 12 + n
    raw = np.frombuffer(zlib.decompress(idat), np.uint8).reshape(h, 1 + 3 * w)
    assert np.all(raw[:, 0] == 0)
    return raw[:, 1:].reshape(h, w, 3)
