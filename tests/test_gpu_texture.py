"""GPU tests of the mip-mapped texture subsystem: the Box example's anisotropic sampler
(PsTexMip) and the perspective-derivative shader (PsPerspDeriv) against the oracle bit
for bit, and swr_build_mip_chain against the numpy restatement of
Texture::generateMipmaps."""
import ctypes

import numpy as np
import pytest

from softwarerenderer_gb300 import _lib, scenes
from softwarerenderer_gb300.abi import DrawMode, RasterMode

from .parity import describe, diff, gpu_render, oracle_render

pytestmark = pytest.mark.gpu


def _check(port, sc, tile=16):
    ref, rst = oracle_render(port, sc)
    got, gst = gpu_render(sc, tile=tile)
    bad = diff(ref, got)
    assert not bad, f"{sc.name}: " + "; ".join(describe(ref, got, k) for k in bad)
    assert gst["fragments"] == rst["fragments"]
    return rst


@pytest.mark.parametrize("frame", range(16))
def test_box_example_frames(gpu_lib, port, frame):
    st = _check(port, scenes.box_scene(frame))
    assert st["fragments"] > 0


@pytest.mark.parametrize("frame", [0, 5])
def test_box_example_tile32(gpu_lib, port, frame):
    _check(port, scenes.box_scene(frame), tile=32)


@pytest.mark.parametrize("mode", [RasterMode.Span, RasterMode.Block, RasterMode.Adaptive])
@pytest.mark.parametrize("frame", range(6))
def test_perspective_derivatives(gpu_lib, port, frame, mode):
    _check(port, scenes.deriv_scene(frame, raster=mode))


@pytest.mark.parametrize("w,h", [(256, 256), (512, 128), (37, 5), (1, 64), (1000, 3), (1, 1), (4096, 4096)])
def test_build_mip_chain(gpu_lib, w, h):
    import torch
    L = _lib.lib()
    L.swr_mip_chain_size.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_int),
                                     ctypes.POINTER(ctypes.c_uint64)]
    L.swr_build_mip_chain.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]
    tex = scenes.rgb_texture(w, h, seed=11) | np.uint32(0xAB000000)  # alpha is cleared
    want = scenes.mip_chain(tex)
    lv, n = ctypes.c_int(), ctypes.c_uint64()
    _lib.check(L.swr_mip_chain_size(w, h, ctypes.byref(lv), ctypes.byref(n)), "size")
    assert n.value == want.size
    base = torch.from_numpy(tex.view(np.int32)).cuda()
    chain = torch.full((n.value,), -1, dtype=torch.int32, device="cuda")
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    _lib.check(L.swr_build_mip_chain(base.data_ptr(), w, h, chain.data_ptr(), stream), "build")
    torch.cuda.synchronize()
    assert np.array_equal(chain.cpu().numpy().view(np.uint32), want)


@pytest.mark.parametrize("mode", [DrawMode.Line, DrawMode.Point])
def test_derivative_shaders_reject_points_and_lines(gpu_lib, mode):
    sc = scenes.box_scene(0)
    sc.draw_mode = mode
    sc.indices = sc.indices[:len(sc.indices) // 6 * 6]
    with pytest.raises(_lib.SwrError) as e:
        gpu_render(sc)
    assert e.value.code == _lib.SWR_EINVAL
