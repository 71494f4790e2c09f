"""Headless presentation (swr_write_image): PPM and PNG files of the three target formats
decode to the expected 8-bit RGB, on the host (no GPU needed) and, on a GPU, from a device
framebuffer after a draw."""
import numpy as np
import pytest

from softwarerenderer_gb300 import _lib, scenes
from softwarerenderer_gb300.image import RGBA8, XRGB8, read_image, save_image


def _packed(rng, h, w):
    return rng.integers(0, 2 ** 32, (h, w), dtype=np.uint64).astype(np.uint32)


@pytest.mark.parametrize("ext", ["ppm", "png"])
@pytest.mark.parametrize("h,w", [(1, 1), (7, 13), (480, 640), (300, 300)])
def test_rgba8_and_xrgb8(tmp_path, ext, h, w):
    rng = np.random.default_rng(h * 1000 + w)
    px = _packed(rng, h, w)
    save_image(tmp_path / f"a.{ext}", px, RGBA8)
    got = read_image(tmp_path / f"a.{ext}")
    assert np.array_equal(got[..., 0], px & 255) and np.array_equal(got[..., 2], (px >> 16) & 255)
    save_image(tmp_path / f"b.{ext}", px, XRGB8)
    got = read_image(tmp_path / f"b.{ext}")
    assert np.array_equal(got[..., 0], (px >> 16) & 255) and np.array_equal(got[..., 2], px & 255)
    assert np.array_equal(got[..., 1], (px >> 8) & 255)


def test_rgba32f_clamps_and_rounds(tmp_path):
    px = np.array([[[-1.0, 0.0, 0.5, 1.0], [2.0, 1.0 / 255.0, np.nan, 0.0]]], np.float32)
    save_image(tmp_path / "f.png", px)
    got = read_image(tmp_path / "f.png")
    assert got.tolist() == [[[0, 0, 128], [255, 1, 0]]]


def test_rejects_bad_requests(tmp_path):
    with pytest.raises(_lib.SwrError):
        save_image(tmp_path / "x.bmp", np.zeros((2, 2), np.uint32))
    with pytest.raises(ValueError):
        save_image(tmp_path / "x.png", np.zeros((2, 2, 3), np.float32))


@pytest.mark.gpu
def test_device_framebuffer_dump(gpu_lib, tmp_path):
    from softwarerenderer_gb300.device import DeviceScene, DeviceTarget
    sc = scenes.box_scene(1)
    ds, tg = DeviceScene(sc), DeviceTarget(sc)
    ds.draw(tg)
    save_image(tmp_path / "box.png", tg.color, XRGB8)
    host = tg.color.cpu().numpy().view(np.uint32)
    got = read_image(tmp_path / "box.png")
    assert np.array_equal(got[..., 0], (host >> 16) & 255) and np.array_equal(got[..., 2], host & 255)
    assert got.any()
