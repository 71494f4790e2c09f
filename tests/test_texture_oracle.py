"""CPU tests of the mip-mapped texture subsystem's host pieces: the level-of-detail
logarithm (swr_log2), the mip chain layout, and the oracle's rejection of derivative
shaders on points and lines.  Rendering parity of the Box-example and derivative scenes
against the reference is covered by the golden fixtures (test_oracle_golden)."""
import numpy as np
import pytest

from softwarerenderer_gb300 import scenes
from softwarerenderer_gb300.abi import DrawMode


def test_log2_is_correctly_rounded(port):
    rng = np.random.default_rng(0)
    bits = rng.integers(1, 0x7f800000, 1_000_000, dtype=np.uint32)
    # every binade edge and its neighbours, subnormals included
    edges = (np.arange(1, 255, dtype=np.uint32) << 23)
    bits = np.concatenate([bits, edges, edges - 1, edges + 1, np.arange(1, 4096, dtype=np.uint32)])
    x = bits.view(np.float32)
    got = port.log2(x)
    want = np.log2(x.astype(np.float64)).astype(np.float32)
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))


def test_log2_special_values(port):
    x = np.array([0.0, np.inf, -1.0, np.nan, 1.0, 2.0, 0.5, 1e-6], np.float32)
    got = port.log2(x)
    assert got[0] == -np.inf and got[1] == np.inf and np.isnan(got[2]) and np.isnan(got[3])
    assert got[4] == 0.0 and got[5] == 1.0 and got[6] == -1.0
    assert got[7] == np.float32(np.log2(np.float64(np.float32(1e-6))))


@pytest.mark.parametrize("w,h", [(256, 256), (512, 128), (37, 5), (1, 64), (1000, 3), (1, 1)])
def test_mip_chain_layout(w, h):
    tex = scenes.rgb_texture(w, h, seed=3)
    chain = scenes.mip_chain(tex)
    sizes, ww, hh = [w * h], w, h
    while ww > 1 or hh > 1:
        ww, hh = max(1, ww // 2), max(1, hh // 2)
        sizes.append(ww * hh)
    assert chain.size == sum(sizes)
    assert np.array_equal(chain[:w * h], tex.reshape(-1) & 0xFFFFFF)
    assert chain[-1] <= 0xFFFFFF and np.all(chain >> 24 == 0)


def test_mip_chain_box_filter():
    tex = np.array([[0x000000, 0x040404], [0x080808, 0x0c0c0c]], np.uint32)
    chain = scenes.mip_chain(tex)
    assert chain[-1] == 0x060606  # (0 + 4 + 8 + 12) >> 2 per channel
    odd = np.array([[0x101010, 0x202020, 0x303030]], np.uint32)  # 3 x 1: p01, p11 repeat p00
    ch = scenes.mip_chain(odd)
    assert ch[3] == ((0x10 * 3 + 0x20) >> 2) * 0x010101


@pytest.mark.parametrize("mode", [DrawMode.Line, DrawMode.Point])
def test_derivative_shaders_reject_points_and_lines(port, mode):
    sc = scenes.box_scene(0)
    sc.draw_mode = mode
    sc.indices = sc.indices[:len(sc.indices) // 6 * 6]
    with pytest.raises(ValueError):
        port.draw(sc, scenes.Target(sc))


def _ref_or_skip():
    import os
    from oracle import oracle
    if not os.path.exists(oracle.PATHS["ref"]):
        pytest.skip("reference library not built (needs the reference checkout, SWR_REFERENCE)")
    return oracle.load("ref")


def _footprints(rng, n):
    """Texture coordinates across several wraps and pixel footprints from far below one
    texel to far above the whole texture, isotropic to strongly anisotropic, any sign."""
    q = np.empty((n, 6), np.float32)
    q[:, 0:2] = rng.uniform(-3.0, 3.0, (n, 2))
    mag = np.exp2(rng.uniform(-16.0, 2.0, (n, 4))) * rng.choice([-1.0, 1.0], (n, 4))
    squash = rng.random(n) < 0.3  # one axis far shorter than the other
    mag[squash, 2:4] *= np.exp2(rng.uniform(-8.0, 0.0, (int(squash.sum()), 1)))
    zero = rng.random((n, 4)) < 0.02
    mag[zero] = 0.0
    q[:, 2:6] = mag
    return q


@pytest.mark.parametrize("w,h,aniso", [(256, 256, 0), (512, 128, 16), (37, 5, 3), (64, 64, 1), (1, 32, 0)])
def test_sampler_matches_reference_texture(port, w, h, aniso):
    """swr_tex_sample (the GPU shader's sampler) against the reference's own Texture::sample
    and Texture::generateMipmaps (src/examples/Texture.h:35-293, compiled unmodified over
    memory surfaces): the mip chain and every sampled colour bit for bit."""
    ref = _ref_or_skip()
    rng = np.random.default_rng(w * 7 + h)
    tex = scenes.rgb_texture(w, h, seed=w + h)
    q = _footprints(rng, 200_000)
    want, ref_chain = ref.tex_sample(tex, q, max_aniso=aniso)
    chain = scenes.mip_chain(tex)
    assert np.array_equal(chain, ref_chain)
    got = port.tex_sample_chain(chain, w, h, q, max_aniso=aniso)
    bad = np.nonzero(got != want)[0]
    assert bad.size == 0, (bad.size, q[bad[:3]], got[bad[:3]], want[bad[:3]])
