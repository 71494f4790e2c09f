"""CPU tests of the differentiable-rendering oracle (no GPU).

The oracle's fixed-visibility colour is checked against the forward image of the port
(which is pinned to the reference), its primitive-source map against the identity where
nothing is culled or clipped, and its analytic gradient against central finite
differences (h = 1e-3) of its own loss.
"""
import numpy as np
import pytest

from softwarerenderer_gb300 import scenes
from softwarerenderer_gb300.abi import CullMode

from .diffcheck import fd, oracle_views, rel_err, sample_params, well_conditioned_vertices


@pytest.fixture(scope="module")
def small(port):
    P = scenes.diff_problem(n_views=3, level=4, size=256, tex_size=256, clip_views=1)
    views, images = oracle_views(port, P, with_images=True)
    loss, gv, gt = port.diff_eval(P, views)
    return P, views, images, gv, gt


def test_prim_src_identity_without_cull_or_clip(port):
    P = scenes.diff_problem(n_views=2, level=2, size=64, tex_size=16, cull=CullMode.None_)
    for view in oracle_views(port, P):
        n = len(P.indices) // 3
        assert view["nprims"] == n
        assert np.array_equal(view["prim_src"][:n], np.arange(n, dtype=np.int32))


def test_prim_src_with_cull_and_clip(small):
    P, views, _, _, _ = small
    n = len(P.indices) // 3
    for k, view in enumerate(views):
        src = view["prim_src"][:view["nprims"]]
        assert src.min() >= 0 and src.max() < n
        if k == 0:  # the near plane cuts the sphere: split triangles repeat their source
            assert len(np.unique(src)) < len(src)
        else:
            assert np.all(np.diff(src) > 0)  # culling keeps submission order


def test_recomputed_colour_matches_forward(port, small):
    """The fixed-visibility colour recomputed from the clip-space vertices (double) equals
    the port's forward image (binary32 fold arithmetic) to within 1e-5 per channel."""
    P, views, images, _, _ = small
    for view, img in zip(views, images):
        w = view["winner"]
        cov = w >= 0
        assert cov.sum() > 1000
        one = [dict(view, target=img["color"])]
        loss, _, _ = port.diff_eval(P, one, grads=False)
        assert loss <= 4 * cov.sum() * (1e-5) ** 2, loss


@pytest.mark.parametrize("group", ["rgb", "uv", "tex"])
def test_fd_attributes_and_texels(port, small, group):
    P, views, _, gv, gt = small
    rng = np.random.default_rng({"rgb": 1, "uv": 2, "tex": 3}[group])
    kind, index = sample_params(rng, gv, gt, 256, group)
    ana = (gv if group != "tex" else gt).reshape(-1)[index.astype(np.int64)]
    num = fd(port, P, views, kind, index, h=1e-3)
    assert rel_err(ana, num) <= 1e-3, rel_err(ana, num)


def test_fd_positions_central(port):
    """Level-4 sphere at 512 x 512 (triangles of ~27 px): central differences, h = 1e-3."""
    P = scenes.diff_problem(n_views=2, level=4, size=512, tex_size=256)
    views = oracle_views(port, P)
    _, gv, gt = port.diff_eval(P, views)
    ok = well_conditioned_vertices(P, views, min_alt=2.0)
    kind, index = sample_params(np.random.default_rng(4), gv, gt, 256, "pos", ok)
    num = fd(port, P, views, kind, index, h=1e-3)
    ana = gv.reshape(-1)[index.astype(np.int64)]
    assert rel_err(ana, num) <= 1e-3, rel_err(ana, num)


def test_fd_positions_richardson_level6(port):
    """Level-6 sphere at 512 x 512 (the differentiable-rendering workload's density):
    Richardson-extrapolated central differences at h = 1e-3 and 5e-4."""
    P = scenes.diff_problem(n_views=2, level=6, size=512, tex_size=1024)
    views = oracle_views(port, P)
    _, gv, gt = port.diff_eval(P, views)
    ok = well_conditioned_vertices(P, views, min_alt=1.0)
    kind, index = sample_params(np.random.default_rng(5), gv, gt, 256, "pos", ok)
    num = fd(port, P, views, kind, index, h=1e-3, richardson=True)
    ana = gv.reshape(-1)[index.astype(np.int64)]
    assert rel_err(ana, num) <= 1e-3, rel_err(ana, num)


def test_diff_eval_rejects_bad_ids(port, small):
    P, views, _, _, _ = small
    bad = dict(views[1])
    bad["winner"] = np.where(views[1]["winner"] >= 0, 10 ** 8, -1).astype(np.int32)
    with pytest.raises(ValueError):
        port.diff_eval(P, [bad])
