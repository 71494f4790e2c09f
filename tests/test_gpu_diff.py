"""GPU tests of differentiable rendering: the batched forward of the differentiable shader
against the oracle (bit-exact, primitive-source map included), and swr_backward against
the oracle's double-precision reference gradient and central finite differences.

Gradient tolerance: relative error (2-norm over the checked parameters) <= 1e-3.  The
finite-difference protocol (h = 1e-3; Richardson extrapolation for positions at level-6
density; well-conditioned vertices for positions) is described in tests/diffcheck.py.
"""
import numpy as np
import pytest

from softwarerenderer_gb300 import _lib, scenes

from .diffcheck import fd, oracle_views, rel_err, sample_params, well_conditioned_vertices

pytestmark = pytest.mark.gpu


def _renderer(P, tile=16, graph=True):
    import torch
    from softwarerenderer_gb300.diff import DiffRenderer
    dr = DiffRenderer(P.indices, P.vertices.shape[0], P.texture.shape[1], P.texture.shape[0], P.mvps,
                      P.width, P.height, cull=P.cull, raster=P.raster, tile=tile, graph=graph)
    v = torch.from_numpy(P.vertices).cuda()
    t = torch.from_numpy(P.texture).cuda()
    tg = torch.from_numpy(P.targets).cuda()
    return dr, v, t, tg


def _gpu_grads(dr, v, t, tg):
    import torch
    img = dr.forward(v, t)
    g = (2.0 * (img - tg)).contiguous()
    gv, gt, _ = dr.backward(v, t, grad_color=g)
    torch.cuda.synchronize()
    return img, g, gv.cpu().numpy(), gt.cpu().numpy()


def _check_forward(port, P, dr, v, t):
    dr.forward(v, t)
    views, images = oracle_views(port, P, with_images=True)
    col, dep, win = dr.color.cpu().numpy(), dr.depth.cpu().numpy(), dr.winner.cpu().numpy()
    src = dr.prim_src.cpu().numpy()
    for k, (view, img) in enumerate(zip(views, images)):
        assert col[k].tobytes() == img["color"].tobytes(), f"view {k}: colour"
        assert dep[k].tobytes() == img["depth"].tobytes(), f"view {k}: depth"
        assert np.array_equal(win[k], img["winner"]), f"view {k}: winner"
        n = view["nprims"]
        assert np.array_equal(src[k][:n], view["prim_src"][:n]), f"view {k}: primitive sources"
    return views


@pytest.fixture(scope="module")
def small(gpu_lib, port):
    P = scenes.diff_problem(n_views=4, level=4, size=256, tex_size=256, clip_views=1)
    return (P,) + _renderer(P)


@pytest.fixture(scope="module")
def full(gpu_lib, port):
    """The differentiable-rendering workload: 16 views of the level-6 icosphere at 512 x 512,
    1024 x 1024 RGBA32F texture."""
    P = scenes.diff_problem()
    dr, v, t, tg = _renderer(P)
    views = _check_forward(port, P, dr, v, t)
    img, g, gv, gt = _gpu_grads(dr, v, t, tg)
    return P, dr, v, t, tg, views, img, g, gv, gt


@pytest.mark.parametrize("tile", [16, 32])
def test_forward_parity_small(port, small, tile):
    P = small[0]
    dr, v, t, _ = _renderer(P, tile=tile)
    _check_forward(port, P, dr, v, t)


def test_forward_parity_full(full):
    pass  # the fixture compared all 16 views with the oracle bit for bit


def _views_with_grad(views, g):
    gn = g.cpu().numpy()
    return [dict(view, grad_color=gn[k], target=None) for k, view in enumerate(views)]


def test_backward_matches_reference_small(port, small):
    P, dr, v, t, tg = small
    views = oracle_views(port, P)
    img, g, gv, gt = _gpu_grads(dr, v, t, tg)
    _, rv, rt = port.diff_eval(P, _views_with_grad(views, g))
    for name, a, b in (("pos", gv[:, :3], rv[:, :3]), ("rgb", gv[:, 3:6], rv[:, 3:6]), ("uv", gv[:, 6:], rv[:, 6:]),
                       ("tex", gt, rt)):
        assert rel_err(a, b) <= 1e-3, (name, rel_err(a, b))


def test_backward_matches_reference_full(port, full):
    P, dr, v, t, tg, views, img, g, gv, gt = full
    _, rv, rt = port.diff_eval(P, _views_with_grad(views, g))
    for name, a, b in (("pos", gv[:, :3], rv[:, :3]), ("rgb", gv[:, 3:6], rv[:, 3:6]), ("uv", gv[:, 6:], rv[:, 6:]),
                       ("tex", gt, rt)):
        assert rel_err(a, b) <= 1e-3, (name, rel_err(a, b))


@pytest.mark.parametrize("group", ["rgb", "uv", "tex"])
def test_fd_attributes_and_texels_full(port, full, group):
    P, dr, v, t, tg, views, img, g, gv, gt = full
    kind, index = sample_params(np.random.default_rng(11), gv, gt, 256, group)
    ana = (gv if group != "tex" else gt).reshape(-1)[index.astype(np.int64)]
    num = fd(port, P, views, kind, index, h=1e-3)
    assert rel_err(ana, num) <= 1e-3, rel_err(ana, num)


def test_fd_positions_full(port, full):
    P, dr, v, t, tg, views, img, g, gv, gt = full
    ok = well_conditioned_vertices(P, views, min_alt=1.0)
    kind, index = sample_params(np.random.default_rng(12), gv, gt, 256, "pos", ok)
    ana = gv.reshape(-1)[index.astype(np.int64)]
    num = fd(port, P, views, kind, index, h=1e-3, richardson=True)
    assert rel_err(ana, num) <= 1e-3, rel_err(ana, num)


def test_fused_loss_matches_explicit(full):
    import torch
    P, dr, v, t, tg, views, img, g, gv, gt = full
    dr.forward(v, t)
    fv, ft, loss = dr.backward(v, t, target=tg)
    torch.cuda.synchronize()
    ref_loss = float(((dr.color.double() - tg.double()) ** 2).sum())
    assert abs(float(loss) - ref_loss) <= 1e-5 * ref_loss
    assert rel_err(fv.cpu().numpy(), gv) <= 1e-5
    assert rel_err(ft.cpu().numpy(), gt) <= 1e-5


def test_autograd_function(small):
    """loss.backward() through RenderFunction equals the explicit backward, and matches
    central differences (h = 1e-3) of the loss through the real forward renderer for
    vertex colours and texels (whose perturbation leaves the visibility unchanged)."""
    import torch
    from softwarerenderer_gb300.diff import render
    P, dr, v0, t0, tg = small
    v = v0.clone().requires_grad_(True)
    t = t0.clone().requires_grad_(True)
    loss = ((render(v, t, dr) - tg) ** 2).sum()
    loss.backward()
    _, _, gv, gt = _gpu_grads(dr, v0, t0, tg)
    assert rel_err(v.grad.cpu().numpy(), gv) <= 1e-5
    assert rel_err(t.grad.cpu().numpy(), gt) <= 1e-5

    def L(vv, tt):
        img = dr.forward(vv, tt)
        return float(((img.double() - tg.double()) ** 2).sum())

    rng = np.random.default_rng(13)
    for group in ("rgb", "tex"):
        kind, index = sample_params(rng, gv, gt, 24, group)
        num, ana = [], []
        for k, i in zip(kind, index.astype(np.int64)):
            base = (v0 if k == 0 else t0).reshape(-1)
            x = float(base[i])
            hi, lo = np.float32(x + 1e-3), np.float32(x - 1e-3)
            vp, tp = v0.clone(), t0.clone()
            (vp if k == 0 else tp).reshape(-1)[i] = float(hi)
            fp = L(vp, tp)
            (vp if k == 0 else tp).reshape(-1)[i] = float(lo)
            fm = L(vp, tp)
            num.append((fp - fm) / (float(hi) - float(lo)))
            ana.append((gv if k == 0 else gt).reshape(-1)[i])
        assert rel_err(ana, num) <= 1e-3, (group, rel_err(ana, num))


def test_backward_rejects_bad_ids(small):
    import torch
    P, dr, v, t, tg = small
    dr.forward(v, t)
    bad = torch.where(dr.winner >= 0, torch.full_like(dr.winner, 1 << 30), dr.winner).contiguous()
    with pytest.raises(_lib.SwrError) as e:
        dr.backward(v, t, target=tg, winner=bad)
    assert e.value.code == _lib.SWR_EINDEX


def test_primitive_source_capacity(small):
    P, dr, v, t, tg = small
    dr.items[1].prim_src_capacity = 8
    try:
        with pytest.raises(_lib.SwrError) as e:
            dr.forward(v, t)
        assert e.value.code == _lib.SWR_EINVAL
    finally:
        dr.items[1].prim_src_capacity = dr.prim_cap
    dr.forward(v, t)
