"""Shared helpers of the differentiable-rendering tests.

Finite differences of the fixed-visibility L2 loss are taken by the oracle in double.
Central differences with h = 1e-3 are used for vertex colours, texture coordinates and
texels.  Vertex positions enter through the perspective-correct barycentrics, whose
curvature grows as a triangle's screen size shrinks: a step of h moves a vertex by about
0.15 px at 512 x 512, a sizeable fraction of a 1.7 px triangle of the level-6 sphere and all
of a near-edge-on silhouette sliver.  Position checks therefore sample vertices whose
visible triangles all have a screen-space altitude of at least `min_alt` px, and at
level-6 density cancel the O(h^2) term by Richardson extrapolation of the central
differences at h and h/2.
"""
import numpy as np

from softwarerenderer_gb300 import scenes


def oracle_views(port, P, with_images=False):
    """Forward of every view with the oracle port: view dicts for diff_eval / diff_fd."""
    views, images = [], []
    for v in range(P.n_views):
        sc = P.scene(v)
        tg = scenes.Target(sc)
        ps = np.full(2 * len(P.indices) // 3 + 1024, -1, np.int32)
        st = port.draw(sc, tg, prim_src=ps)
        views.append(dict(mvp=P.mvps[v], winner=tg.winner, prim_src=ps, target=P.targets[v],
                          nprims=int(st["primitives"])))
        images.append(tg.arrays())
    return (views, images) if with_images else views


def rel_err(a, ref):
    a, ref = np.asarray(a, np.float64).reshape(-1), np.asarray(ref, np.float64).reshape(-1)
    return float(np.linalg.norm(a - ref) / max(np.linalg.norm(ref), 1e-300))


def well_conditioned_vertices(P, views, min_alt):
    """Vertices whose visible incident triangles all have screen altitude >= min_alt px."""
    tri = P.indices.reshape(-1, 3)
    ok = np.ones(P.vertices.shape[0], bool)
    pos = np.concatenate([P.vertices[:, :3].astype(np.float64), np.ones((P.vertices.shape[0], 1))], 1)
    for v, view in enumerate(views):
        w = view["winner"]
        vis = np.unique(view["prim_src"][w[w >= 0]])
        ph = pos @ P.mvps[v].reshape(4, 4).astype(np.float64).T
        sx = ph[:, 0] / ph[:, 3] * (P.width / 2) + P.width / 2
        sy = -ph[:, 1] / ph[:, 3] * (P.height / 2) + P.height / 2
        t = tri[vis]
        a = np.stack([sx[t[:, 0]], sy[t[:, 0]]], 1)
        b = np.stack([sx[t[:, 1]], sy[t[:, 1]]], 1)
        c = np.stack([sx[t[:, 2]], sy[t[:, 2]]], 1)
        area2 = np.abs((b[:, 0] - a[:, 0]) * (c[:, 1] - a[:, 1]) - (c[:, 0] - a[:, 0]) * (b[:, 1] - a[:, 1]))
        lmax = np.maximum(np.maximum(np.hypot(*(b - a).T), np.hypot(*(c - b).T)), np.hypot(*(a - c).T))
        ok[t[area2 / np.maximum(lmax, 1e-300) < min_alt].reshape(-1)] = False
        # a vertex behind the camera has no meaningful screen altitude
        ok[np.unique(t.reshape(-1))[ph[np.unique(t.reshape(-1)), 3] <= 0]] = False
    return ok


def sample_params(rng, gv, gt, n, group, vertex_mask=None):
    """(kind, index) of n parameters of `group` (pos, rgb, uv, tex) that some pixel reaches."""
    if group == "tex":
        cand = np.nonzero(np.abs(gt.reshape(-1)) > 0)[0]
        return np.ones(n, np.int32), rng.choice(cand, n, replace=len(cand) < n).astype(np.uint64)
    reach = np.abs(gv).sum(1) > 0
    if vertex_mask is not None:
        reach &= vertex_mask
    cand = np.nonzero(reach)[0]
    vv = rng.choice(cand, n, replace=len(cand) < n)
    comp = {"pos": rng.integers(0, 3, n), "rgb": 3 + rng.integers(0, 3, n), "uv": 6 + rng.integers(0, 2, n)}[group]
    return np.zeros(n, np.int32), (vv * 8 + comp).astype(np.uint64)


def fd(port, P, views, kind, index, h=1e-3, richardson=False):
    f1 = port.diff_fd(P, views, kind, index, h=h)
    if not richardson:
        return f1
    f2 = port.diff_fd(P, views, kind, index, h=h / 2)
    return (4.0 * f2 - f1) / 3.0
