"""Seeded synthetic scenes for the rasterization pipeline.

Every value is produced with +, -, *, / and sqrt only (IEEE correctly rounded in numpy
float64 elementwise ufuncs and in Python floats) and numpy's PCG64 generator, so a scene
is bit-identical on every platform: fixtures generated on one machine check runs on
another.  No trigonometric or exponential functions are used (their last bits may differ
between libm builds); the 60 degree field of view uses cot(30 deg) = sqrt(3) exactly, and
the log-uniform area distribution of the triangle soup is approximated piecewise-linearly
per octave.

Workloads (sizes as named by the benchmark configurations of this project):
  cube_scene        textured 24-vertex cube, 640x480, Span, CullMode.CW, 100 seeded poses
  sphere_scene      icosphere subdivision 7 (163,842 v / 327,680 t), 1920x1080, Block,
                    Lambert, 32 seeded poses of which 3 put the near plane through the mesh
  soup_scene        1,048,576 independent triangles at 3840x2160, Adaptive
  random_scene      small randomized scenes exercising every mode and quirk (tests)
"""
from dataclasses import dataclass, field
from typing import List, Optional, Tuple

import numpy as np

from .abi import (CullMode, DrawMode, PS, PS_INFO, RASTER_VERTEX_FLOATS, RasterMode, VS,
                  VS_INFO)

SQRT3 = 3.0 ** 0.5


@dataclass
class Scene:
    name: str
    vs: VS
    ps: PS
    width: int
    height: int
    draw_mode: DrawMode = DrawMode.Triangle
    cull: CullMode = CullMode.CW
    raster: RasterMode = RasterMode.Span
    viewport: Tuple[int, int, int, int] = (0, 0, 0, 0)
    depth_range: Tuple[float, float] = (0.0, 1.0)
    scissor: Tuple[int, int, int, int] = (0, 0, 0, 0)
    attribs: List[Tuple[np.ndarray, int]] = field(default_factory=list)
    indices: Optional[np.ndarray] = None
    raster_vertices: Optional[np.ndarray] = None  # (n, 36) float32: direct Rasterizer path
    mvp: np.ndarray = field(default_factory=lambda: np.eye(4, dtype=np.float32).reshape(16))
    light: np.ndarray = field(default_factory=lambda: np.array([0, 0, 1, 0.15], np.float32))
    checker: int = 16
    texture: Optional[np.ndarray] = None
    tex_size: Optional[Tuple[int, int]] = None  # (w, h) of level 0 when `texture` is a mip chain
    max_aniso: int = 0                          # mip-mapped sampler's anisotropy limit (0 = 8)

    def texture_wh(self):
        if self.tex_size is not None:
            return int(self.tex_size[0]), int(self.tex_size[1])
        if self.texture is None:
            return 0, 0
        return int(self.texture.shape[1]), int(self.texture.shape[0])

    @property
    def rgba32f(self) -> bool:
        return bool(PS_INFO[self.ps][5])

    @property
    def has_depth(self) -> bool:
        return bool(PS_INFO[self.ps][4])

    @property
    def n_prims_submitted(self) -> int:
        per = {DrawMode.Point: 1, DrawMode.Line: 2, DrawMode.Triangle: 3}[self.draw_mode]
        return int(len(self.indices)) // per

    def vertex_count(self) -> int:
        if self.raster_vertices is not None:
            return int(self.raster_vertices.shape[0])
        return min(a.nbytes // s for a, s in self.attribs)


class Target:
    """Host render target: colour, depth and the two optional per-pixel records."""

    def __init__(self, scene: Scene, clear_color=0, clear_depth=np.inf, aux=True):
        h, w = scene.height, scene.width
        if scene.rgba32f:
            self.color = np.full((h, w, 4), clear_color, dtype=np.float32)
        else:
            self.color = np.full((h, w), clear_color, dtype=np.uint32)
        self.depth = np.full((h, w), clear_depth, dtype=np.float32)
        self.frag_count = np.zeros((h, w), dtype=np.uint32) if aux else None
        self.winner = np.full((h, w), -1, dtype=np.int32) if aux else None

    def arrays(self):
        out = {"color": self.color, "depth": self.depth}
        if self.frag_count is not None:
            out["frag_count"] = self.frag_count
            out["winner"] = self.winner
        return out


# ----------------------------------------------------------------------------
# small exact matrix helpers (Python floats: IEEE double, no FMA)

def _matmul4(a, b):
    return [[sum_exact(a[r][k] * b[k][c] for k in range(4)) for c in range(4)] for r in range(4)]


def sum_exact(it):
    s = 0.0
    for v in it:
        s = s + v
    return s


def perspective(aspect, near, far, cot=SQRT3):
    """Column-vector projection matrix with cot(fovy/2) given (sqrt(3) for 60 degrees)."""
    return [[cot / aspect, 0.0, 0.0, 0.0],
            [0.0, cot, 0.0, 0.0],
            [0.0, 0.0, (far + near) / (near - far), (2.0 * far * near) / (near - far)],
            [0.0, 0.0, -1.0, 0.0]]


def translate(x, y, z):
    return [[1.0, 0.0, 0.0, x], [0.0, 1.0, 0.0, y], [0.0, 0.0, 1.0, z], [0.0, 0.0, 0.0, 1.0]]


def random_rotation(rng):
    """Uniform random rotation from a uniformly sampled unit quaternion (rejection)."""
    while True:
        q = rng.random(4) * 2.0 - 1.0
        n2 = float(q[0] * q[0] + q[1] * q[1] + q[2] * q[2] + q[3] * q[3])
        if 1e-4 < n2 <= 1.0:
            break
    n = n2 ** 0.5
    w, x, y, z = (float(q[0]) / n, float(q[1]) / n, float(q[2]) / n, float(q[3]) / n)
    return [[1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w), 0.0],
            [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w), 0.0],
            [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y), 0.0],
            [0.0, 0.0, 0.0, 1.0]]


def mat_to_f32(m):
    return np.array([m[r][c] for r in range(4) for c in range(4)], dtype=np.float64).astype(np.float32)


def normalized(v):
    n = (v[0] * v[0] + v[1] * v[1] + v[2] * v[2]) ** 0.5
    return [v[0] / n, v[1] / n, v[2] / n]


# ----------------------------------------------------------------------------
# config: textured cube, 640x480, Span

def checker_texture(size=256, square=32):
    y, x = np.mgrid[0:size, 0:size].astype(np.uint32)
    on = ((x // square + y // square) & 1).astype(bool)
    r = np.where(on, x, 40).astype(np.uint32)
    g = np.where(on, y, 40).astype(np.uint32)
    b = np.where(on, 200, 60).astype(np.uint32)
    return (r | (g << 8) | (b << 16) | (np.uint32(255) << 24)).astype(np.uint32)


def cube_mesh():
    """24 vertices {x, y, z, u, v} (4 per face), 36 indices, CCW front faces."""
    faces = [  # (normal axis, sign): corners ordered CCW seen from outside
        ((1, 0, 0), [(1, -1, -1), (1, 1, -1), (1, 1, 1), (1, -1, 1)]),
        ((-1, 0, 0), [(-1, -1, 1), (-1, 1, 1), (-1, 1, -1), (-1, -1, -1)]),
        ((0, 1, 0), [(-1, 1, -1), (-1, 1, 1), (1, 1, 1), (1, 1, -1)]),
        ((0, -1, 0), [(-1, -1, 1), (-1, -1, -1), (1, -1, -1), (1, -1, 1)]),
        ((0, 0, 1), [(-1, -1, 1), (1, -1, 1), (1, 1, 1), (-1, 1, 1)]),
        ((0, 0, -1), [(1, -1, -1), (-1, -1, -1), (-1, 1, -1), (1, 1, -1)]),
    ]
    uvs = [(0.0, 0.0), (1.0, 0.0), (1.0, 1.0), (0.0, 1.0)]
    verts, idx = [], []
    for n, corners in faces:
        base = len(verts)
        a, b, c = np.array(corners[0]), np.array(corners[1]), np.array(corners[2])
        if np.dot(np.cross(b - a, c - a), np.array(n)) < 0:
            corners = corners[::-1]
        for (x, y, z), (u, v) in zip(corners, uvs):
            verts.append((x * 0.5, y * 0.5, z * 0.5, u, v))
        idx += [base, base + 1, base + 2, base, base + 2, base + 3]
    return np.array(verts, dtype=np.float32), np.array(idx, dtype=np.int32)


def cube_scene(frame: int = 0, seed: int = 1) -> Scene:
    rng = np.random.default_rng(seed)
    rots = [random_rotation(rng) for _ in range(frame + 1)]
    model = rots[frame]
    view = translate(0.0, 0.0, -3.0)
    proj = perspective(4.0 / 3.0, 0.1, 10.0)
    mvp = mat_to_f32(_matmul4(proj, _matmul4(view, model)))
    v, i = cube_mesh()
    return Scene(name=f"cube[{frame}]", vs=VS.POS_UV, ps=PS.TEX_NEAREST, width=640, height=480,
                 cull=CullMode.CW, raster=RasterMode.Span, viewport=(0, 0, 640, 480),
                 scissor=(0, 0, 640, 480), attribs=[(v, 20)], indices=i, mvp=mvp,
                 texture=checker_texture())


def rgb_texture(w: int, h: int, seed: int = 7):
    """0x00RRGGBB texels (the SDL surface format of the reference's example texture): a
    checker of seeded colours with per-texel ramps, so every mip level differs."""
    rng = np.random.default_rng(seed)
    y, x = np.mgrid[0:h, 0:w].astype(np.uint32)
    sq = max(2, min(w, h) // 8)
    col = rng.integers(0, 256, (2, 3)).astype(np.uint32)
    on = ((x // sq + y // sq) & 1).astype(bool)
    r = np.where(on, col[0, 0], col[1, 0]) ^ (x & 31)
    g = np.where(on, col[0, 1], col[1, 1]) ^ (y & 31)
    b = np.where(on, col[0, 2], col[1, 2]) ^ ((x + y) & 15)
    return ((r << 16) | (g << 8) | b).astype(np.uint32)


def mip_chain(tex: np.ndarray) -> np.ndarray:
    """Level 0 (alpha cleared) followed by every 2x2 box-filtered level down to 1x1, each
    max(1, w // 2) x max(1, h // 2) (Texture::generateMipmaps, Texture.h:220-293); edge
    texels of odd sizes repeat the top-left texel as the reference does."""
    lv = np.asarray(tex, dtype=np.uint32) & np.uint32(0x00FFFFFF)
    out = [lv.reshape(-1)]
    h, w = lv.shape
    while w > 1 or h > 1:
        nw, nh = max(1, w // 2), max(1, h // 2)
        y, x = np.mgrid[0:nh, 0:nw]
        p00 = lv[2 * y, 2 * x]
        p10 = np.where(2 * x + 1 < w, lv[2 * y, np.minimum(2 * x + 1, w - 1)], p00)
        p01 = np.where(2 * y + 1 < h, lv[np.minimum(2 * y + 1, h - 1), 2 * x], p00)
        p11 = np.where((2 * x + 1 < w) & (2 * y + 1 < h),
                       lv[np.minimum(2 * y + 1, h - 1), np.minimum(2 * x + 1, w - 1)], p00)
        ch = [((p00 >> s) & 255) + ((p10 >> s) & 255) + ((p01 >> s) & 255) + ((p11 >> s) & 255)
              for s in (16, 8, 0)]
        lv = (((ch[0] >> 2) << 16) | ((ch[1] >> 2) << 8) | (ch[2] >> 2)).astype(np.uint32)
        out.append(lv.reshape(-1))
        w, h = nw, nh
    return np.concatenate(out).astype(np.uint32)


BOX_TEXTURES = ((256, 256), (512, 128), (64, 64), (1024, 512))


def box_scene(frame: int = 0, seed: int = 1) -> Scene:
    """The reference's Box example (Box.cpp): the textured cube drawn in Span mode without
    depth test through a mip-mapped anisotropic sampler fed by perspective-correct
    derivatives, 640x480, CullMode CW.  The frame picks a seeded rotation, a camera
    distance in {3, 5, 7, 9} and one of BOX_TEXTURES."""
    rng = np.random.default_rng(seed)
    rots = [random_rotation(rng) for _ in range(frame + 1)]
    d = 3.0 + 2.0 * (frame % 4)
    mvp = mat_to_f32(_matmul4(perspective(4.0 / 3.0, 0.1, 10.0), _matmul4(translate(0.0, 0.0, -d), rots[frame])))
    v, i = cube_mesh()
    tw, th = BOX_TEXTURES[frame % len(BOX_TEXTURES)]
    return Scene(name=f"box[{frame}]", vs=VS.POS_UV, ps=PS.TEX_MIP, width=640, height=480,
                 cull=CullMode.CW, raster=RasterMode.Span, viewport=(0, 0, 640, 480),
                 scissor=(0, 0, 640, 480), attribs=[(v, 20)], indices=i, mvp=mvp,
                 texture=mip_chain(rgb_texture(tw, th, seed=frame)), tex_size=(tw, th),
                 max_aniso=(0, 4, 16, 1)[frame % 4])


def deriv_scene(frame: int = 0, seed: int = 1, raster: RasterMode = RasterMode.Span) -> Scene:
    """The cube with the derivative-writing shader (du/dx, du/dy, dv/dx, dv/dy as RGBA32F,
    depth-tested): PixelData::computePerspectiveDerivatives on every covered pixel."""
    sc = box_scene(frame, seed)
    sc.name = f"deriv[{frame}]"
    sc.ps = PS.PERSP_DERIV
    sc.raster = raster
    sc.texture, sc.tex_size, sc.max_aniso = None, None, 0
    return sc


def icosphere_obj_text(level: int = 3) -> bytes:
    """An OBJ file of the unit icosphere: v, vn (= position), vt (planar), faces v/t/n."""
    p, f = icosphere(level)
    out = ["# icosphere level %d" % level]
    out += ["v %.7g %.7g %.7g" % tuple(x) for x in p]
    out += ["vn %.7g %.7g %.7g" % tuple(x) for x in p]
    out += ["vt %.7g %.7g" % ((x[0] + 1.0) * 0.5, (x[1] + 1.0) * 0.5) for x in p]
    out += ["f " + " ".join("%d/%d/%d" % (k + 1, k + 1, k + 1) for k in tri) for tri in f]
    return ("\n".join(out) + "\n").encode()


def obj_scene(vdata: np.ndarray, idata: np.ndarray, pose: int = 0, width: int = 640, height: int = 480,
              raster: RasterMode = RasterMode.Block) -> Scene:
    """A mesh loaded from OBJ (vertex records {position, normal, texcoord}, 32 B) drawn
    with the Lambert shader: stream 0 reads position + normal, stream 1 the texcoord of
    the same records (offset 24 B, stride 32 B)."""
    rot, d, _ = sphere_poses(2)[pose]
    mvp = mat_to_f32(_matmul4(perspective(width / height, 0.1, 100.0), _matmul4(translate(0.0, 0.0, -d), rot)))
    v = np.ascontiguousarray(vdata, dtype=np.float32).reshape(-1)
    l = normalized([0.3, 0.5, 0.8])
    return Scene(name=f"obj[{pose}]", vs=VS.POS_NRM_UV, ps=PS.LAMBERT, width=width, height=height,
                 cull=CullMode.CW, raster=raster, viewport=(0, 0, width, height), scissor=(0, 0, width, height),
                 attribs=[(v, 32), (v[6:], 32)], indices=np.asarray(idata, dtype=np.int32), mvp=mvp,
                 light=np.array([l[0], l[1], l[2], 0.15], np.float32), checker=8)


# ----------------------------------------------------------------------------
# config: dense icosphere, 1920x1080, Block

_ICO_CACHE = {}


def icosphere(level: int):
    """Unit icosphere by `level` midpoint subdivisions with shared-edge dedup.

    Returns (positions float64 (V,3), faces int64 (F,3)) with CCW outward faces.
    """
    if level in _ICO_CACHE:
        return _ICO_CACHE[level]
    t = (1.0 + 5.0 ** 0.5) / 2.0
    p = np.array([[-1, t, 0], [1, t, 0], [-1, -t, 0], [1, -t, 0], [0, -1, t], [0, 1, t],
                  [0, -1, -t], [0, 1, -t], [t, 0, -1], [t, 0, 1], [-t, 0, -1], [-t, 0, 1]],
                 dtype=np.float64)
    f = np.array([[0, 11, 5], [0, 5, 1], [0, 1, 7], [0, 7, 10], [0, 10, 11], [1, 5, 9],
                  [5, 11, 4], [11, 10, 2], [10, 7, 6], [7, 1, 8], [3, 9, 4], [3, 4, 2],
                  [3, 2, 6], [3, 6, 8], [3, 8, 9], [4, 9, 5], [2, 4, 11], [6, 2, 10],
                  [8, 6, 7], [9, 8, 1]], dtype=np.int64)

    def norm(v):
        n = np.sqrt(v[:, 0] * v[:, 0] + v[:, 1] * v[:, 1] + v[:, 2] * v[:, 2])
        return v / n[:, None]

    p = norm(p)
    # orient faces outward
    a, b, c = p[f[:, 0]], p[f[:, 1]], p[f[:, 2]]
    cr = np.cross(b - a, c - a)
    flip = (cr[:, 0] * a[:, 0] + cr[:, 1] * a[:, 1] + cr[:, 2] * a[:, 2]) < 0
    f[flip] = f[flip][:, ::-1]
    for _ in range(level):
        nv = p.shape[0]
        e = np.concatenate([f[:, [0, 1]], f[:, [1, 2]], f[:, [2, 0]]], axis=0)
        lo, hi = np.minimum(e[:, 0], e[:, 1]), np.maximum(e[:, 0], e[:, 1])
        key = lo * nv + hi
        uniq, inv = np.unique(key, return_inverse=True)
        ulo, uhi = uniq // nv, uniq % nv
        mid = norm((p[ulo] + p[uhi]) * 0.5)
        p = np.concatenate([p, mid], axis=0)
        nf = f.shape[0]
        ab = nv + inv[:nf]
        bc = nv + inv[nf:2 * nf]
        ca = nv + inv[2 * nf:]
        f = np.concatenate([np.stack([f[:, 0], ab, ca], 1), np.stack([f[:, 1], bc, ab], 1),
                            np.stack([f[:, 2], ca, bc], 1), np.stack([ab, bc, ca], 1)], axis=0)
    _ICO_CACHE[level] = (p, f)
    return p, f


def sphere_buffers(level: int = 7):
    p, f = icosphere(level)
    pn = np.concatenate([p, p], axis=1).astype(np.float32)        # pos + normal (24 B)
    uv = np.stack([(p[:, 0] + 1.0) * 0.5, (p[:, 1] + 1.0) * 0.5], 1).astype(np.float32)
    return pn, uv, f.reshape(-1).astype(np.int32)


SPHERE_POSES = 32
SPHERE_NEAR_CLIP_POSES = 3


def sphere_poses(seed: int = 2):
    rng = np.random.default_rng(seed)
    near = set(rng.choice(SPHERE_POSES, SPHERE_NEAR_CLIP_POSES, replace=False).tolist())
    poses = []
    for k in range(SPHERE_POSES):
        rot = random_rotation(rng)
        if k in near:
            # Near the view axis the surface sits at view depth ~ (d - 1) + r^2/2; with
            # d - 1 just under the near distance 0.1 the near plane cuts a disc of radius
            # r = sqrt(2 (0.1 - (d - 1))) < 0.055 out of the middle of the view.
            d = 1.0985 + 0.0013 * float(rng.random())
        else:
            d = 2.2 + 1.8 * float(rng.random())
        poses.append((rot, d, k in near))
    return poses


def sphere_scene(pose: int = 0, level: int = 7, width: int = 1920, height: int = 1080,
                 seed: int = 2, raster: RasterMode = RasterMode.Block) -> Scene:
    rot, d, _ = sphere_poses(seed)[pose]
    proj = perspective(width / height, 0.1, 100.0)
    mvp = mat_to_f32(_matmul4(proj, _matmul4(translate(0.0, 0.0, -d), rot)))
    pn, uv, idx = sphere_buffers(level)
    l = normalized([0.3, 0.5, 0.8])
    return Scene(name=f"sphere{level}[{pose}]", vs=VS.POS_NRM_UV, ps=PS.LAMBERT,
                 width=width, height=height, cull=CullMode.CW, raster=raster,
                 viewport=(0, 0, width, height), scissor=(0, 0, width, height),
                 attribs=[(pn, 24), (uv, 8)], indices=idx, mvp=mvp,
                 light=np.array([l[0], l[1], l[2], 0.15], np.float32), checker=16)


# ----------------------------------------------------------------------------
# config: triangle soup, 3840x2160, Adaptive

def soup_scene(n_tris: int = 1 << 20, width: int = 3840, height: int = 2160,
               seed: int = 3, raster: RasterMode = RasterMode.Adaptive) -> Scene:
    """Independent triangles: centre uniform on screen, area piecewise-log-uniform in
    [0.5, 1e4] px^2, base view depth uniform in [0.05, 200] and per-vertex depth in
    [0.5, 1.5] x base (about a third of the triangles cross the far plane at 100 or the
    near plane at 0.1), random winding, per-vertex RGB."""
    rng = np.random.default_rng(seed)
    n = n_tris
    cx = rng.random(n) * width
    cy = rng.random(n) * height
    # area: octave e uniform in 0..14, linear within the octave; resample above 1e4
    e = rng.integers(0, 15, n)
    fr = rng.random(n)
    area = 0.5 * np.ldexp(1.0, e) * (1.0 + fr)   # power of two scaling is exact
    big = area > 1e4
    area[big] = 8192.0 + (1e4 - 8192.0) * rng.random(int(big.sum()))
    pts = rng.random((n, 3, 2)) * 2.0 - 1.0
    ax, ay = pts[:, 1, 0] - pts[:, 0, 0], pts[:, 1, 1] - pts[:, 0, 1]
    bx, by = pts[:, 2, 0] - pts[:, 0, 0], pts[:, 2, 1] - pts[:, 0, 1]
    a0 = np.abs(ax * by - ay * bx) * 0.5
    a0 = np.maximum(a0, 0.05)
    s = np.sqrt(area / a0)
    sx = cx[:, None] + s[:, None] * pts[:, :, 0]
    sy = cy[:, None] + s[:, None] * pts[:, :, 1]
    flip = rng.random(n) < 0.5
    sx[flip] = sx[flip][:, [0, 2, 1]]
    sy[flip] = sy[flip][:, [0, 2, 1]]
    zb = 0.05 + (200.0 - 0.05) * rng.random(n)
    zv = zb[:, None] * (0.5 + rng.random((n, 3)))
    aspect = width / height
    xn = (sx - width * 0.5) / (width * 0.5)
    yn = -(sy - height * 0.5) / (height * 0.5)
    xv = xn * zv * aspect / SQRT3
    yv = yn * zv / SQRT3
    rgb = rng.random((n, 3, 3))
    verts = np.empty((n, 3, 6), np.float64)
    verts[:, :, 0] = xv
    verts[:, :, 1] = yv
    verts[:, :, 2] = -zv
    verts[:, :, 3:6] = rgb
    verts = verts.reshape(-1, 6).astype(np.float32)
    mvp = mat_to_f32(perspective(aspect, 0.1, 100.0))
    idx = np.arange(3 * n, dtype=np.int32)
    return Scene(name=f"soup{n}", vs=VS.POS_RGB, ps=PS.VCOLOR, width=width, height=height,
                 cull=CullMode.CW, raster=raster, viewport=(0, 0, width, height),
                 scissor=(0, 0, width, height), attribs=[(verts, 24)], indices=idx, mvp=mvp)


# ----------------------------------------------------------------------------
# randomized small scenes for parity tests

_COMPAT = [(VS.POS_UV, PS.TEX_NEAREST), (VS.POS_NRM_UV, PS.LAMBERT),
           (VS.POS_NRM_UV, PS.LAMBERT_TEX), (VS.POS_NRM_UV, PS.TEX_NEAREST),
           (VS.POS_NRM_UV, PS.VCOLOR_AFFINE), (VS.POS_RGB, PS.VCOLOR),
           (VS.POS_RGB, PS.TEX_NEAREST), (VS.POS_RGB_AFFINE, PS.VCOLOR_AFFINE),
           (VS.POS_RGB_UV, PS.DIFF), (VS.POS_RGB_UV, PS.VCOLOR)]


def _snap(rng, a, p_snap):
    if rng.random() < p_snap:
        q = [1.0, 0.5, 0.25][int(rng.integers(0, 3))]
        return np.round(a / q) * q
    return a


def small_texture(rng, rgba32f, size=64):
    if rgba32f:
        return rng.random((size, size, 4)).astype(np.float32)
    return rng.integers(0, 2 ** 32, (size, size), dtype=np.uint64).astype(np.uint32)


def random_scene(seed: int, direct: Optional[bool] = None, draw_mode: Optional[DrawMode] = None,
                 n_prims: Optional[int] = None) -> Scene:
    """A small random scene exercising modes, clipping, culling, scissor and tie quirks."""
    rng = np.random.default_rng(10_000 + seed)
    vs, ps = _COMPAT[int(rng.integers(0, len(_COMPAT)))]
    if draw_mode is None:
        r = rng.random()
        draw_mode = DrawMode.Triangle if r < 0.7 else (DrawMode.Line if r < 0.85 else DrawMode.Point)
    if direct is None:
        direct = rng.random() < 0.3
    w = int(rng.integers(24, 160))
    h = int(rng.integers(24, 160))
    if rng.random() < 0.3:
        w, h = 8 * max(3, w // 8), 8 * max(3, h // 8)
    per = {DrawMode.Point: 1, DrawMode.Line: 2, DrawMode.Triangle: 3}[draw_mode]
    n = n_prims if n_prims is not None else int(rng.integers(1, 200 if draw_mode == DrawMode.Triangle else 120))
    raster = RasterMode(int(rng.integers(0, 3)))
    cull = CullMode(int(rng.integers(0, 3)))
    r = rng.random()
    if r < 0.5:
        scissor = (0, 0, w, h)
    elif r < 0.85:
        sx, sy = int(rng.integers(-5, w // 2)), int(rng.integers(-5, h // 2))
        scissor = (sx, sy, int(rng.integers(1, w)), int(rng.integers(1, h)))
    else:
        scissor = (0, 0, 0, 0)  # the reference Rasterizer's default scissor
    if rng.random() < 0.7:
        viewport = (0, 0, w, h)
    else:
        viewport = (int(rng.integers(-8, 16)), int(rng.integers(-8, 16)),
                    int(rng.integers(8, w + 16)), int(rng.integers(8, h + 16)))
    depth_range = (0.0, 1.0) if rng.random() < 0.8 else (float(np.float32(rng.random() * 0.3)),
                                                           float(np.float32(0.6 + rng.random() * 0.4)))
    na, np_ = VS_INFO[vs][1], VS_INFO[vs][2]
    ps_na, ps_np = PS_INFO[ps][0], PS_INFO[ps][1]
    tex = small_texture(rng, bool(PS_INFO[ps][5])) if ps in (PS.TEX_NEAREST, PS.LAMBERT_TEX, PS.DIFF) else None
    l = normalized([float(rng.random()) - 0.5, float(rng.random()) - 0.5, 1.0])
    light = np.array([l[0], l[1], l[2], 0.2], np.float32)
    nverts = int(max(3, n * per * (0.6 if rng.random() < 0.5 else 1.0)))
    idx = rng.integers(0, nverts, n * per).astype(np.int32)
    if direct:
        rv = np.zeros((nverts, RASTER_VERTEX_FLOATS), np.float32)
        small = rng.random() < 0.5
        span = 12.0 if small else float(max(w, h))
        centers = rng.random((nverts, 2)) * np.array([w + 20, h + 20]) - 10
        if small:
            rv[:, 0:2] = centers + (rng.random((nverts, 2)) - 0.5) * span
        else:
            rv[:, 0:2] = rng.random((nverts, 2)) * np.array([w + 40, h + 40]) - 20
        rv[:, 0:2] = _snap(rng, rv[:, 0:2], 0.3)
        rv[:, 2] = rng.random(nverts)
        rv[:, 3] = 0.5 + 1.5 * rng.random(nverts)
        rv[:, 4:36] = rng.random((nverts, 32))
        return Scene(name=f"rand{seed}d", vs=vs, ps=ps, width=w, height=h, draw_mode=draw_mode,
                     cull=cull, raster=raster, viewport=viewport, depth_range=depth_range,
                     scissor=scissor, indices=idx, raster_vertices=rv, light=light, texture=tex,
                     checker=int(rng.integers(2, 20)))
    # vertex-processor path: random model-space points seen through a perspective camera
    spread = float(rng.choice([0.3, 1.0, 3.0]))
    pos = (rng.random((nverts, 3)) - 0.5) * 2.0 * spread
    pos = _snap(rng, pos, 0.2)
    d = float(rng.choice([1.0, 2.0, 3.0, 5.0]))
    proj = perspective(w / h, 0.1 + 0.4 * float(rng.random()), 4.0 + 6.0 * float(rng.random()))
    mvp = mat_to_f32(_matmul4(proj, _matmul4(translate(0.0, 0.0, -d), random_rotation(rng))))
    if vs == VS.POS_UV:
        v = np.concatenate([pos, rng.random((nverts, 2))], 1).astype(np.float32)
        attribs = [(v, 20)]
    elif vs == VS.POS_NRM_UV:
        nrm = rng.random((nverts, 3)) * 2 - 1
        v = np.concatenate([pos, nrm], 1).astype(np.float32)
        attribs = [(v, 24), (rng.random((nverts, 2)).astype(np.float32), 8)]
    elif vs in (VS.POS_RGB, VS.POS_RGB_AFFINE):
        v = np.concatenate([pos, rng.random((nverts, 3))], 1).astype(np.float32)
        attribs = [(v, 24)]
    else:
        v = np.concatenate([pos, rng.random((nverts, 5))], 1).astype(np.float32)
        attribs = [(v, 32)]
    return Scene(name=f"rand{seed}", vs=vs, ps=ps, width=w, height=h, draw_mode=draw_mode,
                 cull=cull, raster=raster, viewport=viewport, depth_range=depth_range,
                 scissor=scissor, attribs=attribs, indices=idx, mvp=mvp, light=light,
                 texture=tex, checker=int(rng.integers(2, 20)))


def stack_scene(seed: int, n: int, ps: PS = PS.VCOLOR, raster: RasterMode = RasterMode.Block,
                width: int = 48, height: int = 40) -> Scene:
    """A pile of n triangles over a small target: each triangle 3-30 px across, at one of six
    constant depths (so equal depths tie often), either winding, no culling.  Its tiles hold
    hundreds to thousands of bin entries: the heavy-tile path of the tile rasterizer."""
    rng = np.random.default_rng(50_000 + seed)
    c = rng.random((n, 1, 2)) * np.array([width, height])
    size = 3.0 + 27.0 * rng.random((n, 1, 1))
    pts = c + (rng.random((n, 3, 2)) - 0.5) * size
    ndc = np.empty((n, 3, 3), np.float64)
    ndc[:, :, 0] = pts[:, :, 0] / (width * 0.5) - 1.0
    ndc[:, :, 1] = 1.0 - pts[:, :, 1] / (height * 0.5)
    ndc[:, :, 2] = np.array([-0.5, -0.25, 0.0, 0.25, 0.5, 0.75])[rng.integers(0, 6, n)][:, None]
    pos = ndc.reshape(-1, 3)
    nv = 3 * n
    if ps in (PS.LAMBERT, PS.LAMBERT_TEX):
        vs = VS.POS_NRM_UV
        nrm = rng.random((nv, 3)) * 2 - 1
        attribs = [(np.concatenate([pos, nrm], 1).astype(np.float32), 24),
                   (rng.random((nv, 2)).astype(np.float32), 8)]
    else:
        vs = VS.POS_RGB
        attribs = [(np.concatenate([pos, rng.random((nv, 3))], 1).astype(np.float32), 24)]
    tex = small_texture(rng, False) if ps in (PS.TEX_NEAREST, PS.LAMBERT_TEX) else None
    return Scene(name=f"stack{n}s{seed}", vs=vs, ps=ps, width=width, height=height, cull=CullMode.None_,
                 raster=raster, viewport=(0, 0, width, height), scissor=(0, 0, width, height),
                 attribs=attribs, indices=np.arange(nv, dtype=np.int32), light=np.array([0.3, -0.2, 0.93, 0.15], np.float32),
                 texture=tex, checker=5)


# ----------------------------------------------------------------------------
# Benchmark.cpp-shaped scene and spec-driven construction (fixtures, tests, bench)

class SubtractiveRandom:
    """Knuth's subtractive generator (The Art of Computer Programming, vol. 2, 3.6) in the
    form of .NET's System.Random, which the reference's examples/Random.cpp reproduces:
    a 55-entry lagged table seeded from MSEED - |seed|, shuffled four times, then
    x[n] = x[n-55] - x[n-24] mod (2^31 - 1); next_double() = sample / (2^31 - 1)."""

    MBIG = 2147483647
    MSEED = 161803398

    @staticmethod
    def _i32(x: int) -> int:  # 32-bit two's-complement wrap of the C++ int arithmetic
        return (x + 2147483648) % 4294967296 - 2147483648

    def __init__(self, seed: int = 0):
        w, mbig = self._i32, self.MBIG
        sub = mbig if seed == -2147483648 else abs(seed)
        t = [0] * 56
        mj = w(self.MSEED - sub)
        t[55] = mj
        mk = 1
        for i in range(1, 55):
            ii = (21 * i) % 55
            t[ii] = mk
            mk = w(mj - mk)
            if mk < 0:
                mk = w(mk + mbig)
            mj = t[ii]
        for _ in range(1, 5):
            for i in range(1, 56):
                t[i] = w(t[i] - t[1 + (i + 30) % 55])
                if t[i] < 0:
                    t[i] = w(t[i] + mbig)
        self.t, self.inext, self.inextp = t, 0, 21

    def next_int(self) -> int:
        w = self._i32
        self.inext = self.inext + 1 if self.inext + 1 < 56 else 1
        self.inextp = self.inextp + 1 if self.inextp + 1 < 56 else 1
        r = w(self.t[self.inext] - self.t[self.inextp])
        if r == self.MBIG:
            r -= 1
        if r < 0:
            r = w(r + self.MBIG)
        self.t[self.inext] = r
        return r

    def next_doubles(self, n: int) -> np.ndarray:
        """n values of next_double(), i.e. next_int() * (1.0 / (2^31 - 1)) in binary64."""
        scale = 1.0 / self.MBIG
        return np.array([self.next_int() for _ in range(n)], dtype=np.float64) * scale


def benchmark_scene(n_tris: int = 4096 * 10, seed: int = 0) -> Scene:
    """The reference's own benchmark scene (Benchmark.cpp:66-105): 40,960 triangles of three
    fresh vertices each, x, y, z, r, g, b = (float)Random(0).NextDouble() in that order,
    w = 1 (identity transform), 640x480 viewport and scissor, CullMode None, default Span
    mode, an affine-colour pixel shader without depth test."""
    v = SubtractiveRandom(seed).next_doubles(3 * n_tris * 6).astype(np.float32).reshape(3 * n_tris, 6)
    return Scene(name=f"benchmark{n_tris}", vs=VS.POS_RGB_AFFINE, ps=PS.VCOLOR_AFFINE, width=640,
                 height=480, cull=CullMode.None_, raster=RasterMode.Span, viewport=(0, 0, 640, 480),
                 scissor=(0, 0, 640, 480), attribs=[(v, 24)],
                 indices=np.arange(3 * n_tris, dtype=np.int32))


def scene_from_spec(spec: dict) -> Scene:
    k = spec["kind"]
    if k == "random":
        dm = spec.get("draw_mode")
        return random_scene(spec["seed"], direct=spec.get("direct"),
                            draw_mode=DrawMode(dm) if dm is not None else None,
                            n_prims=spec.get("n_prims"))
    if k == "cube":
        return cube_scene(spec["frame"])
    if k == "sphere":
        return sphere_scene(spec["pose"], level=spec.get("level", 7), width=spec.get("width", 1920),
                            height=spec.get("height", 1080), raster=RasterMode(spec.get("raster", 1)))
    if k == "soup":
        return soup_scene(spec["n"], width=spec.get("width", 3840), height=spec.get("height", 2160),
                          raster=RasterMode(spec.get("raster", 2)))
    if k == "benchmark":
        return benchmark_scene(spec.get("n", 4096 * 10))
    if k == "box":
        return box_scene(spec["frame"])
    if k == "deriv":
        return deriv_scene(spec["frame"], raster=RasterMode(spec.get("raster", 0)))
    if k == "batch":
        return _batch_cached(spec.get("n", 256), spec.get("seed", 4))[spec["item"]]
    raise ValueError(k)


_BATCH_CACHE = {}


def _batch_cached(n, seed):
    """batch_scenes(n, seed) built once per process (fixtures pick single items of it)."""
    if (n, seed) not in _BATCH_CACHE:
        _BATCH_CACHE.clear()
        _BATCH_CACHE[(n, seed)] = batch_scenes(n, seed=seed)
    return _BATCH_CACHE[(n, seed)]


def scene_digest(scene: Scene) -> str:
    """SHA-256 (32 hex digits) of every input of a scene: proves that a scene rebuilt from
    its spec on another machine is bit-identical to the one a fixture was made from."""
    import hashlib
    h = hashlib.sha256()
    for a, s in scene.attribs:
        h.update(np.ascontiguousarray(a).tobytes())
        h.update(str(s).encode())
    for a in (scene.indices, scene.raster_vertices, scene.mvp, scene.light, scene.texture):
        if a is not None:
            h.update(np.ascontiguousarray(a).tobytes())
    h.update(repr((int(scene.vs), int(scene.ps), scene.width, scene.height, int(scene.draw_mode),
                   int(scene.cull), int(scene.raster), tuple(scene.viewport),
                   tuple(float(x) for x in scene.depth_range), tuple(scene.scissor),
                   scene.checker)).encode())
    if scene.tex_size is not None or scene.max_aniso:
        h.update(repr((scene.texture_wh(), scene.max_aniso)).encode())
    return h.hexdigest()[:32]


# ----------------------------------------------------------------------------
# config: batched rendering of many meshes, each to its own target

def _deformed_sphere(level: int, ntris: int, rng):
    """The first `ntris` triangles of an icosphere level, radially deformed by a seeded
    polynomial (no transcendental functions), with normals from the deformed positions'
    face-normal average and planar uv."""
    p, f = icosphere(level)
    f = f[:ntris]
    c = rng.random(6) * 0.4 - 0.2
    x, y, z = p[:, 0], p[:, 1], p[:, 2]
    r = 1.0 + c[0] * x * y + c[1] * y * z + c[2] * z * x + c[3] * x * x + c[4] * y * y * y + c[5] * z
    q = p * r[:, None]
    a, b, cc = q[f[:, 0]], q[f[:, 1]], q[f[:, 2]]
    fn = np.cross(b - a, cc - a)
    nrm = np.zeros_like(q)
    for k in range(3):
        np.add.at(nrm, f[:, k], fn)
    ln = np.sqrt(nrm[:, 0] * nrm[:, 0] + nrm[:, 1] * nrm[:, 1] + nrm[:, 2] * nrm[:, 2])
    ln[ln == 0] = 1.0
    nrm = nrm / ln[:, None]
    pn = np.concatenate([q, nrm], axis=1).astype(np.float32)
    uv = np.stack([(p[:, 0] + 1.0) * 0.5, (p[:, 2] + 1.0) * 0.5], 1).astype(np.float32)
    return pn, uv, f.reshape(-1).astype(np.int32)


def _mesh_texture(rng, size=512):
    y, x = np.mgrid[0:size, 0:size].astype(np.uint32)
    sq = int(rng.integers(8, 64))
    col = rng.integers(0, 256, (2, 3)).astype(np.uint32)
    on = ((x // sq + y // sq) & 1).astype(bool)
    r = np.where(on, col[0, 0], col[1, 0]) ^ (x & 15)
    g = np.where(on, col[0, 1], col[1, 1]) ^ (y & 15)
    b = np.where(on, col[0, 2], col[1, 2])
    return (r | (g << 8) | (b << 16) | (np.uint32(255) << 24)).astype(np.uint32)


def batch_scenes(n: int = 256, seed: int = 4, max_tris: int = 200_000, min_tris: int = 100,
                 sides=(256, 512, 768, 1024), texture_size: int = 512):
    """`n` meshes for one batched submission: triangle counts piecewise-log-uniform in
    [min_tris, max_tris] (octave + linear, truncating the index list of the icosphere level
    that has enough triangles), target side drawn from `sides`, own camera and RGBA8 texture.
    Block mode, CullMode CW, Lambert x nearest texture."""
    rng = np.random.default_rng(seed)
    lo, hi = float(min_tris), float(max_tris)
    out = []
    for i in range(n):
        # log-uniform via octave + linear fraction (exact powers of two)
        span = hi / lo
        octs = int(np.floor(np.log2(span)))  # deterministic: exact for these integer bounds
        while True:
            e = int(rng.integers(0, octs + 1))
            t = lo * float(np.ldexp(1.0, e)) * (1.0 + float(rng.random()))
            if t <= hi:
                break
        ntris = max(1, int(t))
        level = 0
        while 20 * 4 ** level < ntris:
            level += 1
        pn, uv, idx = _deformed_sphere(level, ntris, rng)
        side = int(sides[int(rng.integers(0, len(sides)))])
        d = 2.4 + 1.6 * float(rng.random())
        mvp = mat_to_f32(_matmul4(perspective(1.0, 0.1, 100.0), _matmul4(translate(0.0, 0.0, -d),
                                                                          random_rotation(rng))))
        l = normalized([float(rng.random()) - 0.5, float(rng.random()) - 0.5, 1.0])
        out.append(Scene(name=f"batch{i}[{ntris}t,{side}px]", vs=VS.POS_NRM_UV, ps=PS.LAMBERT_TEX,
                         width=side, height=side, cull=CullMode.CW, raster=RasterMode.Block,
                         viewport=(0, 0, side, side), scissor=(0, 0, side, side),
                         attribs=[(pn, 24), (uv, 8)], indices=idx, mvp=mvp,
                         light=np.array([l[0], l[1], l[2], 0.2], np.float32),
                         texture=_mesh_texture(rng, texture_size)))
    return out


# ----------------------------------------------------------------------------
# config: differentiable rendering (forward + backward of PsDiff)

@dataclass
class DiffProblem:
    """A mesh seen from several views, rendered with the differentiable shader.

    vertices: (V, 8) float32 records {x, y, z, r, g, b, u, v} (VS.POS_RGB_UV stream 0);
    indices: (3F,) int32 triangle list; texture: (T, T, 4) float32 RGBA; mvps: one (16,)
    float32 matrix per view; targets: (views, H, W, 4) float32 images of the L2 loss."""
    name: str
    vertices: np.ndarray
    indices: np.ndarray
    texture: np.ndarray
    mvps: List[np.ndarray]
    targets: np.ndarray
    width: int
    height: int
    cull: CullMode = CullMode.CW
    raster: RasterMode = RasterMode.Block

    @property
    def viewport(self):
        return (0, 0, self.width, self.height)

    @property
    def n_views(self):
        return len(self.mvps)

    def scene(self, view: int) -> Scene:
        """View `view` as an ordinary Scene (for the oracle and single-draw paths)."""
        return Scene(name=f"{self.name}[{view}]", vs=VS.POS_RGB_UV, ps=PS.DIFF, width=self.width,
                     height=self.height, cull=self.cull, raster=self.raster, viewport=self.viewport,
                     scissor=self.viewport, attribs=[(self.vertices, 32)], indices=self.indices,
                     mvp=self.mvps[view], texture=self.texture)


def _smooth_texture(rng, size):
    """RGBA32F texture from seeded cubic polynomials in (x, y) scaled into [0.15, 0.95] (alpha
    [0.5, 1]): smooth, so the bilinear interpolant's slope changes little between texels."""
    t = np.linspace(0.0, 1.0, size)
    y, x = np.meshgrid(t, t, indexing="ij")
    out = np.empty((size, size, 4), np.float64)
    for c in range(4):
        a = rng.random(10) * 2.0 - 1.0
        v = (a[0] + a[1] * x + a[2] * y + a[3] * x * x + a[4] * x * y + a[5] * y * y +
             a[6] * x * x * x + a[7] * x * x * y + a[8] * x * y * y + a[9] * y * y * y)
        lo, hi = float(v.min()), float(v.max())
        v = (v - lo) / (hi - lo if hi > lo else 1.0)
        out[:, :, c] = 0.5 + 0.5 * v if c == 3 else 0.15 + 0.8 * v
    return out.astype(np.float32)


def diff_problem(n_views: int = 16, level: int = 6, size: int = 512, tex_size: int = 1024,
                 seed: int = 5, raster: RasterMode = RasterMode.Block, clip_views: int = 0,
                 cull: CullMode = CullMode.CW) -> DiffProblem:
    """Icosphere at subdivision `level` (level 6: 40,962 v / 81,920 t) with seeded per-vertex
    RGB in [0.2, 0.8] and planar uv, a `tex_size`^2 RGBA32F texture sampled bilinearly, seen
    from `n_views` seeded cameras (60 degree perspective, distance in [2.5, 3.5]) at
    size x size; L2 targets are seeded uniform images.  The first `clip_views` cameras sit
    at distance 1.11, so the near plane (0.1) cuts the sphere and clipping splits triangles."""
    rng = np.random.default_rng(seed)
    p, f = icosphere(level)
    rgb = rng.random((p.shape[0], 3)) * 0.6 + 0.2
    uv = np.stack([(p[:, 0] + 1.0) * 0.5, (p[:, 1] + 1.0) * 0.5], 1)
    verts = np.concatenate([p, rgb, uv], axis=1).astype(np.float32)
    tex = _smooth_texture(rng, tex_size)
    mvps = []
    for k in range(n_views):
        d = 2.5 + float(rng.random())
        if k < clip_views:
            d = 1.11
        mvps.append(mat_to_f32(_matmul4(perspective(1.0, 0.1, 100.0),
                                        _matmul4(translate(0.0, 0.0, -d), random_rotation(rng)))))
    targets = rng.random((n_views, size, size, 4)).astype(np.float32)
    return DiffProblem(name=f"diff_ico{level}x{n_views}@{size}", vertices=verts,
                       indices=f.reshape(-1).astype(np.int32), texture=tex, mvps=mvps, targets=targets,
                       width=size, height=size, raster=raster, cull=cull)
