"""The rounding bound behind the raster's depth cull (z_not_below in csrc/swr_stages.cuh).

A covered pixel's z is the plane evaluated ((a x) + (b y)) + c in binary32 at the walk's
start and then stepped k times by b (rows) or a (columns), each step one rounding, as the
reference's PixelData stepping does.  The cull assumes that this stepped z differs from the
exact plane value at the pixel by at most 2^-23 (k + 4) Q + 2^-126, with
Q = |a| X + |b| Y + |c| and X, Y bounds of the walk's coordinates.  These tests check that
bound against exact rational arithmetic on random and adversarial planes (no GPU needed).
"""
from fractions import Fraction

import numpy as np
import pytest

f32 = np.float32


def stepped(a, b, c, fx, fy, kb, ka):
    """binary32 evaluation then kb steps by b and ka steps by a (sequential, no FMA)."""
    e = f32(f32(f32(a * fx) + f32(b * fy)) + c)
    for _ in range(kb):
        e = f32(e + b)
    for _ in range(ka):
        e = f32(e + a)
    return e


def check(a, b, c, x0, y0, kb, ka):
    a, b, c = f32(a), f32(b), f32(c)
    fx, fy = f32(x0 + 0.5), f32(y0 + 0.5)
    z = stepped(a, b, c, fx, fy, kb, ka)
    if not np.isfinite(z):
        return
    exact = Fraction(float(a)) * (Fraction(float(fx)) + ka) + Fraction(float(b)) * (Fraction(float(fy)) + kb) \
        + Fraction(float(c))
    k = ka + kb
    X = float(fx) + ka
    Y = float(fy) + kb
    q = abs(float(a)) * X + abs(float(b)) * Y + abs(float(c))
    margin = Fraction(2.0 ** -23) * (k + 4) * Fraction(q) + Fraction(2.0 ** -126)
    err = abs(Fraction(float(z)) - exact)
    assert err <= margin, (a, b, c, x0, y0, kb, ka, float(err), float(margin))


def test_random_planes_block_walks():
    rng = np.random.default_rng(1)
    for _ in range(3000):
        a, b = rng.normal(0, 10.0 ** rng.uniform(-6, 2), 2)
        c = rng.normal(0, 10.0 ** rng.uniform(-3, 3))
        x0, y0 = int(rng.integers(0, 4096)) & ~7, int(rng.integers(0, 4096)) & ~7
        check(a, b, c, x0, y0, int(rng.integers(0, 8)), int(rng.integers(0, 8)))


def test_random_planes_span_walks():
    rng = np.random.default_rng(2)
    for _ in range(400):
        a = rng.normal(0, 10.0 ** rng.uniform(-6, 0))
        b = rng.normal(0, 10.0 ** rng.uniform(-6, 0))
        c = rng.normal(0, 10.0 ** rng.uniform(-2, 2))
        x0, y0 = int(rng.integers(0, 3840)), int(rng.integers(0, 2160))
        check(a, b, c, x0, y0, 0, int(rng.integers(0, 600)))


@pytest.mark.parametrize("a,b,c", [
    (1e-3, -2e-3, 0.999),          # window depths near 1 (perspective soup)
    (3.0e-4, 3.0e-4, -1.0),        # cancellation of a x + c
    (-1.0, 1.0, 4000.0),           # large terms, small result near the far corner
    (1e-30, 1e-30, 1e-38),         # subnormal results
    (0.0, 0.0, 0.5),               # constant plane (exact)
])
def test_adversarial_planes(a, b, c):
    for x0, y0 in ((0, 0), (1912, 1072), (3832, 2152)):
        for kb, ka in ((0, 0), (7, 7), (0, 255), (3, 5)):
            check(a, b, c, x0, y0, kb, ka)
