"""The exact fast-forward of incremental stepping (swr_fold, csrc/swr_math.h).

The reference builds every per-pixel value by repeated v = fl(v + a) (PixelData.h:61-125,
EdgeData.h:37-80); swr_fold must return bit for bit what k serial steps return.  The same
header is compiled into the CUDA kernels, so these CPU checks cover the device code path.
"""
import math
import struct

import numpy as np
import pytest


def f32(x):
    return float(np.float32(x))


def bits(x):
    return struct.unpack("<I", struct.pack("<f", x))[0]


def serial(v, a, k):
    v, a = np.float32(v), np.float32(a)
    for _ in range(k):
        v = np.float32(v + a)
    return float(v)


def same(x, y):
    return (math.isnan(x) and math.isnan(y)) or bits(x) == bits(y)


def test_randomized_against_serial(port):
    assert port.lib.oracle_fold_selftest(1_500_000, 7) == 0


EDGE = [
    (1.0, 2.0 ** -24, 5000),          # exactly half an ulp: ties to even, never moves
    (1.0 + 2.0 ** -23, 2.0 ** -24, 3000),  # odd significand: first tie rounds up, then stays
    (1.0, 3 * 2.0 ** -24, 4000),      # 1.5 ulp ties alternate parity
    (1.0, -2.0 ** -25, 100),          # shrinking from exactly 2^0 reaches the finer grid
    (0.75, 1e-3, 20000),              # crosses the binade at 1.0 and 2.0 ...
    (-3.0, 1e-3, 9000),               # crosses zero
    (1e-38, -1e-39, 50),              # into subnormals
    (3.4e38, 3e31, 200),              # overflow to +inf
    (0.0, 0.0, 10), (-0.0, 0.0, 10), (-0.0, -0.0, 10), (5.0, -0.0, 10),
    (float("inf"), -1.0, 10), (1.0, float("nan"), 10), (1.0, float("inf"), 10),
    (2.0 ** 24, 1.0, 100),            # a below half an ulp of v
    (123.456, 0.1, 3840),             # a 4K span
]


@pytest.mark.parametrize("v,a,k", EDGE)
def test_edge_cases(port, v, a, k):
    v, a = f32(v), f32(a)
    for kk in (0, 1, 2, 6, 7, 8, 31, k):
        assert same(port.fold(v, a, kk), serial(v, a, kk)), (v, a, kk)
