"""The cached kernel's Sobol sampler (csrc/qmc.cuh, orn_state.sampler =
SOBOL), through the host copy of the same inline code (orn_qmc_points):
every power-of-two prefix of a pixel's samples is a (0,m,2)-net in each of
its four uses (each elementary interval of area 2^-m holds exactly one
point), points lie in [0, 1), and uses and pixels are decorrelated."""
import ctypes as C

import numpy as np
import pytest

from zig_ornament_gb300 import _lib


def _points(pixel, pair, first, count):
    out = np.zeros((count, 2), np.float32)
    assert _lib.load().orn_qmc_points(pixel, pair, first, count, out.ctypes.data_as(C.c_void_p)) == 0
    return out


def _is_net(pts, m):
    n = 1 << m
    for k in range(m + 1):
        cx = np.floor(pts[:, 0].astype(np.float64) * (1 << k)).astype(np.int64)
        cy = np.floor(pts[:, 1].astype(np.float64) * (1 << (m - k))).astype(np.int64)
        cells = cx * (1 << (m - k)) + cy
        if len(np.unique(cells)) != n:
            return False
    return True


@pytest.mark.parametrize("pixel", [0, 7, 12345, 2073599])
@pytest.mark.parametrize("pair", [0, 1, 2, 3])
def test_prefixes_are_nets(pixel, pair):
    pts = _points(pixel, pair, 0, 1024)
    assert (pts >= 0).all() and (pts < 1).all()
    for m in range(1, 11):
        assert _is_net(pts[: 1 << m], m), (pixel, pair, m)


def test_uses_and_pixels_differ():
    a = _points(5, 0, 0, 256)
    assert not np.allclose(a, _points(5, 1, 0, 256))
    assert not np.allclose(a, _points(6, 0, 0, 256))
    # the two coordinates of different uses are uncorrelated over many pixels
    xs = np.array([_points(p, 0, 3, 1)[0, 0] for p in range(2000)])
    ys = np.array([_points(p, 2, 3, 1)[0, 0] for p in range(2000)])
    assert abs(np.corrcoef(xs, ys)[0, 1]) < 0.1
    assert abs(xs.mean() - 0.5) < 0.03


def test_bad_pair_is_refused():
    out = np.zeros(2, np.float32)
    assert _lib.load().orn_qmc_points(0, 4, 0, 1, out.ctypes.data_as(C.c_void_p)) == 1
