"""The oracle's mixed-precision Jacobi-PCG on the CPU: the FP32 form keeps
the true residual as a float pair and updates it incrementally at each
refresh (as the GPU solver does); its reported residual must equal an FP64
recomputation of b - A x for the returned x, and the solution must agree
with the FP64-field solve."""
import ctypes

import numpy as np
import pytest

from helpers import P


def _problem(orc, n, sigma):
    c = np.zeros(24)
    a = np.zeros(8)
    orc.orc_gaussian_sources(n, n, n, ctypes.c_uint64(7), P(c), P(a))
    z, y, x = np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij")
    f = np.zeros((n, n, n))
    for k in range(8):
        f += a[k] * np.exp(-((x - c[3 * k]) ** 2 + (y - c[3 * k + 1]) ** 2 + (z - c[3 * k + 2]) ** 2) / (2 * sigma ** 2))
    bd = np.zeros(n ** 3, np.int8)
    orc.orc_box_boundary(n, n, n, P(bd))
    f = f.ravel()
    f[bd == 0] = 0.0
    return f, bd


@pytest.mark.parametrize("n,h,refresh", [(24, 1.0, 50), (20, 0.3, 7)])
def test_float_pair_refresh_tracks_the_true_residual(orc, n, h, refresh):
    f, bd = _problem(orc, n, 4.0)
    b32 = f.astype(np.float32)
    x32 = np.zeros(n ** 3)
    res = np.zeros(4)
    orc.orc_pcg_f32(n, n, n, ctypes.c_double(h), P(bd), P(b32), P(x32), ctypes.c_double(1e-8), 3000, refresh, P(res), 1)
    assert res[1] == 1 and res[3] >= 2, res  # converged, with refreshes on the way
    ax = np.zeros(n ** 3)
    orc.orc_laplacian_f64(n, n, n, ctypes.c_double(h), P(x32), P(bd), P(ax))
    free = bd == 1
    b = b32.astype(np.float64)
    true = np.linalg.norm((b - ax)[free]) / np.linalg.norm(b[free])
    assert true <= 1e-8
    assert abs(res[2] - true) <= 1e-6 * true, (res[2], true)
    x64 = np.zeros(n ** 3)
    res64 = np.zeros(4)
    orc.orc_pcg_f64(n, n, n, ctypes.c_double(h), P(bd), P(b), P(x64), ctypes.c_double(1e-8), 3000, refresh, P(res64), 1)
    assert res64[1] == 1
    assert np.linalg.norm(x32 - x64) / np.linalg.norm(x64) <= 1e-7
