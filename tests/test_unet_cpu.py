"""CPU checks of the U-Net oracle itself: the BF16 rounding against torch, the
convolution adjoint identity, and the analytic gradient against central finite
differences (without roundings)."""
import numpy as np
import pytest

from oracle import unet_oracle as U


def test_bf16_rounding_matches_torch():
    torch = pytest.importorskip("torch")
    x = np.random.default_rng(0).standard_normal(100000) * 10.0 ** np.random.default_rng(1).integers(-20, 20, 100000)
    ref = torch.from_numpy(x.astype(np.float32)).to(torch.bfloat16).float().numpy().astype(np.float64)
    assert np.array_equal(U.bf16(x), ref)


def test_conv_adjoint_identity():
    rng = np.random.default_rng(2)
    x = rng.standard_normal((6, 5, 7, 16))
    w = rng.standard_normal((8, 27, 16))
    y = rng.standard_normal((6, 5, 7, 8))
    lhs = np.sum(U.conv(x, w) * y)
    rhs = np.sum(x * U.conv_bwd_data(y, w))
    assert abs(lhs - rhs) <= 1e-10 * abs(lhs)
    # and the weight gradient is the derivative of <conv(x, w), y> in w
    dw = U.conv_bwd_weight(x, y)
    assert abs(np.sum(dw * w) - lhs) <= 1e-10 * abs(lhs)


def test_gradient_matches_finite_differences():
    rng = np.random.default_rng(3)
    n = 8
    W = {k: rng.standard_normal((co, 27, ci)) * np.sqrt(2.0 / (27 * ci)) for k, ci, co in U.LAYERS}
    r = rng.standard_normal(n ** 3)
    e = rng.standard_normal(n ** 3)

    def loss(Wd):
        z, cache = U.forward(Wd, r, n, rounding=False)
        return 0.5 * np.sum((z - e) ** 2), z, cache

    L0, z, cache = loss(W)
    g = U.backward(cache, z - e)
    for name in ("c0a", "c1c", "c2b", "c0d"):
        idx = tuple(rng.integers(0, s) for s in W[name].shape)
        h = 1e-6
        Wp = {k: v.copy() for k, v in W.items()}
        Wm = {k: v.copy() for k, v in W.items()}
        Wp[name][idx] += h
        Wm[name][idx] -= h
        fd = (loss(Wp)[0] - loss(Wm)[0]) / (2 * h)
        assert abs(fd - g[name][idx]) <= 1e-5 * max(1.0, abs(fd)), (name, fd, g[name][idx])
