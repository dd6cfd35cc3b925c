"""Flexible CG with the learned U-Net preconditioner on the fine grid (small
grids): the training data are solver-generated residual/error pairs, FCG
reaches the 1e-8 true relative residual without the Jacobi-PCG fallback,
agrees with Jacobi-PCG's solution and needs fewer iterations than
Jacobi-PCG; the trained network needs fewer iterations than the untrained
one. The multilevel form, the one the
benchmark uses, is tested in test_mg_gpu.py."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_cg_pairs_are_residual_error_pairs(ngb, cuda):
    import torch
    from neon_gb300 import fcg
    n = 32
    pairs = fcg.cg_pairs(n, 3, {2, 10}, cuda, tol=1e-9)
    assert len(pairs) == 2
    d = ngb.poisson_desc(n, n, n, "f32", 1.0)
    for r, e in pairs:
        ae = torch.empty_like(e)
        ngb.laplacian_apply(d, e, ae)
        mask = fcg.free_mask(n, cuda)
        # A e = r on the Free rows (up to the final CG residual and FP32 rounding)
        assert float(((ae - r) * mask).norm() / (r * mask).norm()) < 1e-4


@pytest.fixture(scope="module")
def trained(ngb, cuda):
    from neon_gb300 import fcg
    from neon_gb300.learned import UNet
    n = 32
    pairs = []
    for s in range(24):
        pairs += fcg.cg_pairs(n, 100 + s, {1, 3, 6, 12, 24, 48}, cuda)
    net = UNet(seed=0, device=cuda)
    losses = fcg.train(net, pairs, epochs=3, lr=2e-3)
    return net, losses


def test_training_lowers_the_error_loss(trained):
    net, losses = trained
    k = len(losses) // 3
    assert np.mean(losses[-k:]) < 0.7 * np.mean(losses[:k]), (np.mean(losses[:k]), np.mean(losses[-k:]))


def test_fcg_converges_and_beats_jacobi_pcg(ngb, orc, cuda, trained):
    import torch
    from neon_gb300 import fcg
    from neon_gb300.learned import UNet
    from helpers import P
    net, _ = trained
    n = 32
    b = fcg.grf_k2(n, 999, cuda)
    x = torch.zeros(n ** 3, dtype=torch.float64, device=cuda)
    # at 32^3 the fine-grid form converges without the Jacobi-PCG fallback
    # (it stalls on larger grids, where the network's BF16 output noise,
    # amplified by A, grows with n^2; the V-cycle form serves those)
    res = fcg.fcg_solve(net, b, x, tol=1e-8, max_iter=400, fallback=True)
    assert res["converged"] and not res["fallback"], res
    # Jacobi-PCG on the same system
    d = ngb.poisson_desc(n, n, n, "f32", 1.0)
    ws = ngb.cg_workspace(d, cuda)
    x2 = torch.zeros_like(x)
    pcg = ngb.cg_solve(d, b, x2, ws, tol=1e-8, max_iter=5000, refresh_every=50, check_every=10, jacobi=True)
    assert pcg["converged"]
    assert float((x - x2).norm() / x2.norm()) < 1e-6
    assert res["iterations"] < pcg["iterations"], (res["iterations"], pcg["iterations"])
    # the untrained network is worse than the trained one
    x3 = torch.zeros_like(x)
    raw = fcg.fcg_solve(UNet(seed=0, device=cuda), b, x3, tol=1e-8, max_iter=400, fallback=True)
    assert raw["converged"], raw
    assert res["iterations"] < raw["iterations"] + raw["fallback_iterations"], (res, raw)
