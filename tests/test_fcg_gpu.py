"""Flexible CG with the learned U-Net preconditioner: the training data are
solver-generated residual/error pairs and training lowers the loss,
deterministically; with a trained network as the coarsest solve of a
V-cycle, FCG reaches the 1e-8 true relative residual without the Jacobi-PCG
fallback, agrees with Jacobi-PCG's solution and needs fewer iterations than
Jacobi-PCG, than the cycle without the network and than the cycle with the
untrained network. More of the multilevel form is tested in test_mg_gpu.py."""
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


def test_fcg_converges_and_beats_jacobi_pcg(ngb, orc, cuda):
    """A trained network (the committed neon_gb300/weights/unet_poisson_64.ngbw,
    trained at 64^3 by bench.py --workload learned) as the 64^3 coarsest
    solve of a V-cycle inside FCG at 128^3: converges to 1e-8 without the
    Jacobi-PCG fallback, to the Jacobi-PCG solution, in fewer iterations than
    Jacobi-PCG, than the same cycle without the network and than the cycle
    with the untrained network."""
    import os
    import torch
    from neon_gb300 import fcg
    from neon_gb300.learned import UNet
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    net = UNet(seed=0, device=cuda)
    net.load_weights(os.path.join(root, "neon_gb300", "weights", "unet_poisson_64.ngbw"))
    n = 128
    b = fcg.grf_k2(n, 999, cuda)
    x = torch.zeros(n ** 3, dtype=torch.float64, device=cuda)
    res = fcg.fcg_solve_vcycle(fcg.VCycle(n, 1, net, device=cuda), b, x, tol=1e-8, max_iter=400, fallback=True)
    assert res["converged"] and not res["fallback"], res
    d = ngb.poisson_desc(n, n, n, "f32", 1.0)
    ws = ngb.cg_workspace(d, cuda)
    x2 = torch.zeros_like(x)
    pcg = ngb.cg_solve(d, b, x2, ws, tol=1e-8, max_iter=5000, refresh_every=50, check_every=10, jacobi=True)
    assert pcg["converged"]
    assert float((x - x2).norm() / x2.norm()) < 1e-6
    assert res["iterations"] < pcg["iterations"], (res["iterations"], pcg["iterations"])
    x3 = torch.zeros_like(x)
    plain = fcg.fcg_solve_vcycle(fcg.VCycle(n, 1, coarse="none", device=cuda), b, x3, tol=1e-8, max_iter=400, fallback=True)
    assert plain["converged"], plain
    assert res["iterations"] < plain["iterations"] + plain["fallback_iterations"], (res, plain)
    x4 = torch.zeros_like(x)
    raw = fcg.fcg_solve_vcycle(fcg.VCycle(n, 1, UNet(seed=0, device=cuda), device=cuda), b, x4, tol=1e-8, max_iter=400,
                               fallback=True)
    assert raw["converged"], raw
    assert res["iterations"] < raw["iterations"] + raw["fallback_iterations"], (res, raw)


def test_training_is_deterministic(ngb, cuda):
    """Two trainings from the same seed on the same solver pairs give the
    same losses bit for bit (every kernel of the step, the tcgen05 weight
    gradient included, sums in a fixed order)."""
    from neon_gb300 import fcg
    from neon_gb300.learned import UNet
    n = 32
    pairs = []
    for s in range(3):
        pairs += fcg.cg_pairs(n, 300 + s, {2, 8, 32}, cuda)
    runs = []
    for _ in range(2):
        net = UNet(seed=0, device=cuda)
        runs.append(fcg.train(net, pairs, epochs=1, lr=2e-3))
    assert runs[0] == runs[1]
