"""The learned-preconditioner solver behind the C ABI (ngb_learned_*) against
the Python orchestration of the same kernels (neon_gb300.fcg), which the
earlier tests check against the oracle: the preconditioner application must be
bit-identical, the solve must reach 1e-8 with the same iteration count within
+-2, and a broken network must hand over to Jacobi-PCG."""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _rhs(ngb, n, cuda):
    import torch
    d = ngb.poisson_desc(n, n, n, "f32", 1.0)
    c, a = ngb.gaussian_sources(n, n, n, 2024)
    b = torch.empty(n ** 3, dtype=torch.float32, device=cuda)
    ngb.poisson_rhs(d, torch.from_numpy(c).to(cuda), torch.from_numpy(a).to(cuda), 8.0, b)
    return b


@pytest.mark.parametrize("n,levels", [(64, 1), (128, 2)])
def test_precondition_bit_identical_to_python_vcycle(ngb, cuda, n, levels):
    import torch
    from neon_gb300 import fcg
    from neon_gb300.learned import UNet
    net = UNet(seed=0, device=cuda)
    g = torch.Generator(device=cuda).manual_seed(5)
    r = torch.randn(n ** 3, device=cuda, generator=g) * fcg.free_mask(n, cuda)
    z_py = fcg.VCycle(n, levels, net, device=cuda)(r).clone()
    S = ngb.LearnedSolver(n, levels, net.flat_weights())
    z_c = torch.full_like(r, float("nan"))
    S.precondition(r, z_c)
    net.check()
    torch.cuda.synchronize()
    assert torch.equal(z_c, z_py)
    S.close()


@pytest.mark.parametrize("n,levels", [(64, 1), (128, 2)])
def test_cycle_without_network_bit_identical_to_python(ngb, cuda, n, levels):
    """weights=None: the same V-cycle without the coarsest correction, equal
    to VCycle(coarse="none") bit for bit, and its FCG solve converges."""
    import torch
    from neon_gb300 import fcg
    g = torch.Generator(device=cuda).manual_seed(6)
    r = torch.randn(n ** 3, device=cuda, generator=g) * fcg.free_mask(n, cuda)
    z_py = fcg.VCycle(n, levels, coarse="none", device=cuda)(r).clone()
    S = ngb.LearnedSolver(n, levels, None)
    z_c = torch.full_like(r, float("nan"))
    S.precondition(r, z_c)
    torch.cuda.synchronize()
    assert torch.equal(z_c, z_py)
    b = _rhs(ngb, n, cuda)
    x = torch.zeros(n ** 3, dtype=torch.float64, device=cuda)
    got = S.solve(b, x, tol=1e-8, max_iter=4000)
    assert got["converged"] and not got["fallback"] and got["rel_residual"] <= 1e-8
    S.close()


def test_solve_matches_python_fcg(ngb, cuda):
    import torch
    from neon_gb300 import fcg
    from neon_gb300.learned import UNet
    n, levels = 128, 1
    net = UNet(seed=0, device=cuda)
    b = _rhs(ngb, n, cuda)
    x_py = torch.zeros(n ** 3, dtype=torch.float64, device=cuda)
    ref = fcg.fcg_solve_vcycle(fcg.VCycle(n, levels, net, device=cuda), b, x_py, tol=1e-8, max_iter=2000, fallback=True)
    S = ngb.LearnedSolver(n, levels, net.flat_weights())
    x = torch.zeros(n ** 3, dtype=torch.float64, device=cuda)
    got = S.solve(b, x, tol=1e-8)
    assert got["converged"] and got["rel_residual"] <= 1e-8
    assert got["fallback"] == ref["fallback"]
    assert abs(got["iterations"] - ref["iterations"]) <= 2, (got, ref)
    assert float((x - x_py).norm() / x_py.norm()) <= 1e-7
    S.close()


def test_broken_network_hands_over_to_jacobi_pcg(ngb, cuda):
    """NaN weights make every preconditioned direction NaN: the solve must
    detect the breakdown, restart Jacobi-PCG from zero and still converge."""
    import torch
    n, levels = 64, 1
    w = torch.full((int(ngb.lib().ngb_unet_weight_count()),), float("nan"))
    S = ngb.LearnedSolver(n, levels, w)
    b = _rhs(ngb, n, cuda)
    x = torch.zeros(n ** 3, dtype=torch.float64, device=cuda)
    got = S.solve(b, x, tol=1e-8)
    assert got["fallback"] and got["converged"] and got["fallback_iterations"] > 0
    assert math.isfinite(got["rel_residual"]) and got["rel_residual"] <= 1e-8
    assert bool(torch.isfinite(x).all())
    S.close()
