"""Multilevel learned preconditioner: the ngb_mg_* smoothing and grid-transfer
kernels against plain PyTorch float64 restatements (FP32 tolerance 1e-5), the
adjoint pair R = P^T / 8, and FCG with the V-cycle whose coarsest solve is
the trained network: it reaches the 1e-8 true residual, agrees with
Jacobi-PCG's solution, and needs fewer iterations than the same cycle
without the network and than Jacobi-PCG."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _lap64(u, h):
    """7-point operator on interior nodes of a [z, y, x] float64 array, 0 on faces."""
    import torch
    out = torch.zeros_like(u)
    c = u[1:-1, 1:-1, 1:-1]
    s = (u[2:, 1:-1, 1:-1] + u[:-2, 1:-1, 1:-1] + u[1:-1, 2:, 1:-1] + u[1:-1, :-2, 1:-1] + u[1:-1, 1:-1, 2:] +
         u[1:-1, 1:-1, :-2])
    out[1:-1, 1:-1, 1:-1] = (6 * c - s) / (h * h)
    return out


def _interior(n, dev):
    import torch
    m = torch.zeros(n, n, n, dtype=torch.float64, device=dev)
    m[1:-1, 1:-1, 1:-1] = 1
    return m


def _restrict64(res):
    import torch
    t = res
    nc = res.shape[0] // 2
    for dim in range(3):
        t = t.movedim(dim, 0)
        pad = torch.cat([torch.zeros_like(t[:1]), t, torch.zeros_like(t[:1])], 0)
        i = torch.arange(nc, device=res.device) * 2 + 1
        t = (0.25 * pad[i - 1] + 0.5 * pad[i] + 0.25 * pad[i + 1]).movedim(0, dim)
    return t * _interior(nc, res.device)


def _prolong64(e, n):
    import torch
    t = e
    for dim in range(3):
        t = t.movedim(dim, 0)
        out = torch.zeros((n,) + t.shape[1:], dtype=t.dtype, device=t.device)
        out[0::2] = t[:n // 2]
        nxt = torch.cat([t[1:], torch.zeros_like(t[:1])], 0)
        out[1::2] = (0.5 * (t + nxt))[:n // 2]
        t = out.movedim(0, dim)
    return t * _interior(n, e.device)


def _field(n, seed, dev, faces_zero=True):
    import torch
    g = torch.Generator().manual_seed(seed)
    f = torch.randn(n, n, n, generator=g, dtype=torch.float64).to(dev)
    return f * _interior(n, dev) if faces_zero else f


def _close(got, ref, tol=1e-5):
    return float((got.double() - ref).abs().max() / max(float(ref.abs().max()), 1e-30)) <= tol


@pytest.mark.parametrize("n,h", [(20, 1.0), (34, 2.0), (70, 1.0)])
def test_jacobi_and_residual_kernels(ngb, cuda, n, h):
    import torch
    d = ngb.poisson_desc(n, n, n, "f32", h)
    u, r = _field(n, 1, cuda), _field(n, 2, cuda)
    out = torch.empty(n ** 3, dtype=torch.float32, device=cuda)
    w = 6.0 / 7.0
    c = w * h * h / 6.0
    ngb.mg_jacobi(d, u.float().reshape(-1), r.float().reshape(-1), out, w)
    assert _close(out.reshape(n, n, n), (u + c * (r - _lap64(u, h))) * _interior(n, cuda))
    ngb.mg_jacobi(d, None, r.float().reshape(-1), out, w)  # two sweeps from zero
    u1 = c * r
    u2 = (u1 + c * (r - _lap64(u1, h))) * _interior(n, cuda)
    assert _close(out.reshape(n, n, n), u2)
    ngb.mg_residual(d, u.float().reshape(-1), r.float().reshape(-1), out)
    assert _close(out.reshape(n, n, n), (r - _lap64(u, h)) * _interior(n, cuda))
    ngb.mg_residual(d, None, r.float().reshape(-1), out)
    assert _close(out.reshape(n, n, n), r * _interior(n, cuda))
    ngb.mg_apply(d, u.float().reshape(-1), out)
    assert _close(out.reshape(n, n, n), _lap64(u, h) * _interior(n, cuda))


@pytest.mark.parametrize("dims", [(37, 70, 19), (96, 33, 45), (130, 66, 9)])
def test_stencil_passes_on_ragged_tiles(ngb, cuda, dims):
    """Box sizes that are no multiple of the 32 x 32 column tiles or of the
    plane chunks, with non-zero values on the faces (the interior nodes next
    to a face read them): every mode against float64."""
    import torch
    nx, ny, nz = dims
    h = 0.5
    d = ngb.poisson_desc(nx, ny, nz, "f32", h)
    g = torch.Generator().manual_seed(nx * ny + nz)
    u = torch.randn(nz, ny, nx, generator=g, dtype=torch.float64).to(cuda)
    r = torch.randn(nz, ny, nx, generator=g, dtype=torch.float64).to(cuda)
    m = torch.zeros_like(u)
    m[1:-1, 1:-1, 1:-1] = 1
    out = torch.full((nx * ny * nz,), float("nan"), dtype=torch.float32, device=cuda)
    w = 6.0 / 7.0
    c = w * h * h / 6.0
    uf, rf = u.float().reshape(-1), r.float().reshape(-1)
    ub, rb = uf.double().reshape(nz, ny, nx), rf.double().reshape(nz, ny, nx)  # the FP32 inputs, exactly
    ngb.mg_jacobi(d, uf, rf, out, w)
    assert _close(out.reshape(nz, ny, nx), (ub + c * (rb - _lap64(ub, h))) * m)
    ngb.mg_jacobi(d, None, rf, out, w)
    assert _close(out.reshape(nz, ny, nx), (2 * c * rb - c * c * _lap64(rb, h)) * m)
    ngb.mg_residual(d, uf, rf, out)
    assert _close(out.reshape(nz, ny, nx), (rb - _lap64(ub, h)) * m)
    ngb.mg_residual(d, None, rf, out)
    assert torch.equal(out.reshape(nz, ny, nx), (rb * m).float())
    ngb.mg_apply(d, uf, out)
    assert _close(out.reshape(nz, ny, nx), _lap64(ub, h) * m)


@pytest.mark.parametrize("n", [12, 40])
def test_restrict_prolong_kernels_and_adjoint(ngb, cuda, n):
    import torch
    d = ngb.poisson_desc(n, n, n, "f32", 1.0)
    nc = n // 2
    a = _field(n, 3, cuda)
    rc = torch.full((nc ** 3,), float("nan"), dtype=torch.float32, device=cuda)
    ngb.mg_restrict(d, a.float().reshape(-1), rc, 2.0)
    assert _close(rc.reshape(nc, nc, nc), 2.0 * _restrict64(a.float().double()))
    e = _field(nc, 4, cuda)
    u = _field(n, 5, cuda)
    uf = u.float().reshape(-1).clone()
    ngb.mg_prolong_add(d, e.float().reshape(-1), uf)
    assert _close(uf.reshape(n, n, n), u.float().double() + _prolong64(e.float().double(), n))
    # R = P^T / 8 on fields that vanish on the faces
    lhs = 8.0 * float((_restrict64(a) * e).sum())
    rhs = float((a * _prolong64(e, n)).sum())
    assert abs(lhs - rhs) <= 1e-10 * abs(rhs)


def test_mg_kernels_reject_bad_arguments(ngb, cuda):
    import torch
    d = ngb.poisson_desc(13, 12, 12, "f32", 1.0)
    a = torch.zeros(13 * 12 * 12, device=cuda)
    b = torch.zeros(13 * 12 * 12, device=cuda)
    with pytest.raises(ngb.NeonError, match="even"):
        ngb.mg_restrict(d, a, b)
    d64 = ngb.poisson_desc(12, 12, 12, "f64", 1.0)
    with pytest.raises(ngb.NeonError, match="FP32"):
        ngb.mg_residual(d64, None, a, b)


@pytest.fixture(scope="module")
def trained32(ngb, cuda):
    """The network trained on solver pairs at 32^3: the coarsest level of a
    two-coarsening cycle on 128^3."""
    from neon_gb300 import fcg
    from neon_gb300.learned import UNet
    pairs = []
    for s in range(24):
        pairs += fcg.cg_pairs(32, 300 + s, {1, 3, 6, 12, 24, 48}, cuda)
    net = UNet(seed=0, device=cuda)
    fcg.train(net, pairs, epochs=3, lr=2e-3)
    return net


def test_vcycle_fcg_converges_and_the_network_helps(ngb, cuda, trained32):
    import torch
    from neon_gb300 import fcg
    n = 128
    b = fcg.grf_k2(n, 4242, cuda)
    x = torch.zeros(n ** 3, dtype=torch.float64, device=cuda)
    res = fcg.fcg_solve_vcycle(fcg.VCycle(n, 2, trained32, device=cuda), b, x, tol=1e-8, max_iter=500, fallback=False)
    assert res["converged"], res
    # Jacobi-PCG on the same system
    d = ngb.poisson_desc(n, n, n, "f32", 1.0)
    ws = ngb.cg_workspace(d, cuda)
    x2 = torch.zeros_like(x)
    pcg = ngb.cg_solve(d, b, x2, ws, tol=1e-8, max_iter=5000, refresh_every=50, check_every=10, jacobi=True)
    assert pcg["converged"]
    assert float((x - x2).norm() / x2.norm()) < 1e-6
    # the same cycle without the network's coarse correction
    x3 = torch.zeros_like(x)
    plain = fcg.fcg_solve_vcycle(fcg.VCycle(n, 2, coarse="none", device=cuda), b, x3, tol=1e-8, max_iter=500,
                                 fallback=False)
    assert plain["converged"], plain
    assert res["iterations"] < plain["iterations"] < pcg["iterations"], (res["iterations"], plain["iterations"],
                                                                         pcg["iterations"])


def test_fcg_vector_steps_match_torch(ngb, cuda):
    """ngb_fcg_direction / ngb_fcg_update against float64 torch restatements."""
    import ctypes
    import torch
    L = ngb.lib()
    n = 1_000_003
    g = torch.Generator().manual_seed(7)
    rnd = lambda: torch.randn(n, generator=g, dtype=torch.float64)
    z, az, pp, qp, r = (rnd().float().to(cuda) for _ in range(5))
    x = rnd().to(cuda)
    scratch = torch.empty(L.ngb_fcg_scratch_doubles(n), dtype=torch.float64, device=cuda)
    scal = torch.tensor([0.37, 0.0, 0.0, 0.0, 1.9], dtype=torch.float64, device=cuda)  # zq, rr, pq, pr, pq_prev
    P = lambda t: ctypes.c_void_p(t.data_ptr())
    z0, az0, r0, x0 = z.double(), az.double(), r.double(), x.clone()
    coef = 0.37 / 1.9
    assert L.ngb_fcg_direction(n, P(z), P(az), P(pp), P(qp), P(r), P(scal[0:1]), P(scal[4:5]), P(scal[2:4]), P(scratch),
                               None) == 0
    p_ref = z0 - coef * pp.double()
    q_ref = az0 - coef * qp.double()
    assert float((z.double() - p_ref).abs().max()) <= 1e-6 * float(p_ref.abs().max())
    assert float((az.double() - q_ref).abs().max()) <= 1e-6 * float(q_ref.abs().max())
    pq, pr = float((z.double() * az.double()).sum()), float((z.double() * r0).sum())
    assert abs(float(scal[2]) - pq) <= 1e-9 * float((z.double() * az.double()).abs().sum())
    assert abs(float(scal[3]) - pr) <= 1e-9 * float((z.double() * r0).abs().sum())
    assert L.ngb_fcg_update(n, P(x), P(z), P(r), P(az), P(scal[2:4]), P(scal[1:2]), P(scratch), None) == 0
    alpha = float(scal[3]) / float(scal[2])
    assert float((x - (x0 + alpha * z.double())).abs().max()) <= 1e-12 * float(x0.abs().max())
    r_ref = r0 - alpha * az.double()
    assert float((r.double() - r_ref).abs().max()) <= 1e-6 * float(r_ref.abs().max())
    assert abs(float(scal[1]) - float((r.double() ** 2).sum())) <= 1e-9 * float((r.double() ** 2).sum())
    # first direction: z and az are left as they are
    z1 = z.clone()
    assert L.ngb_fcg_direction(n, P(z), P(az), None, None, P(r), None, None, P(scal[2:4]), P(scratch), None) == 0
    assert torch.equal(z, z1)


def test_network_device_apply_matches_forward(ngb, cuda):
    """UNet.apply (scale kept on the device, ngb_unet_input / ngb_unet_output)
    against the torch-glued forward on the same weights: equal up to the BF16
    rounding of an input whose scale differs in the last bit."""
    import torch
    from neon_gb300 import fcg
    from neon_gb300.learned import UNet
    n = 32
    net = UNet(seed=3, device=cuda)
    r = fcg.grf_k2(n, 5, cuda)
    e = torch.full_like(r, float("nan"))
    net.apply(r, e, 16.0)
    net.check()
    ref = net.forward(r) * 16.0 * fcg.free_mask(n, cuda)
    torch.cuda.synchronize()
    assert torch.isfinite(e).all()
    assert float((e - ref).abs().max()) <= 1e-2 * float(ref.abs().max())
    assert float(e.reshape(n, n, n)[0].abs().max()) == 0.0  # faces


def test_scale_by_ratio(ngb, cuda):
    import ctypes
    import torch
    L = ngb.lib()
    P = lambda t: ctypes.c_void_p(t.data_ptr())
    e = torch.arange(1000, dtype=torch.float32, device=cuda)
    s = torch.tensor([3.0, 4.0, -1.0], dtype=torch.float64, device=cuda)
    assert L.ngb_scale_by_ratio(1000, P(e), P(s[0:1]), P(s[1:2]), None) == 0
    torch.cuda.synchronize()
    assert torch.equal(e, torch.arange(1000, dtype=torch.float32, device=cuda) * 0.75)
    assert L.ngb_scale_by_ratio(1000, P(e), P(s[2:3]), P(s[1:2]), None) == 0  # a negative step is no step
    torch.cuda.synchronize()
    assert float(e.abs().max()) == 0.0
