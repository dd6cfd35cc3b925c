"""GPU parity of the Poisson path (C-ABI) against the oracle: the 7-point
Laplacian (Fixed/Free rows, LaplacianMatVec.cu:9-99), the FP64-accumulated
deterministic dot, and the mixed-precision Jacobi-PCG (same iteration count,
solution within tolerance, true residual <= 1e-8)."""
import numpy as np
import pytest

from helpers import P

pytestmark = pytest.mark.gpu


def _rhs(orc, n, seed=7, sigma=None):
    c = np.zeros(24)
    a = np.zeros(8)
    orc.orc_gaussian_sources(n, n, n, seed, P(c), P(a))
    z, y, x = np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij")
    sigma = sigma or max(1.0, 8.0 * n / 256)
    f = np.zeros((n, n, n))
    for k in range(8):
        f += a[k] * np.exp(-((x - c[3 * k]) ** 2 + (y - c[3 * k + 1]) ** 2 + (z - c[3 * k + 2]) ** 2) / (2 * sigma ** 2))
    return f.ravel(), c, a, sigma


def test_gaussian_sources_match_oracle(ngb, orc):
    c, a = ngb.gaussian_sources(64, 64, 64, 11)
    c2 = np.zeros(24)
    a2 = np.zeros(8)
    orc.orc_gaussian_sources(64, 64, 64, 11, P(c2), P(a2))
    assert np.array_equal(c, c2) and np.array_equal(a, a2)


@pytest.mark.parametrize("field", ["f32", "f64"])
@pytest.mark.parametrize("with_bd", [False, True])
def test_laplacian_matches_oracle(ngb, orc, cuda, field, with_bd):
    import torch
    nx, ny, nz = 37, 20, 17
    rng = np.random.default_rng(0)
    dt = np.float32 if field == "f32" else np.float64
    u = rng.standard_normal(nx * ny * nz).astype(dt)
    bd = np.zeros(nx * ny * nz, np.int8)
    orc.orc_box_boundary(nx, ny, nz, P(bd))
    if with_bd:
        bd = (rng.random(nx * ny * nz) < 0.8).astype(np.int8)  # arbitrary Fixed/Free pattern
    ref = np.zeros_like(u)
    (orc.orc_laplacian_f32 if field == "f32" else orc.orc_laplacian_f64)(nx, ny, nz, 0.5, P(u), P(bd), P(ref))
    tbd = torch.from_numpy(bd).to(cuda) if with_bd else None
    d = ngb.poisson_desc(nx, ny, nz, field, 0.5, tbd)
    tu = torch.from_numpy(u).to(cuda)
    out = torch.empty_like(tu)
    ngb.laplacian_apply(d, tu, out)
    assert np.array_equal(out.cpu().numpy(), ref)


@pytest.mark.parametrize("n", [1, 1000, 1 << 20, 3_000_001])
def test_dot_fp64_accumulate_deterministic(ngb, cuda, n):
    import torch
    g = torch.Generator().manual_seed(n)
    a = torch.randn(n, generator=g).to(cuda)
    b = torch.randn(n, generator=g).to(cuda)
    r1 = torch.zeros(1, dtype=torch.float64, device=cuda)
    r2 = torch.zeros(1, dtype=torch.float64, device=cuda)
    ngb.dot(a, b, r1)
    ngb.dot(a, b, r2)
    ref = float(np.dot(a.cpu().numpy().astype(np.float64), b.cpu().numpy().astype(np.float64)))
    assert r1.item() == r2.item()
    assert abs(r1.item() - ref) <= 1e-12 * max(1.0, np.sqrt(n))


@pytest.mark.parametrize("field", ["f32", "f64"])
@pytest.mark.parametrize("jacobi", [True, False])
def test_pcg_matches_oracle(ngb, orc, cuda, field, jacobi):
    """Zero-Dirichlet box, Gaussian sources: GPU PCG and the oracle take the
    same number of iterations (+-2) and reach the same solution."""
    import torch
    n = 40
    f, c, a, sigma = _rhs(orc, n)
    dt = np.float32 if field == "f32" else np.float64
    b = f.astype(dt)
    bd = np.zeros(n ** 3, np.int8)
    orc.orc_box_boundary(n, n, n, P(bd))
    xo = np.zeros(n ** 3)
    res = np.zeros(4)
    (orc.orc_pcg_f32 if field == "f32" else orc.orc_pcg_f64)(n, n, n, 1.0, P(bd), P(b), P(xo), 1e-8, 2000, 50, P(res),
                                                              int(jacobi))
    d = ngb.poisson_desc(n, n, n, field, 1.0)
    ws = ngb.cg_workspace(d, cuda)
    tb = torch.from_numpy(b).to(cuda)
    x = torch.zeros(n ** 3, dtype=torch.float64, device=cuda)
    r = ngb.cg_solve(d, tb, x, ws, tol=1e-8, max_iter=2000, refresh_every=50, check_every=20, jacobi=jacobi)
    assert res[1] == 1 and r["converged"]
    assert abs(r["iterations"] - res[0]) <= 2, (r["iterations"], res[0])
    assert r["rel_residual"] <= 1e-8
    xg = x.cpu().numpy()
    assert np.linalg.norm(xg - xo) / np.linalg.norm(xo) <= 1e-7
    # independent check of the true residual in FP64 on the host
    ax = np.zeros(n ** 3)
    orc.orc_laplacian_f64(n, n, n, 1.0, P(xg), P(bd), P(ax))
    free = bd == 1
    assert np.linalg.norm((b.astype(np.float64) - ax)[free]) / np.linalg.norm(b.astype(np.float64)[free]) <= 1e-8


def test_reference_cg_fp64_fixed_iterations(ngb, orc, cuda):
    """Plain CG in FP64 (libNeonSolver sequence), 60 iterations, solution
    within 1e-12 of the oracle's."""
    import torch
    n = 24
    f, *_ = _rhs(orc, n)
    bd = np.zeros(n ** 3, np.int8)
    orc.orc_box_boundary(n, n, n, P(bd))
    xo = np.zeros(n ** 3)
    orc.orc_reference_cg_f64(n, n, n, 1.0, P(bd), P(f), P(xo), 60)
    d = ngb.poisson_desc(n, n, n, "f64", 1.0)
    ws = ngb.cg_workspace(d, cuda)
    x = torch.zeros(n ** 3, dtype=torch.float64, device=cuda)
    r = ngb.cg_solve(d, torch.from_numpy(f).to(cuda), x, ws, tol=0.0, max_iter=60, refresh_every=1000, check_every=60,
                     jacobi=False)
    assert r["iterations"] == 60
    xg = x.cpu().numpy()
    assert np.linalg.norm(xg - xo) / np.linalg.norm(xo) <= 1e-12


def test_rhs_kernel(ngb, orc, cuda):
    import torch
    n = 32
    f, c, a, sigma = _rhs(orc, n)
    d = ngb.poisson_desc(n, n, n, "f64", 1.0)
    out = torch.empty(n ** 3, dtype=torch.float64, device=cuda)
    ngb.poisson_rhs(d, torch.from_numpy(c).to(cuda), torch.from_numpy(a).to(cuda), sigma, out)
    assert np.allclose(out.cpu().numpy(), f, rtol=1e-13, atol=1e-15)


def test_cg_rejects_bad_arguments(ngb, cuda):
    import torch
    d = ngb.poisson_desc(8, 8, 8, "f32", 1.0)
    ws = torch.empty(16, dtype=torch.uint8, device=cuda)
    b = torch.zeros(512, device=cuda)
    x = torch.zeros(512, dtype=torch.float64, device=cuda)
    with pytest.raises(ngb.NeonError, match="workspace too small"):
        ngb.cg_solve(d, b, x, ws)
    d.field = 2
    with pytest.raises(ngb.NeonError, match="field"):
        ngb.cg_solve(d, b, x, ws)
