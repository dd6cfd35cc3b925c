"""CPU checks of the oracle itself (no GPU): storage conversions against
numpy / torch, agreement of the two D3Q19 restatements, conservation and
symmetry properties of the cavity."""
import numpy as np
import pytest

from helpers import P, oracle_cavity, oracle_velocity, rel_max


def test_f16_conversion_matches_numpy(orc):
    rng = np.random.default_rng(1)
    x = np.concatenate([rng.standard_normal(200000).astype(np.float32) * s for s in (1e-8, 1e-5, 1e-2, 1, 1e3, 7e4)])
    x = np.concatenate([x, np.array([0.0, -0.0, 65504, 65520, 65519.99, 6e-8, 2.98e-8, 1e-9, np.inf, -np.inf], np.float32)])
    out = np.zeros(x.size, np.uint16)
    orc.orc_f32_to_f16(P(x), P(out), x.size)
    assert np.array_equal(out, x.astype(np.float16).view(np.uint16))
    back = np.zeros(x.size, np.float32)
    orc.orc_f16_to_f32(P(out), P(back), x.size)
    assert np.array_equal(back, out.view(np.float16).astype(np.float32))


def test_bf16_conversion_matches_torch(orc):
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(2)
    x = np.concatenate([rng.standard_normal(100000).astype(np.float32) * s for s in (1e-30, 1e-3, 1, 1e30)])
    out = np.zeros(x.size, np.uint16)
    orc.orc_f32_to_bf16(P(x), P(out), x.size)
    ref = torch.from_numpy(x).to(torch.bfloat16).view(torch.int16).numpy().view(np.uint16)
    assert np.array_equal(out, ref)


def test_d3q19_reference_and_generic_forms_agree(orc):
    """The unrolled reference arithmetic and the per-direction BGK are two
    restatements of the same step: FP64 results agree to rounding."""
    a, flags, _ = oracle_cavity(orc, 16, 19, 0, 100, mode=0)
    b, _, _ = oracle_cavity(orc, 16, 19, 0, 100, mode=1, compute_float=0)
    assert rel_max(a, b) < 1e-13


def test_cavity_mass_conservation_and_symmetry(orc):
    n = 20
    pop, flags, _ = oracle_cavity(orc, n, 19, 0, 300)
    bulk = (flags >> 28) == 2
    mass = pop.reshape(19, -1)[:, bulk].sum()
    assert abs(mass - bulk.sum()) < 1e-9 * bulk.sum()
    u = oracle_velocity(orc, n, 19, 0, flags, pop).reshape(3, n, n, n)  # [a][z][y][x]
    # mirror symmetry z -> n-1-z: u_x, u_y even, u_z odd
    assert np.abs(u[0] - u[0][::-1]).max() < 1e-13
    assert np.abs(u[2] + u[2][::-1]).max() < 1e-13
    # the lid drags the fluid: positive u_x just below the lid
    assert u[0][n // 2, n - 2, n // 2] > 0.01


def test_d3q27_mass_conservation(orc):
    n = 14
    pop, flags, _ = oracle_cavity(orc, n, 27, 0, 100)
    bulk = (flags >> 28) == 2
    assert abs(pop.reshape(27, -1)[:, bulk].sum() - bulk.sum()) < 1e-9 * bulk.sum()


def test_wall_mask_semantics(orc):
    """Bit q of a bulk cell is set iff x - c_q is a wall (LbmTools.h:327-376)."""
    import neon_gb300 as ngb
    n = 6
    flags = np.zeros(n ** 3, np.uint32)
    orc.orc_cavity_flags(n, n, n, 19, P(flags))
    f = flags.reshape(n, n, n)
    for (z, y, x) in [(1, 1, 1), (2, 2, 2), (1, 4, 3), (4, 4, 4)]:
        mask = int(f[z, y, x]) & 0x7ffffff
        for q, c in enumerate(ngb.C19):
            sx, sy, sz = x - c[0], y - c[1], z - c[2]
            wall = sx in (0, n - 1) or sy in (0, n - 1) or sz in (0, n - 1)
            assert bool(mask >> q & 1) == (wall and c != (0, 0, 0))


def test_cavity_profiles_format(tmp_path):
    """Centre-line profiles as the reference's cavity run writes them
    (RunCavityTwoPop.cu:110-148): u_x / ulid along y at (nx/2, nz/2),
    u_y / ulid along x at (ny/2, nz/2), "%g %g" lines, 5-digit iteration."""
    import neon_gb300 as ngb
    nx, ny, nz = 6, 5, 4
    u = np.zeros((3, nz, ny, nx))
    u[0] = np.arange(nx * ny * nz).reshape(nz, ny, nx) * 0.01
    u[1] = -np.arange(nx * ny * nz).reshape(nz, ny, nx) * 0.02
    xp, yp = ngb.cavity_profiles(u.ravel(), nx, ny, nz, 0.1)
    assert [p for p, _ in yp] == [y / ny for y in range(ny)]
    assert np.allclose([v for _, v in yp], [u[0, 2, y, 3] / 0.1 for y in range(ny)])
    assert np.allclose([v for _, v in xp], [u[1, 2, 2, x] / 0.1 for x in range(nx)])
    py, px = ngb.write_cavity_profiles(str(tmp_path), 42, xp, yp)
    assert py.endswith("NeonUniformLBM_00042_Y.dat") and px.endswith("NeonUniformLBM_00042_X.dat")
    lines = open(py).read().splitlines()
    assert len(lines) == ny and lines[1] == "%g %g" % (yp[1][0], yp[1][1])


def test_cpu_baselines_quick():
    """The CPU-baseline report runs (tiny sizes) and its numbers are sane."""
    from oracle import cpu_baselines
    out = cpu_baselines.main(quick=True)
    assert all(r["mlups"] > 0 for r in out["lbm_d3q19_f32_cavity"])
    assert all(r["mlups_active"] > 0 and r["active_cells"] > 0 for r in out["lbm_d3q19_f32_sphere"])
    assert all(r["converged"] for r in out["poisson_jacobi_pcg_f32"])
