"""The CUDA path, through the C ABI, against the committed golden
known-answer vectors (tests/golden/neon_kat.npz): integer stencil and bGrid
construction bit for bit, FP64 D3Q19 cavity populations within 1e-12."""
import os

import numpy as np
import pytest

from bgrid_helpers import active_voxels, dense_to_bgrid, voxel_map
from helpers import rel_max

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "neon_kat.npz")


@pytest.fixture(scope="module")
def kat():
    return np.load(GOLDEN)


def _masked(nx, ny, nz):
    z, y, x = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    return (z + y * 10 ** 3 + x * 10 ** 6 + 10 ** 10).astype(np.int64).ravel()


@pytest.mark.parametrize("tag", ["full", "sparse"])
def test_integer_laplace_matches_golden(ngb, cuda, kat, tag):
    import torch
    nx, ny, nz = (int(v) for v in kat["lap_%s_dims" % tag])
    V = nx * ny * nz
    active = kat["lap_%s_active" % tag]
    x0 = _masked(nx, ny, nz)
    y_ref, x_ref = kat["lap_%s_y" % tag], kat["lap_%s_x" % tag]
    if tag == "full":
        X = torch.from_numpy(x0).to(cuda)
        Y = torch.empty_like(X)
        ngb.dense_laplace_i64(nx, ny, nz, X, Y)
        ngb.dense_laplace_i64(nx, ny, nz, Y, X)
        assert np.array_equal(Y.cpu().numpy(), y_ref)
        assert np.array_equal(X.cpu().numpy(), x_ref)
    g = ngb.BGrid(nx, ny, nz, torch.from_numpy(active).to(cuda))
    nb = g.n_blocks
    origin = g.origin[:3 * nb].cpu().numpy().reshape(nb, 3)
    mask = g.mask[:16 * nb].cpu().numpy().view(np.uint32).reshape(nb, 16)
    vmap = voxel_map(origin, nx, ny, nz)
    act = active_voxels(mask)
    X = torch.from_numpy(dense_to_bgrid(x0.reshape(1, V), vmap, 1)).to(cuda)
    Y = torch.zeros_like(X)
    d = g.desc()
    ngb.bgrid_laplace_i64(d, X, Y)
    ngb.bgrid_laplace_i64(d, Y, X)
    assert np.array_equal(Y.cpu().numpy().reshape(nb, 512)[act], y_ref[vmap[act]])
    assert np.array_equal(X.cpu().numpy().reshape(nb, 512)[act], x_ref[vmap[act]])


def test_bgrid_construction_matches_golden(ngb, cuda, kat):
    import torch
    nx, ny, nz = (int(v) for v in kat["bg_dims"])
    g = ngb.BGrid(nx, ny, nz, torch.from_numpy(kat["bg_active"]).to(cuda))
    nb = g.n_blocks
    assert nb == kat["bg_origin"].shape[0]
    assert g.n_active_voxels == int(kat["bg_nactive"])
    assert np.array_equal(g.origin[:3 * nb].cpu().numpy().reshape(nb, 3), kat["bg_origin"])
    assert np.array_equal(g.mask[:16 * nb].cpu().numpy().view(np.uint32).reshape(nb, 16), kat["bg_mask"])
    assert np.array_equal(g.conn[:27 * nb].cpu().numpy().view(np.uint32).reshape(nb, 27), kat["bg_conn"])


@pytest.mark.parametrize("box", [True, False])
def test_cavity_f64_matches_golden(ngb, cuda, kat, box):
    import torch
    n, steps = int(kat["cav_n"]), int(kat["cav_steps"])
    ulb = 0.1
    omega = ngb.cavity_omega(n, ulb, 100.0)
    assert abs(omega - float(kat["cav_omega"])) <= 1e-15
    desc = ngb.lbm_dense_desc(n, n, n, 19, "f64", omega, ngb.lid_wall_terms(19, ulb), box_cavity=box)
    fa = torch.empty(19 * n ** 3, dtype=torch.float64, device=cuda)
    fb = torch.empty_like(fa)
    flags = torch.empty(n ** 3, dtype=torch.int32, device=cuda)
    ngb.lbm_cavity_init(desc, ulb, fa, fb, flags)
    ngb.lbm_dense_run(desc, fa, fb, steps, flags=None if box else flags)
    torch.cuda.synchronize()
    out = (fa if steps % 2 == 0 else fb).cpu().numpy()
    assert rel_max(out, kat["cav_pops"]) <= 1e-12
