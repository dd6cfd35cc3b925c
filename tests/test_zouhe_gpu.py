"""Zou-He pressure / velocity boundary nodes on the dense grid (flag arrays),
CUDA path through the C ABI against the oracle: the wall mask bit for bit,
FP64 (the reference's arithmetic) and the shifted FP32 form with FP32, FP16
and stochastically rounded FP16 storage bit for bit over 150 steps of a
channel with a velocity inlet and a pressure outlet; and, physically, the
steady channel carries the same mass flux through every cross-section."""
import numpy as np
import pytest

from helpers import P
from zouhe_helpers import channel_flags, channel_init

pytestmark = pytest.mark.gpu

TDT = {0: "float64", 1: "float32", 2: "float16", 4: "float16"}


def _gpu_channel(ngb, cuda, storage, steps, nx, ny, nz, rho_b, u_b, omega):
    import torch
    V = nx * ny * nz
    desc = ngb.lbm_dense_desc(nx, ny, nz, 19, storage, omega, box_cavity=False, zouhe_rho=rho_b, zouhe_u=u_b)
    flags = torch.from_numpy(channel_flags(nx, ny, nz).view(np.int32)).to(cuda)
    ngb.lbm_wall_mask(nx, ny, nz, 19, flags)
    if storage in (0, 1):
        f0 = torch.from_numpy(channel_init(nx, ny, nz, np.float64 if storage == 0 else np.float32)).to(cuda)
    else:
        f0 = torch.zeros(19 * V, dtype=torch.float16, device=cuda)  # g = f - w = 0 at rest
    fa, fb = f0.clone(), f0.clone()
    ngb.lbm_dense_run(desc, fa, fb, steps, flags=flags)
    torch.cuda.synchronize()
    return desc, (fa if steps % 2 == 0 else fb), flags


@pytest.mark.parametrize("storage", [0, 1, 2, 4])
def test_zouhe_channel_bit_exact(ngb, orc, cuda, storage):
    import torch
    nx, ny, nz, steps = 40, 18, 14, 150
    rho_b, u_b, omega = 1.0, (0.05, 0.0, 0.0), 1.2
    _, out, flags = _gpu_channel(ngb, cuda, storage, steps, nx, ny, nz, rho_b, u_b, omega)
    oflags = channel_flags(nx, ny, nz)
    orc.orc_wall_mask(nx, ny, nz, 19, P(oflags))
    assert np.array_equal(flags.cpu().numpy().view(np.uint32), oflags)
    if storage in (0, 1):
        a = channel_init(nx, ny, nz, np.float64 if storage == 0 else np.float32)
    else:
        a = np.zeros(19 * nx * ny * nz, np.uint16)
    b = a.copy()
    orc.orc_set_zouhe(rho_b, *u_b)
    orc.orc_set_dither_seed(0)
    mode = 0 if storage == 0 else 2
    assert orc.orc_lbm_run(nx, ny, nz, 19, storage, mode, 0 if storage == 0 else 1, omega, P(np.zeros((4, 27))), P(oflags),
                           P(a), P(b), steps, 0) == 0
    ref = a if steps % 2 == 0 else b
    got = out.cpu()
    got = got.numpy() if storage in (0, 1) else got.view(torch.int16).numpy().view(np.uint16)
    assert np.array_equal(got.view(np.uint8), ref.view(np.uint8)), int((got != ref).sum())


def test_steady_channel_conserves_mass_flux(ngb, cuda):
    """Velocity inlet u = 0.04, pressure outlet rho = 1: after the transient the
    mass flux sum(rho u_x) through each interior cross-section agrees within
    0.5 % and the density falls from inlet to outlet (the pressure drop that
    drives the flow)."""
    import torch
    nx, ny, nz = 64, 18, 14
    desc, out, flags = _gpu_channel(ngb, cuda, 0, 12000, nx, ny, nz, 1.0, (0.04, 0.0, 0.0), 1.6)
    V = nx * ny * nz
    rho = torch.zeros(V, dtype=torch.float64, device=cuda)
    u = torch.zeros(3 * V, dtype=torch.float64, device=cuda)
    ngb.lbm_dense_macroscopic(desc, out, rho=rho, u=u, flags=flags)
    rho = rho.view(nz, ny, nx).cpu().numpy()
    ux = u.view(3, nz, ny, nx)[0].cpu().numpy()
    flux = (rho * ux)[1:-1, 1:-1, 4:-4].sum(axis=(0, 1))
    assert flux.min() > 0
    assert (flux.max() - flux.min()) / flux.mean() < 5e-3, flux
    mean_rho = rho[1:-1, 1:-1, :].mean(axis=(0, 1))
    assert mean_rho[2] > mean_rho[nx - 3] > 0.99
