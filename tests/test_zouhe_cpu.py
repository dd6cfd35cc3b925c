"""The Zou-He pressure / velocity boundary nodes in the oracle (the project's
definition of the flow-over-sphere benchmark's boundary,
benchmarks/lbm-flow-over-sphere/src/LbmContainers.h:53-290 in the reference):
after a step, a velocity node carries exactly the prescribed normal momentum
and a pressure node exactly the prescribed density, in both forms of the
arithmetic; the wall mask treats Zou-He nodes as fluid."""
import numpy as np
import pytest

from helpers import P
from zouhe_helpers import PRESSURE, VELOCITY, W19, channel_flags, channel_init

C19 = np.array([[-1, 0, 0], [0, -1, 0], [0, 0, -1], [-1, -1, 0], [-1, 1, 0], [-1, 0, -1], [-1, 0, 1], [0, -1, -1],
                [0, -1, 1], [0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1], [1, 1, 0], [1, -1, 0], [1, 0, 1], [1, 0, -1],
                [0, 1, 1], [0, 1, -1]])


def _run(orc, storage, mode, steps, nx=16, ny=10, nz=9, rho_b=1.02, u_b=(0.04, 0.0, 0.0), omega=1.3):
    V = nx * ny * nz
    flags = channel_flags(nx, ny, nz)
    orc.orc_wall_mask(nx, ny, nz, 19, P(flags))
    dt = np.float64 if storage == 0 else np.float32
    a = channel_init(nx, ny, nz, dt)
    b = a.copy()
    orc.orc_set_zouhe(rho_b, *u_b)
    wall = np.zeros((4, 27))
    assert orc.orc_lbm_run(nx, ny, nz, 19, storage, mode, 0 if storage == 0 else 1, omega, P(wall), P(flags), P(a), P(b),
                           steps, 1) == 0
    out = (a if steps % 2 == 0 else b).reshape(19, V).astype(np.float64)
    return out, flags, (nx, ny, nz)


def test_wall_mask_treats_zouhe_nodes_as_fluid(orc):
    nx, ny, nz = 8, 6, 5
    flags = channel_flags(nx, ny, nz)
    orc.orc_wall_mask(nx, ny, nz, 19, P(flags))
    f = flags.reshape(nz, ny, nx)
    inlet = int(f[2, 2, 0])
    assert inlet >> 28 == VELOCITY
    mask = inlet & 0x07ffffff
    # the 5 directions pulled from x = -1 are masked, the x = 0 neighbours are not
    for q in range(19):
        if q == 9:
            continue
        assert bool(mask >> q & 1) == (C19[q][0] == 1), q
    bulk = int(f[2, 2, 1])
    assert bulk & 0x07ffffff == 0  # its x-neighbour is a Zou-He node: fluid


@pytest.mark.parametrize("storage,mode", [(0, 0), (1, 2)])
def test_zouhe_nodes_carry_the_boundary_values(orc, storage, mode):
    rho_b, u_b = 1.02, (0.04, 0.0, 0.0)
    out, flags, (nx, ny, nz) = _run(orc, storage, mode, 7, rho_b=rho_b, u_b=u_b)
    cls = flags >> 28
    f = out if storage == 0 else out  # populations (FP32 storage holds f)
    rho = f.sum(axis=0)
    jx = (C19[:, 0][:, None] * f).sum(axis=0)
    tol = 1e-13 if storage == 0 else 2e-6
    vel = np.where(cls == VELOCITY)[0]
    assert np.abs(jx[vel] - rho[vel] * u_b[0]).max() <= tol  # normal momentum rho u_b
    prs = np.where(cls == PRESSURE)[0]
    assert np.abs(rho[prs] - rho_b).max() <= tol  # density rho_b
