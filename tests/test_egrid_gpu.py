"""eGrid construction on the device (ngb_egrid_count / ngb_egrid_fill)
bit-identical to the oracle: element count, order, global mapping and the
stencil connectivity."""
import numpy as np
import pytest

from helpers import P
from test_egrid_cpu import STENCILS, active_map

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("dims,kind", [((5, 4, 3), "all"), ((17, 9, 11), "random"), ((20, 13, 7), "sphere"), ((1, 1, 9), "random"),
                                       ((130, 67, 41), "random"), ((96, 64, 80), "sphere")])
@pytest.mark.parametrize("stencil", ["s7", "s27", "r2"])
def test_egrid_build_bit_exact(ngb, orc, cuda, dims, kind, stencil):
    import torch
    nx, ny, nz = dims
    act = active_map(dims, kind, 11)
    pts = STENCILS[stencil]
    g = ngb.EGrid(nx, ny, nz, torch.from_numpy(act).to(cuda), pts)
    pa = np.array(pts, np.int8).ravel()
    count = orc.orc_egrid_build(nx, ny, nz, P(act), P(pa), len(pts), None, None)
    origin = np.zeros(3 * max(count, 1), np.int32)
    conn = np.zeros(len(pts) * max(count, 1), np.int32)
    orc.orc_egrid_build(nx, ny, nz, P(act), P(pa), len(pts), P(origin), P(conn))
    assert g.count == count
    assert np.array_equal(g.origin[:3 * count].cpu().numpy(), origin[:3 * count])
    assert np.array_equal(g.conn[:len(pts) * count].cpu().numpy(), conn[:len(pts) * count])
    eo = g.elem_of.cpu().numpy()
    ref = np.full(act.size, -1, np.int32)
    ref[np.flatnonzero(act)] = np.arange(count, dtype=np.int32)
    assert np.array_equal(eo, ref)


def test_egrid_empty_and_invalid(ngb, cuda):
    import torch
    g = ngb.EGrid(4, 4, 4, torch.zeros(64, dtype=torch.uint8, device=cuda), STENCILS["s7"])
    assert g.count == 0
    with pytest.raises(ngb.NeonError):
        ngb.EGrid(0, 4, 4, torch.zeros(1, dtype=torch.uint8, device=cuda), STENCILS["s7"])
    with pytest.raises(ngb.NeonError):
        ngb.EGrid(4, 4, 4, torch.ones(64, dtype=torch.uint8, device=cuda), [(0, 0, 0)] * 65)
