"""eGrid construction oracle (Partitioner1D at block size 1, one partition)
against an independent numpy restatement: element order, global mapping and
stencil connectivity."""
import numpy as np
import pytest

from helpers import P

STENCILS = {
    "s7": [(1, 0, 0), (-1, 0, 0), (0, 1, 0), (0, -1, 0), (0, 0, 1), (0, 0, -1)],
    "s27": [(x, y, z) for x in (-1, 0, 1) for y in (-1, 0, 1) for z in (-1, 0, 1) if (x, y, z) != (0, 0, 0)],
    "r2": [(2, 0, 0), (-2, 0, 0), (0, 0, 2), (1, -1, 2)],
}


def numpy_egrid(active, dims, points):
    nx, ny, nz = dims
    idx = np.flatnonzero(active)
    count = idx.size
    elem = np.full(active.size, -1, np.int64)
    elem[idx] = np.arange(count)
    x, y, z = idx % nx, (idx // nx) % ny, idx // (nx * ny)
    origin = np.stack([x, y, z], 1).astype(np.int32).ravel()
    conn = np.full((len(points), count), -1, np.int64)
    for s, (px, py, pz) in enumerate(points):
        xx, yy, zz = x + px, y + py, z + pz
        ok = (xx >= 0) & (yy >= 0) & (zz >= 0) & (xx < nx) & (yy < ny) & (zz < nz)
        lin = xx + nx * (yy + ny * zz)
        conn[s, ok] = elem[lin[ok]]
    return count, origin, conn.astype(np.int32).ravel()


def active_map(dims, kind, seed):
    nx, ny, nz = dims
    rng = np.random.default_rng(seed)
    if kind == "all":
        return np.ones(nx * ny * nz, np.uint8)
    if kind == "sphere":
        z, y, x = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
        r = min(dims) / 2.0
        return (((x - nx / 2) ** 2 + (y - ny / 2) ** 2 + (z - nz / 2) ** 2) <= r * r).astype(np.uint8).ravel()
    return (rng.random(nx * ny * nz) < 0.3).astype(np.uint8)


@pytest.mark.parametrize("dims,kind", [((5, 4, 3), "all"), ((17, 9, 11), "random"), ((20, 13, 7), "sphere"), ((1, 1, 9), "random")])
@pytest.mark.parametrize("stencil", ["s7", "s27", "r2"])
def test_egrid_oracle_matches_numpy(orc, dims, kind, stencil):
    nx, ny, nz = dims
    act = active_map(dims, kind, 7)
    pts = STENCILS[stencil]
    pa = np.array(pts, np.int8).ravel()
    count = orc.orc_egrid_build(nx, ny, nz, P(act), P(pa), len(pts), None, None)
    origin = np.zeros(3 * max(count, 1), np.int32)
    conn = np.zeros(len(pts) * max(count, 1), np.int32)
    assert orc.orc_egrid_build(nx, ny, nz, P(act), P(pa), len(pts), P(origin), P(conn)) == count
    c2, o2, k2 = numpy_egrid(act, dims, pts)
    assert count == c2
    assert np.array_equal(origin[:3 * count], o2)
    assert np.array_equal(conn[:len(pts) * count], k2)
