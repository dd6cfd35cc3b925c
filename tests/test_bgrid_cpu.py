"""CPU checks of the bGrid oracle against an independent numpy restatement of
Neon's single-partition block construction (SpanDecomposition.h:71-96,
SpanClassifier.h:228-237, bGrid_imp.h:80-172) and of the integer
6-neighbour known-answer operator (TestData.h:412-443)."""
import numpy as np
import pytest

from bgrid_helpers import oracle_bgrid
from helpers import P


def numpy_bgrid(nx, ny, nz, active):
    bnx, bny, bnz = (nx + 7) // 8, (ny + 7) // 8, (nz + 7) // 8
    pad = np.zeros((bnz * 8, bny * 8, bnx * 8), bool)
    pad[:nz, :ny, :nx] = active.reshape(nz, ny, nx) != 0
    blocks = pad.reshape(bnz, 8, bny, 8, bnx, 8).transpose(0, 2, 4, 1, 3, 5)  # bz,by,bx,k,j,i
    any_ = blocks.reshape(bnz, bny, bnx, -1).any(-1)
    order = np.flatnonzero(any_.ravel())  # z, y, x fastest
    idx = -np.ones(any_.size, np.int64)
    idx[order] = np.arange(order.size)
    idx = idx.reshape(bnz, bny, bnx)
    bz, by, bx = np.unravel_index(order, any_.shape)
    origin = np.stack([bx * 8, by * 8, bz * 8], 1)
    bits = blocks[bz, by, bx].reshape(order.size, 512)  # bit k*64 + j*8 + i
    mask = np.zeros((order.size, 16), np.uint64)
    for w in range(16):
        mask[:, w] = (bits[:, 32 * w:32 * w + 32].astype(np.uint64) << np.arange(32, dtype=np.uint64)).sum(1)
    conn = np.full((order.size, 27), 0xffffffff, np.uint64)
    for e in range(27):
        di, dj, dk = e % 3 - 1, (e // 3) % 3 - 1, e // 9 - 1
        X, Y, Z = bx + di, by + dj, bz + dk
        ok = (X >= 0) & (Y >= 0) & (Z >= 0) & (X < bnx) & (Y < bny) & (Z < bnz)
        nb = np.full(order.size, -1)
        nb[ok] = idx[Z[ok], Y[ok], X[ok]]
        conn[:, e] = np.where(nb >= 0, nb, 0xffffffff)
    return order.size, origin, mask.astype(np.uint32), conn.astype(np.uint32), int(bits.sum())


CASES = [((10, 17, 24), "full"), ((1, 1, 100), "full"), ((17, 1, 77), "full"), ((33, 20, 19), "random"),
         ((64, 40, 24), "sphere")]


def make_active(dims, kind, seed=3):
    nx, ny, nz = dims
    if kind == "full":
        return np.ones(nx * ny * nz, np.uint8)
    if kind == "random":
        rng = np.random.default_rng(seed)
        return (rng.random(nx * ny * nz) < 0.05).astype(np.uint8)
    z, y, x = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    return (((x - 20) ** 2 + (y - 18) ** 2 + (z - 12) ** 2) <= 100).astype(np.uint8).ravel()


@pytest.mark.parametrize("dims,kind", CASES)
def test_bgrid_oracle_matches_numpy(orc, dims, kind):
    nx, ny, nz = dims
    active = make_active(dims, kind)
    got = oracle_bgrid(orc, nx, ny, nz, active)
    ref = numpy_bgrid(nx, ny, nz, active)
    assert got[0] == ref[0]
    for a, b in zip(got[1:4], ref[1:4]):
        assert np.array_equal(a, b)
    assert got[4] == ref[4]


def numpy_laplace(a, valid):
    """b = a - count * sum(valid neighbours), on [z, y, x] arrays."""
    nz, ny, nx = a.shape
    s = np.zeros_like(a)
    c = np.zeros_like(a)
    for ax in range(3):
        for d in (1, -1):
            sh = np.roll(a, -d, axis=ax)
            vv = np.roll(valid, -d, axis=ax)
            edge = [slice(None)] * 3
            edge[ax] = slice(-1, None) if d == 1 else slice(0, 1)
            vv = vv.copy()
            vv[tuple(edge)] = False
            s += np.where(vv, sh, 0)
            c += vv
    return np.where(valid, a - c * s, 0)


@pytest.mark.parametrize("dims,kind", CASES[:4])
def test_integer_laplace_oracle_matches_numpy(orc, dims, kind):
    nx, ny, nz = dims
    active = make_active(dims, kind)
    a = np.zeros(nx * ny * nz, np.int64)
    orc.orc_masked_values_i64(nx, ny, nz, 1, 3, P(a))
    # spot-check the masked values (IODomain.h:236-250, digit 3): z + 1e3 y + 1e6 x + 1e10 offset
    assert a[5 + nx * (2 + ny * 1)] == 1 + 2 * 1000 + 5 * 10 ** 6 + 10 ** 10 if nx > 5 and ny > 2 and nz > 1 else True
    b = np.zeros_like(a)
    orc.orc_laplace_i64(nx, ny, nz, P(active), P(a), P(b))
    ref = numpy_laplace(a.reshape(nz, ny, nx), active.reshape(nz, ny, nx).astype(bool)).ravel()
    act = active.astype(bool)
    assert np.array_equal(b[act], ref[act])
