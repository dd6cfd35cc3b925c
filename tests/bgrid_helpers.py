"""numpy helpers for bGrid tests: oracle construction, dense <-> per-block layouts."""
import ctypes

import numpy as np

from helpers import P


def oracle_bgrid(orc, nx, ny, nz, active):
    """(n_blocks, origin[nb,3], mask[nb,16], conn[nb,27], n_active) from the oracle."""
    active = np.ascontiguousarray(active, np.uint8)
    cnt = ctypes.c_uint64(0)
    nb = orc.orc_bgrid_build(nx, ny, nz, P(active), None, None, None, 0, ctypes.byref(cnt))
    origin = np.zeros(3 * max(nb, 1), np.int32)
    mask = np.zeros(16 * max(nb, 1), np.uint32)
    conn = np.zeros(27 * max(nb, 1), np.uint32)
    nb2 = orc.orc_bgrid_build(nx, ny, nz, P(active), P(origin), P(mask), P(conn), max(nb, 1), ctypes.byref(cnt))
    assert nb2 == nb
    return nb, origin[:3 * nb].reshape(nb, 3), mask[:16 * nb].reshape(nb, 16), conn[:27 * nb].reshape(nb, 27), cnt.value


def voxel_map(origin, nx, ny, nz):
    """For each (block, voxel): dense linear index, or -1 outside the domain."""
    nb = origin.shape[0]
    v = np.arange(512)
    i, j, k = v & 7, (v >> 3) & 7, v >> 6
    x = origin[:, 0:1] + i[None, :]
    y = origin[:, 1:2] + j[None, :]
    z = origin[:, 2:3] + k[None, :]
    inside = (x < nx) & (y < ny) & (z < nz)
    lin = x + nx * (y + ny * z)
    return np.where(inside, lin, -1).reshape(nb, 512)


def active_voxels(mask):
    """[nb, 512] bool from the 16-word masks."""
    words = mask.astype(np.uint64)
    bits = (words[:, :, None] >> np.arange(32, dtype=np.uint64)[None, None, :]) & 1
    return bits.reshape(mask.shape[0], 512).astype(bool)


def dense_to_bgrid(dense_q, vmap, q):
    """dense [q, V] -> per-block SoA [(b*q + c)*512 + v] (outside-domain voxels 0)."""
    nb = vmap.shape[0]
    out = np.zeros((nb, q, 512), dense_q.dtype)
    ok = vmap >= 0
    for c in range(q):
        vals = np.zeros((nb, 512), dense_q.dtype)
        vals[ok] = dense_q[c][vmap[ok]]
        out[:, c, :] = vals
    return out.ravel()


def bgrid_to_dense(b, vmap, q, V, fill=0):
    nb = vmap.shape[0]
    arr = b.reshape(nb, q, 512)
    out = np.full((q, V), fill, arr.dtype)
    ok = vmap >= 0
    for c in range(q):
        out[c][vmap[ok]] = arr[:, c, :][ok]
    return out
