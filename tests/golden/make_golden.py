"""Generate the golden known-answer fixtures in tests/golden/neon_kat.npz.

Test infrastructure. Every value is computed here by plain numpy
restatements of Neon's semantics, written independently of the C++ oracle
(oracle/) and of the CUDA library, so the committed vectors pin both:

* integer 6-neighbour operator of the domain-stencil tests
  (libNeonDomain/tests/domain-stencil/src/stencil.cu:128-205 with
  TestData::laplace, libNeonDomain/include/Neon/domain/tools/TestData.h:412-443):
  b = a - count * sum(valid neighbours), a neighbour valid iff inside the box
  and active; inputs are the "masked" values of IODomain.h:236-250
  (z + y 10^3 + x 10^6 + c 10^9 + offset 10^10, digit 3, offset 1), applied
  twice (Y = L(X), X = L(Y)) as the reference test does;
* bGrid single-partition construction (SpanDecomposition.h:71-96,
  SpanClassifier.h:228-237, Partitioner1D.h:212-255, bGrid_imp.h:80-172):
  block order z, y, x-fastest over 8^3 blocks with any active voxel, 16-word
  active masks (bit i + 8j + 64k), 27-entry connectivity (i + 3j + 9k,
  UINT32_MAX where no block);
* D3Q19 BGK lid-driven cavity in FP64 (benchmarks/lbm-lid-driven-cavity-flow:
  D3Q19.h:23-132 lattice, RunCavityTwoPop.cu:159-242 set-up, LbmTools.h:78-376
  pull with half-way bounce-back, computeWallNghMask, BGK, Config.cpp:105-111
  omega), populations after a fixed number of steps.

Run from the repository root: python tests/golden/make_golden.py
"""
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "neon_kat.npz")

# ---------------------------------------------------------------- integer stencil KAT


def masked_values(nx, ny, nz, offset=1, digit=3):
    z, y, x = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    d = 10 ** digit
    return (z + y * d + x * d * d + offset * 10 * d ** 3).astype(np.int64).ravel()


def laplace_i64(nx, ny, nz, active, a):
    act = active.reshape(nz, ny, nx).astype(bool)
    A = a.reshape(nz, ny, nx)
    s = np.zeros_like(A)
    cnt = np.zeros_like(A)
    for axis in range(3):
        for d in (1, -1):
            src = [slice(None)] * 3
            dst = [slice(None)] * 3
            if d == 1:
                dst[axis], src[axis] = slice(0, -1), slice(1, None)
            else:
                dst[axis], src[axis] = slice(1, None), slice(0, -1)
            ok = np.zeros_like(act)
            ok[tuple(dst)] = act[tuple(src)]
            val = np.zeros_like(A)
            val[tuple(dst)] = A[tuple(src)]
            s += np.where(ok, val, 0)
            cnt += ok
    return np.where(act, A - cnt * s, 0).ravel()


# ---------------------------------------------------------------- bGrid construction


def bgrid(nx, ny, nz, active):
    B = 8
    bnx, bny, bnz = -(-nx // B), -(-ny // B), -(-nz // B)
    vox = np.zeros((bnz * B, bny * B, bnx * B), bool)
    vox[:nz, :ny, :nx] = active.reshape(nz, ny, nx).astype(bool)
    blocks = vox.reshape(bnz, B, bny, B, bnx, B).transpose(0, 2, 4, 1, 3, 5).reshape(bnz, bny, bnx, B ** 3)
    live = blocks.any(-1)
    order = np.flatnonzero(live.ravel())
    rank = np.full(live.size, -1, np.int64)
    rank[order] = np.arange(order.size)
    rank = rank.reshape(live.shape)
    bz, by, bx = np.unravel_index(order, live.shape)
    origin = (np.stack([bx, by, bz], 1) * B).astype(np.int32)
    bits = blocks[bz, by, bx]  # [nb, k*64 + j*8 + i]
    weights = (np.uint64(1) << np.arange(32, dtype=np.uint64))
    mask = (bits.reshape(-1, 16, 32).astype(np.uint64) * weights).sum(-1).astype(np.uint32)
    conn = np.full((order.size, 27), 0xFFFFFFFF, np.uint32)
    for e in range(27):
        X, Y, Z = bx + e % 3 - 1, by + (e // 3) % 3 - 1, bz + e // 9 - 1
        inside = (X >= 0) & (Y >= 0) & (Z >= 0) & (X < bnx) & (Y < bny) & (Z < bnz)
        nb = np.full(order.size, -1, np.int64)
        nb[inside] = rank[Z[inside], Y[inside], X[inside]]
        conn[nb >= 0, e] = nb[nb >= 0].astype(np.uint32)
    return origin, mask, conn, int(bits.sum())


# ---------------------------------------------------------------- D3Q19 cavity (FP64)

C19 = np.array([(-1, 0, 0), (0, -1, 0), (0, 0, -1), (-1, -1, 0), (-1, 1, 0), (-1, 0, -1), (-1, 0, 1), (0, -1, -1),
                (0, -1, 1), (0, 0, 0), (1, 0, 0), (0, 1, 0), (0, 0, 1), (1, 1, 0), (1, -1, 0), (1, 0, 1), (1, 0, -1),
                (0, 1, 1), (0, 1, -1)])
W19 = np.array([1 / 3 if q == 9 else (1 / 18 if q % 10 < 3 else 1 / 36) for q in range(19)])
OPP19 = np.array([q + 10 if q < 9 else (q - 10 if q > 9 else 9) for q in range(19)])
BOUNCE, MOVING, BULK = 0, 1, 2


def cavity_d3q19_f64(n, steps, ulb=0.1, re=100.0):
    nu = ulb * (n - 2) / re
    omega = 1.0 / (3.0 * nu + 0.5)
    f = np.empty((19, n, n, n))  # [q][z][y][x]
    cls = np.full((n, n, n), BULK, np.int64)
    face = np.zeros((n, n, n), bool)
    face[0], face[-1], face[:, 0], face[:, -1], face[:, :, 0], face[:, :, -1] = (True,) * 6
    cls[face] = BOUNCE
    cls[:, n - 1, :] = MOVING
    for q in range(19):
        f[q] = W19[q]
        f[q][face] = 0.0
        f[q][:, n - 1, :] = -6.0 * W19[q] * ulb * C19[q][0]
    inner = (slice(1, n - 1),) * 3

    def src(q):  # interior window shifted to x - c_q, [z][y][x]
        cx, cy, cz = C19[q]
        return (slice(1 - cz, n - 1 - cz), slice(1 - cy, n - 1 - cy), slice(1 - cx, n - 1 - cx))

    bulk = cls[inner] == BULK
    wall = [cls[src(q)] != BULK for q in range(19)]
    for _ in range(steps):
        pop = np.empty((19,) + bulk.shape)
        for q in range(19):
            o = OPP19[q]
            pop[q] = np.where(wall[q], f[o][inner] + f[o][src(q)], f[q][src(q)])
        rho = pop.sum(0)
        u = [np.tensordot(C19[:, a].astype(float), pop, axes=1) / rho for a in range(3)]
        usqr = 1.5 * (u[0] ** 2 + u[1] ** 2 + u[2] ** 2)
        g = f.copy()
        for q in range(19):
            cu = C19[q][0] * u[0] + C19[q][1] * u[1] + C19[q][2] * u[2]
            eq = rho * W19[q] * (1.0 + 3.0 * cu + 4.5 * cu * cu - usqr)
            g[q][inner] = np.where(bulk, (1.0 - omega) * pop[q] + omega * eq, f[q][inner])
        f = g
    return f.reshape(19, -1).ravel(), omega


def main(out=OUT):
    rng = np.random.default_rng(3)
    data = {}
    # integer stencil on the domain-stencil test box and a sparse random domain
    for tag, (nx, ny, nz), frac in (("full", (10, 17, 24), 1.0), ("sparse", (33, 20, 19), 0.05)):
        active = (np.ones(nx * ny * nz, np.uint8) if frac == 1.0 else
                  (rng.random(nx * ny * nz) < frac).astype(np.uint8))
        x0 = masked_values(nx, ny, nz)
        y = laplace_i64(nx, ny, nz, active, x0)
        x = laplace_i64(nx, ny, nz, active, y)
        data["lap_%s_dims" % tag] = np.array([nx, ny, nz], np.int32)
        data["lap_%s_active" % tag] = active
        data["lap_%s_y" % tag] = y
        data["lap_%s_x" % tag] = x
    # bGrid construction: a sphere inside a box that is not a multiple of 8
    nx, ny, nz = 64, 40, 24
    z, yy, xx = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    active = (((xx - 20) ** 2 + (yy - 18) ** 2 + (z - 12) ** 2) <= 100).astype(np.uint8).ravel()
    origin, mask, conn, nact = bgrid(nx, ny, nz, active)
    data.update(bg_dims=np.array([nx, ny, nz], np.int32), bg_active=active, bg_origin=origin, bg_mask=mask,
                bg_conn=conn, bg_nactive=np.array(nact, np.int64))
    # D3Q19 FP64 cavity
    n, steps = 10, 60
    pops, omega = cavity_d3q19_f64(n, steps)
    data.update(cav_n=np.array(n), cav_steps=np.array(steps), cav_omega=np.array(omega), cav_pops=pops)
    np.savez_compressed(out, **data)
    print("wrote %s (%d arrays)" % (out, len(data)))


if __name__ == "__main__":
    main()
