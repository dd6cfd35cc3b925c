"""GPU parity of the bGrid path (C-ABI) against the oracle: construction
bit-exact, the integer 6-neighbour known-answer operator exact, the LBM step
on the flow-over-sphere geometry bit-exact (FP32 / 16-bit shifted forms and
the FP64 reference arithmetic), the wall mask and the drag force."""
import numpy as np
import pytest

from bgrid_helpers import active_voxels, bgrid_to_dense, dense_to_bgrid, oracle_bgrid, voxel_map
from helpers import P
from test_bgrid_cpu import CASES, make_active

pytestmark = pytest.mark.gpu


def _tdtype(storage):
    import torch
    return {0: torch.float64, 1: torch.float32, 2: torch.float16, 3: torch.bfloat16, 4: torch.float16}[storage]


@pytest.mark.parametrize("dims,kind", CASES)
def test_bgrid_construction_bit_exact(ngb, orc, cuda, dims, kind):
    import torch
    nx, ny, nz = dims
    active = make_active(dims, kind)
    g = ngb.BGrid(nx, ny, nz, torch.from_numpy(active).to(cuda))
    nb, origin, mask, conn, cnt = oracle_bgrid(orc, nx, ny, nz, active)
    assert g.n_blocks == nb
    assert g.n_active_voxels == cnt
    assert np.array_equal(g.origin[:3 * nb].cpu().numpy().reshape(nb, 3), origin)
    assert np.array_equal(g.mask[:16 * nb].cpu().numpy().view(np.uint32).reshape(nb, 16), mask)
    assert np.array_equal(g.conn[:27 * nb].cpu().numpy().view(np.uint32).reshape(nb, 27), conn)


@pytest.mark.parametrize("dims,kind", CASES[:4])
def test_integer_laplace_known_answer(ngb, orc, cuda, dims, kind):
    """domain-stencil test (libNeonDomain/tests/domain-stencil/src/stencil.cu:128-205):
    masked int64 values, Y = L(X), X = L(Y) on dGrid and bGrid, exact."""
    import torch
    nx, ny, nz = dims
    V = nx * ny * nz
    active = make_active(dims, kind)
    x0 = np.zeros(V, np.int64)
    orc.orc_masked_values_i64(nx, ny, nz, 1, 3, P(x0))
    y_ref = np.zeros(V, np.int64)
    x_ref = np.zeros(V, np.int64)
    orc.orc_laplace_i64(nx, ny, nz, P(active), P(x0), P(y_ref))
    orc.orc_laplace_i64(nx, ny, nz, P(active), P(y_ref), P(x_ref))
    if kind == "full":
        X = torch.from_numpy(x0).to(cuda)
        Y = torch.empty_like(X)
        ngb.dense_laplace_i64(nx, ny, nz, X, Y)
        ngb.dense_laplace_i64(nx, ny, nz, Y, X)
        assert np.array_equal(Y.cpu().numpy(), y_ref)
        assert np.array_equal(X.cpu().numpy(), x_ref)
    g = ngb.BGrid(nx, ny, nz, torch.from_numpy(active).to(cuda))
    nb, origin, mask, _, _ = oracle_bgrid(orc, nx, ny, nz, active)
    vmap = voxel_map(origin, nx, ny, nz)
    act = active_voxels(mask)
    X = torch.from_numpy(dense_to_bgrid(x0.reshape(1, V), vmap, 1)).to(cuda)
    Y = torch.zeros_like(X)
    d = g.desc()
    ngb.bgrid_laplace_i64(d, X, Y)
    ngb.bgrid_laplace_i64(d, Y, X)
    yb = Y.cpu().numpy().reshape(nb, 512)
    xb = X.cpu().numpy().reshape(nb, 512)
    assert np.array_equal(yb[act], y_ref[vmap[act]])
    assert np.array_equal(xb[act], x_ref[vmap[act]])


def small_sphere(ngb, scale):
    return ngb.sphere_config(scale)


def test_geometry_matches_oracle(ngb, orc, cuda):
    import torch
    for scale in (4, 8):
        g = small_sphere(ngb, scale)
        V = g.nx * g.ny * g.nz
        act = torch.zeros(V, dtype=torch.uint8, device=cuda)
        cls = torch.zeros_like(act)
        ngb.geometry_sphere_tube(g, act, cls)
        a_ref = np.zeros(V, np.uint8)
        c_ref = np.zeros(V, np.uint8)
        sc = np.array(list(g.sphere_c))
        tc = np.array(list(g.tube_c))
        orc.orc_sphere_tube(g.nx, g.ny, g.nz, g.ctrl_dx, P(sc), g.sphere_r, g.band, P(tc), g.tube_r, g.tube_band,
                            g.amplitude, g.seed, P(a_ref), P(c_ref))
        assert np.array_equal(act.cpu().numpy(), a_ref)
        assert np.array_equal(cls.cpu().numpy(), c_ref)


def sphere_setup(ngb, orc, cuda, scale, q, storage, u_in=0.05):
    """Dense oracle state + bGrid device state of the scaled sphere case."""
    import torch
    g = small_sphere(ngb, scale)
    nx, ny, nz = g.nx, g.ny, g.nz
    V = nx * ny * nz
    act = torch.zeros(V, dtype=torch.uint8, device=cuda)
    cls = torch.zeros_like(act)
    ngb.geometry_sphere_tube(g, act, cls)
    grid = ngb.BGrid(nx, ny, nz, act)
    terms = ngb.lid_wall_terms(q, u_in)
    omega = 1.0 / (3.0 * 0.02 + 0.5)
    desc = grid.desc(q, storage, omega, moving_wall_terms=terms)
    nb = grid.n_blocks
    flags = torch.zeros(nb * 512, dtype=torch.int32, device=cuda)
    ngb.bgrid_flags_from_dense(desc, nx, ny, nz, cls, flags)
    ngb.bgrid_wall_mask(desc, flags)
    cls_np = cls.cpu().numpy()
    oflags = np.zeros(V, np.uint32)
    orc.orc_flags_from_classes(nx, ny, nz, q, P(cls_np), P(oflags))
    # dense initial state: f = w on fluid, wall terms on moving-wall nodes, 0 elsewhere
    c, w = ngb.lattice(q)
    w = np.array(w)
    klass = oflags >> 28
    fluid = (klass == 2) | (klass == 4)
    f0 = np.zeros((q, V))
    f0[:, fluid] = w[:, None]
    f0[:, klass == 1] = np.array(terms)[:, None]
    origin = grid.origin[:3 * nb].cpu().numpy().reshape(nb, 3)
    vmap = voxel_map(origin, nx, ny, nz)
    return g, grid, desc, flags, oflags, f0, vmap, omega, terms


@pytest.mark.parametrize("q", [19, 27])
@pytest.mark.parametrize("storage", [0, 1, 2, 3])
def test_bgrid_lbm_sphere_bit_exact(ngb, orc, cuda, q, storage):
    """Scaled flow-over-sphere case (64x32x32, velocity inlet, zero-gradient
    outlet, bounce-back sphere and region walls), 40 steps: every active
    fluid voxel equals the dense oracle bit for bit."""
    import torch
    g, grid, desc, flags, oflags, f0, vmap, omega, terms = sphere_setup(ngb, orc, cuda, 8, q, storage)
    nx, ny, nz = g.nx, g.ny, g.nz
    V = nx * ny * nz
    nb = grid.n_blocks
    # flags: the GPU wall mask equals the oracle's on every active voxel
    gf = flags.cpu().numpy().view(np.uint32).reshape(nb, 512)
    act = active_voxels(grid.mask[:16 * nb].cpu().numpy().view(np.uint32).reshape(nb, 16))
    assert np.array_equal(gf[act], oflags[vmap[act]])
    w = np.array(ngb.lattice(q)[1])
    if storage == 0:
        dense = f0.copy()
        dt = np.float64
    elif storage == 1:
        dense = f0.astype(np.float32)
        dt = np.float32
    else:
        dense = np.zeros((q, V), np.uint16)  # g = 0
        dt = np.uint16
    steps = 40
    a = dense.ravel().copy()  # the oracle runs in place: keep `dense` as the initial state
    b = a.copy()
    wall = np.zeros((4, 27))
    wall[1, :q] = [float(np.float32(t)) if storage else t for t in terms]
    # D3Q19 FP64: the reference's unrolled arithmetic; D3Q27 FP64: the generic
    # per-direction form; FP32 / 16-bit: the shifted FP32 form
    mode = (0 if q == 19 else 1) if storage == 0 else 2
    assert orc.orc_lbm_run(nx, ny, nz, q, storage, mode, 0 if storage == 0 else 1, omega, P(wall), P(oflags), P(a), P(b),
                           steps, 0) == 0
    ref = (a if steps % 2 == 0 else b).reshape(q, V)
    init = dense_to_bgrid(dense, vmap, q)
    if storage >= 2:
        t0 = torch.from_numpy(init.view(np.int16)).to(cuda).view(_tdtype(storage))
    else:
        t0 = torch.from_numpy(init).to(cuda)
    t1 = t0.clone()
    for s in range(steps):
        src, dst = (t0, t1) if s % 2 == 0 else (t1, t0)
        ngb.bgrid_lbm_step(desc, src, dst, flags)
    torch.cuda.synchronize()
    out = t0 if steps % 2 == 0 else t1
    out = out.cpu()
    out = out.view(torch.int16).numpy().view(np.uint16) if storage >= 2 else out.numpy()
    ob = out.reshape(nb, q, 512)
    klass = gf >> 28
    fluid = act & ((klass == 2) | (klass == 4))
    for c in range(q):
        got = ob[:, c, :][fluid]
        exp = ref[c][vmap[fluid]]
        assert np.array_equal(got.view(np.uint8), exp.view(np.uint8)), (c, int((got != exp).sum()))


def test_bgrid_drag_matches_numpy(ngb, orc, cuda):
    import torch
    q, storage = 19, 0
    g, grid, desc, flags, oflags, f0, vmap, omega, terms = sphere_setup(ngb, orc, cuda, 8, q, storage)
    nb = grid.n_blocks
    t0 = torch.from_numpy(dense_to_bgrid(f0, vmap, q)).to(cuda)
    t1 = t0.clone()
    for s in range(30):
        src, dst = (t0, t1) if s % 2 == 0 else (t1, t0)
        ngb.bgrid_lbm_step(desc, src, dst, flags)
    partials = torch.zeros(3 * nb, dtype=torch.float64, device=cuda)
    force = torch.zeros(3, dtype=torch.float64, device=cuda)
    ngb.bgrid_drag(desc, t0, flags, partials, force)
    force2 = torch.zeros(3, dtype=torch.float64, device=cuda)
    ngb.bgrid_drag(desc, t0, flags, partials, force2)
    torch.cuda.synchronize()
    assert torch.equal(force, force2)  # deterministic
    # numpy momentum exchange on the dense image
    nx, ny, nz = g.nx, g.ny, g.nz
    V = nx * ny * nz
    dense = bgrid_to_dense(t0.cpu().numpy(), vmap, q, V)
    c, _ = ngb.lattice(q)
    opp = [c.index((-a[0], -a[1], -a[2])) for a in c]
    klass = (oflags >> 28).reshape(nz, ny, nx)
    mask = (oflags & 0x7ffffff).reshape(nz, ny, nx)
    F = np.zeros(3)
    zz, yy, xx = np.nonzero((klass == 2) & (mask != 0))
    for qq in range(q):
        sel = (mask[zz, yy, xx] >> qq) & 1 == 1
        sx, sy, sz = xx[sel] - c[qq][0], yy[sel] - c[qq][1], zz[sel] - c[qq][2]
        ok = (sx >= 0) & (sy >= 0) & (sz >= 0) & (sx < nx) & (sy < ny) & (sz < nz)
        solid = np.zeros(sel.sum(), bool)
        solid[ok] = klass[sz[ok], sy[ok], sx[ok]] == 0
        o = opp[qq]
        fo = dense[o].reshape(nz, ny, nx)[zz[sel][solid], yy[sel][solid], xx[sel][solid]]
        F += 2.0 * np.array(c[o]) * fo.sum()
    got = force.cpu().numpy()
    assert np.allclose(got, F, rtol=1e-12, atol=1e-15), (got, F)
    assert got[0] > 0  # the flow pushes the sphere downstream


@pytest.mark.parametrize("dims,density", [((512, 512, 512), 0.3), ((1000, 904, 200), 0.55), ((8, 8, 8), 1.0)])
def test_block_ranks_many_candidates(ngb, cuda, dims, density):
    """Block ranks over many candidate blocks (262 144 at 512^3: 64 scan tiles;
    a ragged last tile at 1000 x 904 x 200): the active candidates get ranks
    0 .. n-1 in candidate order, the others -1, against numpy."""
    import torch
    nx, ny, nz = dims
    bnx, bny, bnz = (nx + 7) // 8, (ny + 7) // 8, (nz + 7) // 8
    rng = np.random.default_rng(nx + nz)
    on = rng.random(bnx * bny * bnz) < density
    # one active voxel at a random position inside each active block
    act = torch.zeros(nx * ny * nz, dtype=torch.uint8, device=cuda)
    c = np.nonzero(on)[0]
    bx, by, bz = c % bnx, (c // bnx) % bny, c // (bnx * bny)
    x = np.minimum(bx * 8 + rng.integers(0, 8, c.size), nx - 1)
    y = np.minimum(by * 8 + rng.integers(0, 8, c.size), ny - 1)
    z = np.minimum(bz * 8 + rng.integers(0, 8, c.size), nz - 1)
    act[torch.from_numpy(x + nx * (y + ny * z)).to(cuda)] = 1
    block_of = torch.empty(bnx * bny * bnz, dtype=torch.int32, device=cuda)
    nb = torch.zeros(1, dtype=torch.int32, device=cuda)
    ngb.check(ngb.lib().ngb_bgrid_count(nx, ny, nz, ngb._ptr(act), ngb._ptr(block_of), ngb._ptr(nb), None))
    ref = np.where(on, np.cumsum(on) - 1, -1).astype(np.int32)
    assert int(nb.item()) == int(on.sum())
    assert np.array_equal(block_of.cpu().numpy(), ref)
