"""GPU parity of the dense LBM step (C-ABI) against the CPU oracle.

Cavity of benchmarks/lbm-lid-driven-cavity-flow (lid u along +x on y = N-1,
Re = 100, nu = u (N-2) / Re, equilibrium start). Tolerances: FP64 1e-12 and
FP32 1e-5 relative (max-norm over all populations); FP16/BF16-offset storage
is compared through the velocity field.
"""
import numpy as np
import pytest

from helpers import P, STORE_DTYPE, oracle_cavity, oracle_velocity, rel_max

pytestmark = pytest.mark.gpu

def _tdtype(storage):
    import torch
    return {0: torch.float64, 1: torch.float32, 2: torch.float16, 3: torch.bfloat16, 4: torch.float16}[storage]


def gpu_cavity(ngb, cuda, n, q, storage, steps, ulb=0.1, re=100.0, box=True, use_run=True):
    import torch
    V = n ** 3
    omega = ngb.cavity_omega(n, ulb, re)
    desc = ngb.lbm_dense_desc(n, n, n, q, storage, omega, ngb.lid_wall_terms(q, ulb), box_cavity=box)
    fa = torch.empty(q * V, dtype=_tdtype(storage), device=cuda)
    fb = torch.empty_like(fa)
    flags = torch.empty(V, dtype=torch.int32, device=cuda)
    ngb.lbm_cavity_init(desc, ulb, fa, fb, flags)
    if use_run:
        ngb.lbm_dense_run(desc, fa, fb, steps, flags=None if box else flags)
    else:
        for t in range(steps):
            src, dst = (fa, fb) if t % 2 == 0 else (fb, fa)
            ngb.lbm_dense_step(desc, src, dst, flags=None if box else flags)
    torch.cuda.synchronize()
    out = fa if steps % 2 == 0 else fb
    return desc, out, flags


def to_numpy_storage(t, storage):
    import torch
    if storage in (2, 3, 4):
        return t.view(torch.int16).cpu().numpy().view(np.uint16)
    return t.cpu().numpy()


def test_flags_match_oracle(ngb, orc, cuda):
    for q in (19, 27):
        n = 12
        _, _, flags = gpu_cavity(ngb, cuda, n, q, 1, 0)
        ref = np.zeros(n ** 3, np.uint32)
        orc.orc_cavity_flags(n, n, n, q, P(ref))
        assert np.array_equal(flags.cpu().numpy().view(np.uint32), ref)


@pytest.mark.parametrize("box", [True, False])
def test_d3q19_f64_cavity_64_1000_steps(ngb, orc, cuda, box):
    """Config 0: D3Q19 BGK cavity, dGrid 64^3, FP64, 1000 steps, all populations <= 1e-12."""
    n, steps = 64, 1000
    _, out, _ = gpu_cavity(ngb, cuda, n, 19, 0, steps, box=box)
    ref, _, _ = oracle_cavity(orc, n, 19, 0, steps)
    err = rel_max(out.cpu().numpy(), ref)
    assert err <= 1e-12, err


def test_d3q19_f32_cavity(ngb, orc, cuda):
    n, steps = 48, 1000
    _, out, _ = gpu_cavity(ngb, cuda, n, 19, 1, steps)
    ref, _, _ = oracle_cavity(orc, n, 19, 1, steps)
    err = rel_max(out.cpu().numpy(), ref)
    assert err <= 1e-5, err


def test_d3q27_f64_cavity(ngb, orc, cuda):
    n, steps = 32, 300
    _, out, _ = gpu_cavity(ngb, cuda, n, 27, 0, steps)
    ref, _, _ = oracle_cavity(orc, n, 27, 0, steps)
    err = rel_max(out.cpu().numpy(), ref)
    assert err <= 1e-12, err


def test_d3q27_f32_cavity(ngb, orc, cuda):
    n, steps = 32, 300
    _, out, _ = gpu_cavity(ngb, cuda, n, 27, 1, steps)
    ref, _, _ = oracle_cavity(orc, n, 27, 1, steps)
    err = rel_max(out.cpu().numpy(), ref)
    assert err <= 1e-5, err


@pytest.mark.parametrize("q", [19, 27])
@pytest.mark.parametrize("storage,tol_vs_f64", [(2, 1e-3), (3, 1e-2)])
def test_offset_storage_velocity(ngb, orc, cuda, q, storage, tol_vs_f64):
    """FP16/BF16 g = f - w storage with FP32 collision, 400 steps: the velocity
    error against the FP64 run is within the target and of the size of the
    oracle's own same-storage error (16-bit rounding noise, not a defect)."""
    import torch
    n, steps = 32, 400
    desc, out, flags = gpu_cavity(ngb, cuda, n, q, storage, steps)
    u = torch.zeros(3 * n ** 3, dtype=torch.float64, device=cuda)
    ngb.lbm_dense_macroscopic(desc, out, u=u)
    u = u.cpu().numpy()
    pop16, oflags, _ = oracle_cavity(orc, n, q, storage, steps)
    u16 = oracle_velocity(orc, n, q, storage, oflags, pop16)
    pop64, _, _ = oracle_cavity(orc, n, q, 0, steps)
    u64 = oracle_velocity(orc, n, q, 0, oflags, pop64)
    nrm = np.linalg.norm(u64)
    e_gpu = np.linalg.norm(u - u64) / nrm
    e_orc = np.linalg.norm(u16 - u64) / nrm
    assert e_gpu <= tol_vs_f64, e_gpu
    assert e_gpu <= 2.0 * e_orc + 1e-5, (e_gpu, e_orc)
    assert np.linalg.norm(u - u16) / nrm <= 3.0 * e_orc + 1e-5


@pytest.mark.parametrize("q", [19, 27])
@pytest.mark.parametrize("storage", [1, 2, 3])
def test_single_step_from_developed_state(ngb, orc, cuda, q, storage):
    """One step from the same developed state (FP64 run, 150 steps, converted
    to the storage form): the GPU's FP32 shifted-form arithmetic is an explicit
    IEEE operation sequence that the oracle mirrors with std::fmaf, so every
    stored value is bit-identical."""
    import torch
    n = 20
    V = n ** 3
    pop64, oflags, omega = oracle_cavity(orc, n, q, 0, 150)
    w = np.array(ngb.lattice(q)[1])
    f = pop64.reshape(q, V)
    if storage == 1:
        src = f.astype(np.float32).ravel()
        tsrc = torch.from_numpy(src.copy())
    else:
        g = (f.astype(np.float32) - w[:, None].astype(np.float32))
        if storage == 2:  # FP16 offsets are stored scaled by 2^14 (NGB_F16OFF_SCALE)
            g = g * np.float32(16384.0)
        tsrc = torch.from_numpy(g.ravel()).to(torch.float16 if storage == 2 else torch.bfloat16)
        src = tsrc.view(torch.int16).numpy().view(np.uint16).copy()
    a = src.copy()
    b = src.copy()
    from helpers import wall_table
    wt = wall_table(q, 0.1, storage)
    assert orc.orc_lbm_run(n, n, n, q, storage, 2, 1, omega, P(wt), P(oflags), P(a), P(b), 1, 0) == 0
    desc = ngb.lbm_dense_desc(n, n, n, q, storage, omega, ngb.lid_wall_terms(q, 0.1))
    fa = tsrc.to(cuda)
    fb = fa.clone()
    ngb.lbm_dense_step(desc, fa, fb)
    torch.cuda.synchronize()
    got = fb.cpu()
    got = got.numpy() if storage == 1 else got.view(torch.int16).numpy().view(np.uint16)
    assert np.array_equal(got.view(np.uint32) if storage == 1 else got, b.view(np.uint32) if storage == 1 else b)


@pytest.mark.parametrize("n", [18, 17])
@pytest.mark.parametrize("q", [19, 27])
@pytest.mark.parametrize("storage", [1, 2, 3, 4])
def test_shifted_forms_bit_exact_over_steps(ngb, orc, cuda, n, q, storage):
    """60 steps from the equilibrium start, even n (two cells per thread) and
    odd n (one cell per thread): bit-identical to the oracle's shifted form."""
    steps = 60
    _, out, _ = gpu_cavity(ngb, cuda, n, q, storage, steps)
    ref, _, _ = oracle_cavity(orc, n, q, storage, steps, mode=2, compute_float=1)
    import torch
    got = out.cpu()
    got = got.numpy().view(np.uint32) if storage == 1 else got.view(torch.int16).numpy().view(np.uint16)
    ref = ref.view(np.uint32) if storage == 1 else ref
    assert np.array_equal(got, ref), int((got != ref).sum())


@pytest.mark.parametrize("dims", [(136, 21, 10), (256, 9, 7)])
@pytest.mark.parametrize("q", [19, 27])
@pytest.mark.parametrize("storage", [1, 2, 3, 4])
@pytest.mark.parametrize("box", [True, False])
def test_non_cubic_bit_exact(ngb, orc, cuda, dims, q, storage, box):
    """Non-cubic lattices: two or three 128-cell x blocks (one partial), an odd
    y count, analytic and flag classification; 40 steps bit-identical to the
    oracle's shifted form."""
    import torch
    nx, ny, nz = dims
    steps, ulb = 40, 0.1
    V = nx * ny * nz
    omega = ngb.cavity_omega(32, ulb, 100.0)
    desc = ngb.lbm_dense_desc(nx, ny, nz, q, storage, omega, ngb.lid_wall_terms(q, ulb), box_cavity=box)
    fa = torch.empty(q * V, dtype=_tdtype(storage), device=cuda)
    fb = torch.empty_like(fa)
    flags = torch.empty(V, dtype=torch.int32, device=cuda)
    ngb.lbm_cavity_init(desc, ulb, fa, fb, flags)
    ngb.lbm_dense_run(desc, fa, fb, steps, flags=None if box else flags)
    torch.cuda.synchronize()
    oflags = np.zeros(V, np.uint32)
    orc.orc_cavity_flags(nx, ny, nz, q, P(oflags))
    a = np.zeros(q * V, STORE_DTYPE[storage])
    orc.orc_cavity_init(nx, ny, nz, q, storage, ulb, P(a))
    b = a.copy()
    from helpers import wall_table
    wt = wall_table(q, ulb, storage)
    assert orc.orc_lbm_run(nx, ny, nz, q, storage, 2, 1, omega, P(wt), P(oflags), P(a), P(b), steps, 0) == 0
    assert np.array_equal(flags.cpu().numpy().view(np.uint32), oflags)
    got = to_numpy_storage(fa, storage)
    got = got.view(np.uint32) if storage == 1 else got
    ref = a.view(np.uint32) if storage == 1 else a
    assert np.array_equal(got, ref), int((got != ref).sum())


@pytest.mark.parametrize("storage", [0, 1, 2])
def test_run_graph_equals_steps_and_is_deterministic(ngb, cuda, storage):
    import torch
    n, steps = 24, 70
    _, a, _ = gpu_cavity(ngb, cuda, n, 19, storage, steps, use_run=True)
    _, b, _ = gpu_cavity(ngb, cuda, n, 19, storage, steps, use_run=False)
    _, c, _ = gpu_cavity(ngb, cuda, n, 19, storage, steps, use_run=True)
    assert torch.equal(a, b)
    assert torch.equal(a, c)


def test_macroscopic_matches_oracle(ngb, orc, cuda):
    import torch
    n, steps = 20, 50
    desc, out, flags = gpu_cavity(ngb, cuda, n, 19, 0, steps)
    u = torch.zeros(3 * n ** 3, dtype=torch.float64, device=cuda)
    rho = torch.zeros(n ** 3, dtype=torch.float64, device=cuda)
    ngb.lbm_dense_macroscopic(desc, out, rho=rho, u=u)
    pop, oflags, _ = oracle_cavity(orc, n, 19, 0, steps)
    uo = oracle_velocity(orc, n, 19, 0, oflags, pop)
    bulk = (oflags >> 28) == 2
    un = u.cpu().numpy().reshape(3, -1)
    assert np.abs(un[:, bulk] - uo.reshape(3, -1)[:, bulk]).max() <= 1e-13
    # moving-wall cells report u_x = lid speed (LbmTools.h:411-427)
    lid = (oflags >> 28) == 1
    assert np.allclose(un[0, lid], 0.1, rtol=1e-12)


def test_invalid_arguments_report_errors(ngb, cuda):
    import ctypes
    import torch
    d = ngb.lbm_dense_desc(8, 8, 8, 19, "f32", 1.0)
    x = torch.empty(19 * 512, device=cuda)
    with pytest.raises(ngb.NeonError, match="distinct"):
        ngb.lbm_dense_step(d, x, x)
    d.q = 7
    with pytest.raises(ngb.NeonError, match="q must be 19 or 27"):
        ngb.lbm_dense_step(d, x, torch.empty_like(x))
    d.q = 19
    d.box_cavity = 0
    with pytest.raises(ngb.NeonError, match="flags required"):
        ngb.lbm_dense_step(d, x, torch.empty_like(x))


def test_cavity_profiles_match_oracle(ngb, orc, cuda):
    """The velocity profiles of an FP64 cavity run: GPU macroscopic field
    against the oracle's computeRhoAndU restatement, bit for bit."""
    import torch
    n, q, steps = 24, 19, 60
    desc = ngb.lbm_dense_desc(n, n, n, q, "f64", ngb.cavity_omega(n, 0.1, 100.0), ngb.lid_wall_terms(q, 0.1))
    fa = torch.empty(q * n ** 3, dtype=torch.float64, device=cuda)
    fb = torch.empty_like(fa)
    ngb.lbm_cavity_init(desc, 0.1, fa, fb)
    ngb.lbm_dense_run(desc, fa, fb, steps)
    u = torch.zeros(3 * n ** 3, dtype=torch.float64, device=cuda)
    ngb.lbm_dense_macroscopic(desc, fa, None, u)
    pop64, oflags, _ = oracle_cavity(orc, n, q, 0, steps)
    uo = oracle_velocity(orc, n, q, 0, oflags, pop64)
    xg, yg = ngb.cavity_profiles(u, n, n, n, 0.1)
    xo, yo = ngb.cavity_profiles(uo, n, n, n, 0.1)
    assert xg == xo and yg == yo


@pytest.mark.parametrize("steps", [3, 4, 37])
def test_run_host_matches_device_run(ngb, cuda, steps):
    """ngb_lbm_dense_run_host (host buffers in and out) returns the same
    populations as the device-resident run, for odd counts too (the result
    then lives in fb, whose wall nodes only the upload initialises)."""
    import torch
    n, q = 20, 19
    desc, ref, _ = gpu_cavity(ngb, cuda, n, q, 1, steps)
    desc2, start, _ = gpu_cavity(ngb, cuda, n, q, 1, 0)
    host_in = start.cpu().pin_memory()
    host_out = torch.full_like(host_in, float("nan")).pin_memory()
    fa = torch.full_like(start, float("nan"))
    fb = torch.full_like(start, float("nan"))  # garbage in fb: its walls must come from the upload
    ngb.lbm_dense_run_host(desc2, host_in, host_out, fa, fb, steps)
    torch.cuda.synchronize()
    assert torch.equal(host_out, ref.cpu())


def test_release_graphs_then_rerun(ngb, cuda):
    """Dropping the cached step graphs changes nothing but the next call's set-up."""
    import torch
    _, a, _ = gpu_cavity(ngb, cuda, 16, 19, 1, 64)
    assert ngb.lib().ngb_lbm_release_graphs() == 0
    _, b, _ = gpu_cavity(ngb, cuda, 16, 19, 1, 64)
    assert torch.equal(a, b)
    # more distinct buffer pairs than the cache holds: old graphs are evicted, results unchanged
    outs = [gpu_cavity(ngb, cuda, 16, 19, 1, 64)[1] for _ in range(10)]
    assert all(torch.equal(o, a) for o in outs)


@pytest.mark.parametrize("storage", [1, 2, 4])
def test_checkpoint_resume_is_bit_identical(ngb, cuda, tmp_path, storage):
    """Save after 64 steps, load into fresh buffers, run 36 more: the same bits
    as 100 uninterrupted steps (the loader fills both ping-pong buffers; with
    stochastic rounding the step seeds continue, as 64 = 0 mod 32)."""
    import torch
    n = 24
    desc, ref, _ = gpu_cavity(ngb, cuda, n, 19, storage, 100)
    desc, mid, _ = gpu_cavity(ngb, cuda, n, 19, storage, 64)
    path = tmp_path / "cavity.ngbl"
    ngb.lbm_dense_save(path, desc, mid, 64)
    fa = torch.full_like(mid, float("nan"))
    fb = torch.full_like(mid, float("nan"))
    assert ngb.lbm_dense_load(path, desc, fa, fb) == 64
    bits = (lambda t: t.view(torch.int16)) if storage != 1 else (lambda t: t)
    assert torch.equal(bits(fa), bits(mid))
    ngb.lbm_dense_run(desc, fa, fb, 36)
    torch.cuda.synchronize()
    assert torch.equal(bits(fa), bits(ref))
