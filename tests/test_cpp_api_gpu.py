"""The C++ Neon API (include/Neon/**) on the GPU: programs written like Neon's
own tests and apps (tests/cpp/*.cu) are compiled with nvcc against the
headers and the C-ABI library, run, and their outputs compared with the
oracle."""
import concurrent.futures as cf
import os
import subprocess

import numpy as np
import pytest

from helpers import P

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CPP = os.path.join(ROOT, "tests", "cpp")
BUILD = os.path.join(CPP, "_build")
PROGRAMS = ["api_stencil", "api_lbm", "api_poisson", "api_dataview", "api_learned"]


def _compile(name):
    import importlib
    b = importlib.import_module("neon_gb300.build")
    exe = os.path.join(BUILD, name)
    src = os.path.join(CPP, name + ".cu")
    libdir = os.path.dirname(b.LIB_PATH)
    cmd = [b.nvcc(), "-std=c++17", "--extended-lambda", "--expt-relaxed-constexpr", "-O2", "--fmad=false",
           "-gencode", "arch=compute_103a,code=sm_103a", "-I", os.path.join(ROOT, "include"), src, "-o", exe,
           "-L", libdir, "-lneon_gb300", "-Xlinker", "-rpath," + libdir]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-4000:]
    return exe


@pytest.fixture(scope="module")
def programs(ngb):
    os.makedirs(BUILD, exist_ok=True)
    with cf.ThreadPoolExecutor(len(PROGRAMS)) as ex:
        exes = list(ex.map(_compile, PROGRAMS))
    return dict(zip(PROGRAMS, exes))


def _run(exe, *args):
    r = subprocess.run([exe] + [str(a) for a in args], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, (r.stdout[-2000:], r.stderr[-2000:])
    return r.stdout


def test_domain_and_skeleton_stencil(programs, orc, tmp_path):
    out = _run(programs["api_stencil"], tmp_path)
    assert out.count("stencil-throw=1") == 9, out
    for grid, dims in [(g, d) for d in [(10, 17, 13), (1, 1, 100), (17, 1, 77)] for g in ("dGrid", "eGrid")] + \
                      [("bGrid", d) for d in [(10, 17, 24), (1, 1, 100), (17, 1, 77)]]:
        nx, ny, nz = dims
        V = nx * ny * nz
        x0 = np.zeros(V, np.int64)
        orc.orc_masked_values_i64(nx, ny, nz, 1, 3, P(x0))
        y, x = np.zeros(V, np.int64), np.zeros(V, np.int64)
        orc.orc_laplace_i64(nx, ny, nz, None, P(x0), P(y))
        orc.orc_laplace_i64(nx, ny, nz, None, P(y), P(x))
        tag = tmp_path / ("%s_%dx%dx%d" % (grid, nx, ny, nz))
        assert np.array_equal(np.fromfile(str(tag) + "_run_Y.bin", np.int64), y)
        assert np.array_equal(np.fromfile(str(tag) + "_run_X.bin", np.int64), x)
        xs = x0.copy()
        for _ in range(5):
            orc.orc_laplace_i64(nx, ny, nz, None, P(xs), P(y))
            orc.orc_laplace_i64(nx, ny, nz, None, P(y), P(xs))
        assert np.array_equal(np.fromfile(str(tag) + "_skel_X.bin", np.int64), xs)


def test_egrid_sparse_stencil(programs, orc, tmp_path):
    """eGrid on a sparse domain through newContainer: inactive cells are not
    neighbours (the oracle's TestData::laplace with the same activity map)."""
    out = _run(programs["api_stencil"], tmp_path)
    nx, ny, nz = 19, 11, 23
    z, y, x = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    act = ((x + y + z) % 3 != 0).astype(np.uint8).ravel()
    assert "eGrid sparse 19x11x23 elements=%d" % int(act.sum()) in out, out
    x0 = np.zeros(nx * ny * nz, np.int64)
    orc.orc_masked_values_i64(nx, ny, nz, 1, 3, P(x0))
    y0 = np.zeros_like(x0)
    orc.orc_laplace_i64(nx, ny, nz, P(act), P(x0), P(y0))
    got = np.fromfile(str(tmp_path / "eGrid_19x11x23_sparse_Y.bin"), np.int64)
    m = act.astype(bool)
    assert np.array_equal(got[m], y0[m])


def test_lbm_cavity_user_and_gb300_containers(programs, orc, tmp_path):
    from helpers import oracle_cavity
    _run(programs["api_lbm"], tmp_path)
    ref, _, _ = oracle_cavity(orc, 24, 19, 0, 60)
    for name in ("cavity_user", "cavity_gb300", "cavity_bgrid", "cavity_bgrid_user"):
        got = np.fromfile(str(tmp_path / (name + ".bin")), np.float64)
        # FP64 reference arithmetic everywhere (the user lambda is compiled with --fmad=false)
        assert np.array_equal(got, ref), (name, float(np.abs(got - ref).max()))


def test_poisson_cg_t(programs, orc, tmp_path):
    n = 40
    c = np.zeros(24)
    a = np.zeros(8)
    orc.orc_gaussian_sources(n, n, n, 5, P(c), P(a))
    z, y, x = np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij")
    f = np.zeros((n, n, n))
    for k in range(8):
        f += a[k] * np.exp(-((x - c[3 * k]) ** 2 + (y - c[3 * k + 1]) ** 2 + (z - c[3 * k + 2]) ** 2) / (2 * 1.5 ** 2))
    b = f.astype(np.float32).ravel()
    b.tofile(str(tmp_path / "poisson_b.bin"))
    out = _run(programs["api_poisson"], tmp_path, n)
    assert "status=0" in out, out
    xg = np.fromfile(str(tmp_path / "poisson_x.bin"), np.float32).astype(np.float64)
    bd = np.zeros(n ** 3, np.int8)
    orc.orc_box_boundary(n, n, n, P(bd))
    xo = np.zeros(n ** 3)
    res = np.zeros(4)
    orc.orc_pcg_f32(n, n, n, 1.0, P(bd), P(b), P(xo), 1e-8, 5000, 50, P(res), 1)
    assert res[1] == 1
    its = int(out.split("iterations=")[1].split()[0])
    assert abs(its - res[0]) <= 2, (its, res[0])
    # the program returns x rounded to float (the field type)
    assert np.linalg.norm(xg - xo) / np.linalg.norm(xo) <= 1e-6


def test_data_views_and_occ(programs):
    """DataView INTERNAL / BOUNDARY spans of one partition (dGrid: the
    stencil's z planes at both ends are BOUNDARY; bGrid: every block is
    internal) and a Skeleton with Occ::standard give the STANDARD result."""
    out = _run(programs["api_dataview"])
    assert out.count("ok=1") == 8 and "ok=0" not in out, out


def test_learned_fcg_t(programs, ngb, cuda, tmp_path):
    """LearnedFCG_t::solve through the C++ API on the 128^3 Gaussian-source
    problem (weights from a file written by the library): converges to 1e-8
    with the iteration count of the C-ABI solve (the same calls) and of the
    Python orchestration within +-2."""
    import torch
    from neon_gb300 import fcg
    from neon_gb300.learned import UNet
    n, levels = 128, 1
    net = UNet(seed=0, device=cuda)
    wpath = tmp_path / "unet.ngbw"
    net.save_weights(wpath)
    net.load_weights(wpath)  # the BF16 values the file holds, so both paths run the same network
    d = ngb.poisson_desc(n, n, n, "f32", 1.0)
    c, a = ngb.gaussian_sources(n, n, n, 2024)
    b = torch.empty(n ** 3, dtype=torch.float32, device=cuda)
    ngb.poisson_rhs(d, torch.from_numpy(c).to(cuda), torch.from_numpy(a).to(cuda), 8.0, b)
    b.cpu().numpy().tofile(str(tmp_path / "poisson_b.bin"))
    out = _run(programs["api_learned"], tmp_path, n, wpath, levels)
    assert "status=0" in out, out
    its = int(out.split("iterations=")[1].split()[0])
    x = torch.zeros(n ** 3, dtype=torch.float64, device=cuda)
    ref = fcg.fcg_solve_vcycle(fcg.VCycle(n, levels, net, device=cuda), b, x, tol=1e-8, max_iter=2000, fallback=True)
    assert ref["converged"]
    assert abs(its - (ref["iterations"] + ref["fallback_iterations"])) <= 2, (out, ref)


def test_learned_fcg_t_committed_weights(programs, ngb, cuda, tmp_path):
    """LearnedFCG_t with the committed trained network
    (neon_gb300/weights/unet_poisson_64.ngbw: trained at 64^3 on solver pairs
    of k^-2 fields by bench.py --workload learned --train-n 64) on the 128^3
    Gaussian-source problem, one V-cycle level above the network: reaches
    1e-8 without the Jacobi-PCG fallback, in the iteration count of the
    Python orchestration of the same kernels (+-2), and in far fewer
    iterations than the same cycle without the network."""
    import torch
    from neon_gb300 import fcg
    from neon_gb300.learned import UNet
    n, levels = 128, 1
    wpath = os.path.join(ROOT, "neon_gb300", "weights", "unet_poisson_64.ngbw")
    net = UNet(seed=0, device=cuda)
    net.load_weights(wpath)
    d = ngb.poisson_desc(n, n, n, "f32", 1.0)
    c, a = ngb.gaussian_sources(n, n, n, 2024)
    b = torch.empty(n ** 3, dtype=torch.float32, device=cuda)
    ngb.poisson_rhs(d, torch.from_numpy(c).to(cuda), torch.from_numpy(a).to(cuda), 8.0, b)
    b.cpu().numpy().tofile(str(tmp_path / "poisson_b.bin"))
    out = _run(programs["api_learned"], tmp_path, n, wpath, levels)
    assert "status=0" in out and "fallback=0" in out, out
    its = int(out.split("iterations=")[1].split()[0])
    res = float(out.split("residual=")[1].split()[0])
    assert res <= 1e-8, out
    x = torch.zeros(n ** 3, dtype=torch.float64, device=cuda)
    ref = fcg.fcg_solve_vcycle(fcg.VCycle(n, levels, net, device=cuda), b, x, tol=1e-8, max_iter=2000, fallback=True)
    assert ref["converged"] and not ref["fallback"], ref
    assert abs(its - ref["iterations"]) <= 2, (out, ref)
    x0 = torch.zeros_like(x)
    plain = fcg.fcg_solve_vcycle(fcg.VCycle(n, levels, coarse="none", device=cuda), b, x0, tol=1e-8, max_iter=2000, fallback=True)
    assert its * 3 < plain["iterations"] + plain["fallback_iterations"], (its, plain)
