"""The C++ oracle against the committed golden known-answer vectors
(tests/golden/neon_kat.npz, made by tests/golden/make_golden.py from numpy
restatements of Neon's domain-stencil KAT, bGrid construction and D3Q19
cavity): integer and index results bit for bit, FP64 populations to 1e-13."""
import os

import numpy as np
import pytest

from bgrid_helpers import oracle_bgrid
from helpers import P, oracle_cavity, rel_max

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "neon_kat.npz")


@pytest.fixture(scope="module")
def kat():
    return np.load(GOLDEN)


@pytest.mark.parametrize("tag", ["full", "sparse"])
def test_oracle_integer_laplace_matches_golden(orc, kat, tag):
    nx, ny, nz = (int(v) for v in kat["lap_%s_dims" % tag])
    active = kat["lap_%s_active" % tag]
    x0 = np.zeros(nx * ny * nz, np.int64)
    orc.orc_masked_values_i64(nx, ny, nz, 1, 3, P(x0))
    y = np.zeros_like(x0)
    x = np.zeros_like(x0)
    orc.orc_laplace_i64(nx, ny, nz, P(active), P(x0), P(y))
    orc.orc_laplace_i64(nx, ny, nz, P(active), P(y), P(x))
    act = active.astype(bool)
    assert np.array_equal(y[act], kat["lap_%s_y" % tag][act])
    assert np.array_equal(x[act], kat["lap_%s_x" % tag][act])


def test_oracle_bgrid_matches_golden(orc, kat):
    nx, ny, nz = (int(v) for v in kat["bg_dims"])
    nb, origin, mask, conn, cnt = oracle_bgrid(orc, nx, ny, nz, kat["bg_active"])
    assert nb == kat["bg_origin"].shape[0]
    assert np.array_equal(origin, kat["bg_origin"])
    assert np.array_equal(mask, kat["bg_mask"])
    assert np.array_equal(conn, kat["bg_conn"])
    assert cnt == int(kat["bg_nactive"])


def test_oracle_cavity_matches_golden(orc, kat):
    n, steps = int(kat["cav_n"]), int(kat["cav_steps"])
    pops, _, omega = oracle_cavity(orc, n, 19, 0, steps)
    assert abs(omega - float(kat["cav_omega"])) <= 1e-15
    assert rel_max(pops, kat["cav_pops"]) <= 1e-13


def test_golden_fixture_regenerates(tmp_path, kat):
    """The committed vectors are what tests/golden/make_golden.py produces."""
    import importlib.util
    spec = importlib.util.spec_from_file_location(
        "make_golden", os.path.join(os.path.dirname(GOLDEN), "make_golden.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    out = str(tmp_path / "kat.npz")
    mod.main(out)
    fresh = np.load(out)
    assert sorted(fresh.files) == sorted(kat.files)
    for k in kat.files:
        if kat[k].dtype.kind == "f":  # FP64 sums may round differently under another BLAS
            assert np.allclose(fresh[k], kat[k], rtol=1e-13, atol=0), k
        else:
            assert np.array_equal(fresh[k], kat[k]), k


@pytest.mark.parametrize("n,steps", [(6, 1), (9, 7), (14, 25)])
def test_oracle_cavity_matches_numpy_restatement(orc, n, steps):
    """The C++ oracle's reference-arithmetic D3Q19 cavity against the numpy
    restatement that made the golden vectors, at other sizes and step counts."""
    import importlib.util
    spec = importlib.util.spec_from_file_location(
        "make_golden", os.path.join(os.path.dirname(GOLDEN), "make_golden.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    ref, omega = mod.cavity_d3q19_f64(n, steps)
    pops, _, omega2 = oracle_cavity(orc, n, 19, 0, steps)
    assert abs(omega - omega2) <= 1e-15
    assert rel_max(pops, ref) <= 1e-13
