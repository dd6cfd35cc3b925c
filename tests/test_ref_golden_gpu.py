"""The CUDA path, through the C ABI, against outputs of the reference itself
(tests/golden/neon_ref_cavity.npz: the reference's LbmIterationD3Q19 on Neon's
dGrid, run on its CPU backend; tests/golden/make_ref_golden.py).

FP64 (the reference's arithmetic, LbmTools.h:171-282) must agree bit for bit;
FP32 storage runs the equilibrium-shifted FP32 form, which must stay within
1e-5 relative of the reference's FP32 run (max-norm over all populations)."""
import math
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "neon_ref_cavity.npz")


@pytest.fixture(scope="module")
def ref():
    return np.load(GOLD)


def _run(ngb, cuda, n, steps, storage, box):
    import torch
    ulb = 0.1
    desc = ngb.lbm_dense_desc(n, n, n, 19, storage, ngb.cavity_omega(n, ulb, 100.0), ngb.lid_wall_terms(19, ulb),
                              box_cavity=box)
    dt = torch.float64 if storage == "f64" else torch.float32
    fa = torch.empty(19 * n ** 3, dtype=dt, device=cuda)
    fb = torch.empty_like(fa)
    flags = torch.empty(n ** 3, dtype=torch.int32, device=cuda)
    ngb.lbm_cavity_init(desc, ulb, fa, fb, flags)
    ngb.lbm_dense_run(desc, fa, fb, steps, flags=None if box else flags)
    torch.cuda.synchronize()
    return (fa if steps % 2 == 0 else fb).cpu().numpy()


def _plane_fsums(pop, n, q=19):
    p = np.asarray(pop, np.float64).reshape(q, n, n * n)
    return np.array([[math.fsum(p[k, z].tolist()) for z in range(n)] for k in range(q)])


@pytest.mark.parametrize("box", [True, False])
def test_f64_populations_equal_reference(ngb, cuda, ref, box):
    got = _run(ngb, cuda, 12, 150, "f64", box)
    assert np.array_equal(got, ref["f64_n12_s150"]), int((got != ref["f64_n12_s150"]).sum())


@pytest.mark.parametrize("box", [True, False])
def test_f64_config0_checksums_equal_reference(ngb, cuda, ref, box):
    """Config 0: 64^3, 1000 steps, FP64 - every exactly rounded plane sum equal."""
    got = _run(ngb, cuda, 64, 1000, "f64", box)
    assert np.array_equal(_plane_fsums(got, 64), ref["f64_n64_s1000_planes"])


def test_f32_populations_within_1e5_of_reference(ngb, cuda, ref):
    got = _run(ngb, cuda, 12, 150, "f32", True).astype(np.float64)
    r = ref["f32_n12_s150"].astype(np.float64)
    assert np.abs(got - r).max() / np.abs(r).max() <= 1e-5


def test_f32_config0_checksums_within_1e5_of_reference(ngb, cuda, ref):
    got = _plane_fsums(_run(ngb, cuda, 64, 1000, "f32", True), 64)
    r = ref["f32_n64_s1000_planes"]
    assert np.abs(got - r).max() / np.abs(r).max() <= 1e-5
