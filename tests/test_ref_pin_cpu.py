"""The oracle against the reference itself.

tests/golden/neon_ref_cavity.npz holds outputs of the reference's own D3Q19
cavity iteration (LbmIterationD3Q19 on Neon's dGrid, run on its CPU backend;
generated by tests/golden/make_ref_golden.py). The oracle's restatement of
LbmTools.h:78-376 must reproduce them bit for bit in FP64 and in FP32.

Where the reference sources are present, the reference is also built from
them (oracle/ref_build.py) and run live against the oracle on further cases.
"""
import ctypes
import math
import os
import sys

import numpy as np
import pytest

from helpers import oracle_cavity

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLD = os.path.join(ROOT, "tests", "golden", "neon_ref_cavity.npz")


def _plane_fsums(pop, n, q=19):
    p = np.asarray(pop, np.float64).reshape(q, n, n * n)
    return np.array([[math.fsum(p[k, z].tolist()) for z in range(n)] for k in range(q)])


@pytest.mark.parametrize("prec,tag", [(0, "f64"), (1, "f32")])
def test_oracle_reproduces_reference_populations(orc, prec, tag):
    g = np.load(GOLD)
    pop, _, omega = oracle_cavity(orc, 12, 19, prec, 150)
    ref = g["%s_n12_s150" % tag]
    assert omega == float(g["%s_n12_s150_omega" % tag]) or prec == 1
    assert pop.dtype == ref.dtype
    assert np.array_equal(pop, ref), int((pop != ref).sum())


@pytest.mark.parametrize("prec,tag", [(0, "f64"), (1, "f32")])
def test_oracle_reproduces_reference_config0_checksums(orc, prec, tag):
    """Config 0 (64^3, 1000 steps): the exactly rounded plane sums of the
    oracle's populations equal the reference's."""
    g = np.load(GOLD)
    pop, _, _ = oracle_cavity(orc, 64, 19, prec, 1000)
    assert np.array_equal(_plane_fsums(pop, 64), g["%s_n64_s1000_planes" % tag])


def _ref_lib():
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import ref_build
    if not ref_build.available():
        pytest.skip("reference sources not present")
    return ref_build.lib()


@pytest.mark.parametrize("n,steps,prec", [(20, 333, 0), (33, 200, 1), (40, 1000, 0)])
def test_live_reference_matches_oracle(orc, n, steps, prec):
    L = _ref_lib()
    out = np.zeros(19 * n ** 3)
    om = ctypes.c_double()
    assert L.ref_cavity_run(n, steps, prec, 0.1, 100.0, out.ctypes.data_as(ctypes.c_void_p), ctypes.byref(om)) == 0
    pop, _, _ = oracle_cavity(orc, n, 19, prec, steps)
    assert np.array_equal(out, pop.astype(np.float64)), int((out != pop).sum())
