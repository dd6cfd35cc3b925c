"""Generate tests/golden/neon_ref_cavity.npz from the reference itself.

Test infrastructure. The values come from the reference's own D3Q19 cavity
iteration (LbmIterationD3Q19 over Neon's dGrid, benchmarks/lbm-lid-driven-
cavity-flow/src/LbmIteration.h, LbmTools.h:78-376), compiled from the
reference's sources and run on its CPU backend by oracle/ref_build.py and
oracle/ref_driver.cu. This script can only run where the reference sources
are (the GPU tests read the committed file):

* ``f64_n12_s150`` / ``f32_n12_s150``: every population of the 12^3 cavity
  after 150 steps, FP64 and FP32 storage/compute (element (x, y, z, q) at
  x + n (y + n z) + q n^3);
* ``f64_n64_s1000_planes`` / ``f32_n64_s1000_planes``: config 0 (64^3, 1000
  steps, lid u = 0.1, Re = 100): the exactly rounded sum (math.fsum) of each
  (q, z) plane of the populations, shape (19, 64), a checksum that is
  independent of summation order;
* the reference's omega for each case.

Run from the repository root: python tests/golden/make_ref_golden.py
"""
import ctypes
import math
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
OUT = os.path.join(HERE, "neon_ref_cavity.npz")


def plane_fsums(pop, n, q=19):
    """math.fsum of each (q, z) plane: shape (q, n)."""
    p = pop.reshape(q, n, n * n)
    return np.array([[math.fsum(p[k, z].tolist()) for z in range(n)] for k in range(q)])


def run(L, n, steps, precision):
    out = np.zeros(19 * n ** 3)
    om = ctypes.c_double()
    rc = L.ref_cavity_run(n, steps, precision, 0.1, 100.0, out.ctypes.data_as(ctypes.c_void_p), ctypes.byref(om))
    if rc != 0:
        raise SystemExit("reference run failed (%d)" % rc)
    return out, om.value


def main():
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import ref_build
    L = ref_build.lib()
    d = {}
    for prec, tag in ((0, "f64"), (1, "f32")):
        pop, om = run(L, 12, 150, prec)
        d["%s_n12_s150" % tag] = pop if prec == 0 else pop.astype(np.float32)
        d["%s_n12_s150_omega" % tag] = np.float64(om)
        pop, om = run(L, 64, 1000, prec)
        d["%s_n64_s1000_planes" % tag] = plane_fsums(pop, 64)
        d["%s_n64_s1000_omega" % tag] = np.float64(om)
    np.savez_compressed(OUT, **d)
    print("wrote", OUT)


if __name__ == "__main__":
    main()
