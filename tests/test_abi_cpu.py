"""The C-ABI library loads without a GPU and exports every function that
include/*.h declares; argument validation errors are reported before any
CUDA call."""
import glob
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        src = open(h).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        for m in re.finditer(r"^\s*(?:const\s+)?[A-Za-z_][A-Za-z0-9_]*\s*\*?\s*(ngb_[A-Za-z0-9_]+)\s*\(", src, re.M):
            names.add(m.group(1))
    return sorted(names)


def test_header_declares_entry_points():
    names = declared_functions()
    assert "ngb_lbm_dense_step" in names and "ngb_last_error" in names


def test_library_exports_every_declared_symbol(ngb):
    lib = ngb.lib()
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_validation_without_gpu(ngb):
    import ctypes
    d = ngb.lbm_dense_desc(8, 8, 8, 19, "f32", 1.0)
    d.q = 5
    rc = ngb.lib().ngb_lbm_dense_step(ctypes.byref(d), None, None, None, None)
    assert rc == -1
    assert b"q must be 19 or 27" in ngb.lib().ngb_last_error()
    d.q = 19
    d.nx = 2
    assert ngb.lib().ngb_lbm_dense_step(ctypes.byref(d), None, None, None, None) == -1
    assert b"dims" in ngb.lib().ngb_last_error()


def test_product_package_does_not_import_oracle():
    for f in glob.glob(os.path.join(ROOT, "neon_gb300", "**", "*.py"), recursive=True):
        src = open(f).read()
        assert "import oracle" not in src and "from oracle" not in src, f


def test_kernels_per_step_query(ngb):
    """Launch accounting without a GPU: the analytic cavity runs as two kernels
    (core + wall shell) except for FP64 and 16-bit D3Q27; flag-array grids as one."""
    d = ngb.lbm_dense_desc(64, 64, 64, 19, "f32", 1.0, box_cavity=True)
    assert ngb.lbm_dense_kernels_per_step(d) == 2
    assert ngb.lbm_dense_kernels_per_step(ngb.lbm_dense_desc(64, 64, 64, 19, "f16off", 1.0, box_cavity=True)) == 2
    assert ngb.lbm_dense_kernels_per_step(ngb.lbm_dense_desc(64, 64, 64, 27, "f16off", 1.0, box_cavity=True)) == 1
    assert ngb.lbm_dense_kernels_per_step(ngb.lbm_dense_desc(64, 64, 64, 19, "f64", 1.0, box_cavity=True)) == 1
    assert ngb.lbm_dense_kernels_per_step(ngb.lbm_dense_desc(64, 64, 64, 19, "f32", 1.0, box_cavity=False)) == 1
    assert ngb.lbm_dense_kernels_per_step(ngb.lbm_dense_desc(64, 5, 64, 19, "f32", 1.0, box_cavity=True)) == 1
