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
    (core + wall shell) except for FP64 and for 16-bit storage on an odd x
    extent (the core kernel takes x-pairs there); flag-array grids as one."""
    d = ngb.lbm_dense_desc(64, 64, 64, 19, "f32", 1.0, box_cavity=True)
    assert ngb.lbm_dense_kernels_per_step(d) == 2
    assert ngb.lbm_dense_kernels_per_step(ngb.lbm_dense_desc(64, 64, 64, 19, "f16off", 1.0, box_cavity=True)) == 2
    assert ngb.lbm_dense_kernels_per_step(ngb.lbm_dense_desc(64, 64, 64, 27, "f16off", 1.0, box_cavity=True)) == 2
    assert ngb.lbm_dense_kernels_per_step(ngb.lbm_dense_desc(63, 64, 64, 27, "f16off", 1.0, box_cavity=True)) == 1
    assert ngb.lbm_dense_kernels_per_step(ngb.lbm_dense_desc(64, 64, 64, 19, "f64", 1.0, box_cavity=True)) == 1
    assert ngb.lbm_dense_kernels_per_step(ngb.lbm_dense_desc(64, 64, 64, 19, "f32", 1.0, box_cavity=False)) == 1
    assert ngb.lbm_dense_kernels_per_step(ngb.lbm_dense_desc(64, 5, 64, 19, "f32", 1.0, box_cavity=True)) == 1


def test_new_entry_points_validate_without_gpu(ngb):
    """Argument errors of the multilevel, FCG and network-scaling entry points
    are reported before any CUDA call."""
    import ctypes
    L = ngb.lib()
    odd = ngb.poisson_desc(13, 12, 12, "f32", 1.0)
    assert L.ngb_mg_restrict(ctypes.byref(odd), ctypes.c_void_p(16), ctypes.c_void_p(32), 1.0, None) == -1
    assert b"even" in L.ngb_last_error()
    f64 = ngb.poisson_desc(12, 12, 12, "f64", 1.0)
    assert L.ngb_mg_apply(ctypes.byref(f64), ctypes.c_void_p(16), ctypes.c_void_p(32), None) == -1
    assert b"FP32" in L.ngb_last_error()
    box = ngb.poisson_desc(12, 12, 12, "f32", 1.0)
    assert L.ngb_mg_jacobi(ctypes.byref(box), None, ctypes.c_void_p(16), ctypes.c_void_p(32), 2.5, None) == -1
    assert b"omega" in L.ngb_last_error()
    assert L.ngb_fcg_direction(0, None, None, None, None, None, None, None, None, None, None) == -1
    assert L.ngb_fcg_direction(10, ctypes.c_void_p(16), ctypes.c_void_p(32), None, None, ctypes.c_void_p(48),
                               ctypes.c_void_p(64), None, ctypes.c_void_p(80), ctypes.c_void_p(96), None) == -1
    assert b"zq given" in L.ngb_last_error()
    assert L.ngb_fcg_update(10, None, None, None, None, None, None, None, None) == -1
    assert L.ngb_unet_input(0, None, None, None, 16, None) == -1
    assert L.ngb_unet_output(8, 8, 8, None, 16, None, 1.0, None, None) == -1
    assert L.ngb_scale_by_ratio(0, None, None, None, None) == -1
    assert L.ngb_fcg_scratch_doubles(1000) >= 3


def test_ctypes_structs_match_the_c_layout(ngb):
    """Every ABI struct the Python helpers lay out has the size the library was compiled with."""
    import ctypes
    L = ngb.lib()
    L.ngb_abi_struct_size.restype = ctypes.c_size_t
    L.ngb_abi_struct_size.argtypes = [ctypes.c_int32]
    structs = [ngb.LbmDenseDesc, ngb.BGridDesc, ngb.PoissonDesc, ngb.CgParams, ngb.CgResult, ngb.LearnedParams,
               ngb.LearnedResult]
    for i, st in enumerate(structs):
        assert L.ngb_abi_struct_size(i) == ctypes.sizeof(st), (st.__name__, L.ngb_abi_struct_size(i), ctypes.sizeof(st))
    assert L.ngb_abi_struct_size(99) == 0
