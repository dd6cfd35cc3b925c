"""ORACLE — test infrastructure only.

CPU restatement of the Neon grid-stencil path (LBM cavity, bGrid construction,
7-point Laplacian, CG). It is the checker used by ``tests/``, by
``__graft_entry__.smoke()`` and by the CPU-baseline leg of ``bench.py``; the
product package ``neon_gb300`` never imports it.

``build()`` compiles ``oracle.cpp`` into ``oracle/_build/liboracle.so`` with
g++ (-O2, FP contraction off, OpenMP) and ``lib()`` loads it with ctypes.
"""
import ctypes
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")
LIB_PATH = os.path.join(BUILD_DIR, "liboracle.so")
SOURCES = ["oracle.cpp"]
HEADERS = ["lbm_oracle.hpp", "bgrid_oracle.hpp", "poisson_oracle.hpp"]

_lib = None


def _stale():
    if not os.path.exists(LIB_PATH):
        return True
    t = os.path.getmtime(LIB_PATH)
    return any(os.path.getmtime(os.path.join(HERE, f)) > t for f in SOURCES + HEADERS)


def build(force=False):
    """Compile the oracle shared library (seconds)."""
    if not force and not _stale():
        return LIB_PATH
    os.makedirs(BUILD_DIR, exist_ok=True)
    tmp = LIB_PATH + ".tmp%d" % os.getpid()
    cmd = ["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fno-fast-math", "-fopenmp",
           "-shared", "-fPIC", "-o", tmp] + [os.path.join(HERE, s) for s in SOURCES]
    subprocess.check_call(cmd)
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


def lib():
    """The loaded oracle library (built on first use)."""
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB_PATH)
        c_int, c_double, c_void_p = ctypes.c_int, ctypes.c_double, ctypes.c_void_p
        c_size_t, c_int64, c_uint64 = ctypes.c_size_t, ctypes.c_int64, ctypes.c_uint64
        L.orc_lbm_run.argtypes = [c_int, c_int, c_int, c_int, c_int, c_int, c_int, c_double,
                                  c_void_p, c_void_p, c_void_p, c_void_p, c_int, c_int]
        L.orc_cavity_init.argtypes = [c_int, c_int, c_int, c_int, c_int, c_double, c_void_p]
        L.orc_cavity_flags.argtypes = [c_int, c_int, c_int, c_int, c_void_p]
        L.orc_wall_mask.argtypes = [c_int, c_int, c_int, c_int, c_void_p]
        L.orc_velocity.argtypes = [c_int, c_int, c_int, c_int, c_int, c_void_p, c_void_p, c_void_p, c_void_p,
                                   c_void_p]
        L.orc_time_d3q19_f32.argtypes = [c_int, c_int, c_int, c_int, c_int, c_double, c_void_p, c_void_p, c_void_p]
        L.orc_time_d3q19_f32.restype = c_double
        L.orc_set_zouhe.argtypes = [c_double, c_double, c_double, c_double]
        L.orc_set_dither_seed.argtypes = [ctypes.c_uint32]
        L.orc_f32_to_f16_sr.argtypes = [c_void_p, c_void_p, c_void_p, c_size_t]
        L.orc_dither_bits.argtypes = [c_void_p, c_void_p, ctypes.c_uint32, c_void_p, c_size_t]
        for f in ("orc_f32_to_f16", "orc_f16_to_f32", "orc_f32_to_bf16", "orc_bf16_to_f32"):
            getattr(L, f).argtypes = [c_void_p, c_void_p, c_size_t]
        L.orc_bgrid_build.argtypes = [c_int, c_int, c_int, c_void_p, c_void_p, c_void_p, c_void_p, c_int64, c_void_p]
        L.orc_bgrid_build.restype = c_int64
        L.orc_laplace_i64.argtypes = [c_int, c_int, c_int, c_void_p, c_void_p, c_void_p]
        L.orc_masked_values_i64.argtypes = [c_int, c_int, c_int, c_int64, c_int, c_void_p]
        L.orc_sphere_tube.argtypes = [c_int, c_int, c_int, c_int, c_void_p, c_double, c_double, c_void_p, c_double,
                                      c_double, c_double, c_uint64, c_void_p, c_void_p]
        L.orc_flags_from_classes.argtypes = [c_int, c_int, c_int, c_int, c_void_p, c_void_p]
        L.orc_box_boundary.argtypes = [c_int, c_int, c_int, c_void_p]
        L.orc_egrid_build.argtypes = [c_int, c_int, c_int, c_void_p, c_void_p, c_int, c_void_p, c_void_p]
        L.orc_egrid_build.restype = c_int64
        L.orc_gaussian_sources.argtypes = [c_int, c_int, c_int, c_uint64, c_void_p, c_void_p]
        L.orc_laplacian_f64.argtypes = [c_int, c_int, c_int, c_double, c_void_p, c_void_p, c_void_p]
        L.orc_laplacian_f32.argtypes = [c_int, c_int, c_int, c_double, c_void_p, c_void_p, c_void_p]
        for f in ("orc_pcg_f32", "orc_pcg_f64"):
            getattr(L, f).argtypes = [c_int, c_int, c_int, c_double, c_void_p, c_void_p, c_void_p, c_double,
                                      c_int, c_int, c_void_p, c_int]
        L.orc_reference_cg_f64.argtypes = [c_int, c_int, c_int, c_double, c_void_p, c_void_p, c_void_p, c_int]
        L.orc_reference_cg_f64.restype = c_double
        L.orc_reference_cg_f32.argtypes = [c_int, c_int, c_int, c_double, c_void_p, c_void_p, c_void_p, c_int]
        L.orc_reference_cg_f32.restype = c_double
        _lib = L
    return _lib
