"""neon_gb300 — GB300-native (sm_103a) implementation of Neon's grid-stencil hot path.

The product is the C-ABI shared library ``_build/libneon_gb300.so`` built from
``csrc/`` (declared in ``include/neon_gb300.h``). This module only loads it with
ctypes and offers thin Python helpers over it; every compute call goes to the
CUDA library and fails loudly when the library is missing. There is no CPU
fallback.
"""
import ctypes
import os

from . import build as _build

LIB_PATH = _build.LIB_PATH

NGB_OK = 0
STORE_F64, STORE_F32, STORE_F16OFF, STORE_BF16OFF, STORE_F16SR = 0, 1, 2, 3, 4
STORAGE_NAMES = {"f64": STORE_F64, "f32": STORE_F32, "f16off": STORE_F16OFF, "bf16off": STORE_BF16OFF,
                 "f16sr": STORE_F16SR}
STORAGE_BYTES = {STORE_F64: 8, STORE_F32: 4, STORE_F16OFF: 2, STORE_BF16OFF: 2, STORE_F16SR: 2}
CELL_BOUNCEBACK, CELL_MOVINGWALL, CELL_BULK, CELL_UNDEFINED, CELL_OUTLET, CELL_PRESSURE, CELL_VELOCITY = 0, 1, 2, 3, 4, 5, 6

_lib = None


class NeonError(RuntimeError):
    """A C-ABI call returned a non-zero status."""


class LbmDenseDesc(ctypes.Structure):
    _fields_ = [("nx", ctypes.c_int32), ("ny", ctypes.c_int32), ("nz", ctypes.c_int32),
                ("q", ctypes.c_int32), ("storage", ctypes.c_int32), ("box_cavity", ctypes.c_int32),
                ("plane_stride", ctypes.c_int64), ("omega", ctypes.c_double),
                ("wall_term", (ctypes.c_double * 27) * 2), ("zouhe_rho", ctypes.c_double),
                ("zouhe_u", ctypes.c_double * 3), ("dither_seed", ctypes.c_uint32), ("pad", ctypes.c_uint32)]


def build(force=False):
    """Compile the CUDA library in-tree (see build.py)."""
    return _build.build(force=force)


def lib():
    """The loaded C-ABI library. Raises if it has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise NeonError("neon_gb300 CUDA library not built (%s); run neon_gb300.build()" % LIB_PATH)
        L = ctypes.CDLL(LIB_PATH)
        _declare(L)
        _lib = L
    return _lib


def _declare(L):
    vp, i32, i64, dbl = ctypes.c_void_p, ctypes.c_int32, ctypes.c_int64, ctypes.c_double
    dp = ctypes.POINTER(LbmDenseDesc)
    L.ngb_last_error.restype = ctypes.c_char_p
    L.ngb_version.restype = ctypes.c_int
    L.ngb_lbm_dense_step.argtypes = [dp, vp, vp, vp, vp]
    L.ngb_lbm_dense_run.argtypes = [dp, vp, vp, vp, i32, vp]
    L.ngb_lbm_dense_run_host.argtypes = [dp, vp, vp, vp, vp, vp, i32, vp]
    L.ngb_lbm_wall_mask.argtypes = [i32, i32, i32, i32, vp, vp]
    L.ngb_lbm_cavity_init.argtypes = [dp, dbl, vp, vp, vp, vp]
    L.ngb_lbm_dense_macroscopic.argtypes = [dp, vp, vp, vp, vp, vp]
    L.ngb_lbm_dense_kernels_per_step.argtypes = [dp]
    for name, args in _EXTRA_SIGNATURES.items():
        fn = getattr(L, name, None)
        if fn is not None:
            fn.argtypes = args[0]
            fn.restype = args[1]


class BGridDesc(ctypes.Structure):
    _fields_ = [("n_blocks", ctypes.c_int32), ("q", ctypes.c_int32), ("storage", ctypes.c_int32),
                ("pad", ctypes.c_int32), ("omega", ctypes.c_double), ("wall_term", (ctypes.c_double * 27) * 2),
                ("origin", ctypes.c_void_p), ("mask", ctypes.c_void_p), ("conn", ctypes.c_void_p)]


class SphereTube(ctypes.Structure):
    _fields_ = [("nx", ctypes.c_int32), ("ny", ctypes.c_int32), ("nz", ctypes.c_int32), ("ctrl_dx", ctypes.c_int32),
                ("sphere_c", ctypes.c_double * 3), ("sphere_r", ctypes.c_double), ("band", ctypes.c_double),
                ("tube_c", ctypes.c_double * 2), ("tube_r", ctypes.c_double), ("tube_band", ctypes.c_double),
                ("amplitude", ctypes.c_double), ("seed", ctypes.c_uint64)]


_vp, _i32, _dbl = ctypes.c_void_p, ctypes.c_int32, ctypes.c_double
_bd = ctypes.POINTER(BGridDesc)
# Signatures of the entry points beyond the dense LBM ones: name -> (argtypes, restype).
_EXTRA_SIGNATURES = {
    "ngb_bgrid_count": ([_i32, _i32, _i32, _vp, _vp, _vp, _vp], ctypes.c_int),
    "ngb_egrid_count": ([_i32, _i32, _i32, _vp, _vp, _vp, _vp, _vp], ctypes.c_int),
    "ngb_egrid_fill": ([_i32, _i32, _i32, _vp, _i32, _vp, _i32, _vp, _vp, _vp], ctypes.c_int),
    "ngb_bgrid_fill": ([_i32, _i32, _i32, _vp, _vp, _vp, _vp, _vp, _vp, _vp], ctypes.c_int),
    "ngb_bgrid_wall_mask": ([_bd, _vp, _vp], ctypes.c_int),
    "ngb_bgrid_lbm_step": ([_bd, _vp, _vp, _vp, _vp], ctypes.c_int),
    "ngb_bgrid_drag": ([_bd, _vp, _vp, _vp, _vp, _vp], ctypes.c_int),
    "ngb_geometry_sphere_tube": ([ctypes.POINTER(SphereTube), _vp, _vp, _vp], ctypes.c_int),
    "ngb_bgrid_flags_from_dense": ([_bd, _i32, _i32, _i32, _vp, _vp, _vp], ctypes.c_int),
    "ngb_bgrid_laplace_i64": ([_bd, _vp, _vp, _vp], ctypes.c_int),
    "ngb_dense_laplace_i64": ([_i32, _i32, _i32, _vp, _vp, _vp], ctypes.c_int),
    "ngb_lbm_release_graphs": ([], ctypes.c_int),
    "ngb_unet_weight_count": ([], ctypes.c_int64),
    "ngb_lbm_dense_save": ([ctypes.c_char_p, ctypes.POINTER(LbmDenseDesc), _vp, ctypes.c_int64, _vp], ctypes.c_int),
    "ngb_lbm_dense_load": ([ctypes.c_char_p, ctypes.POINTER(LbmDenseDesc), _vp, _vp, ctypes.POINTER(ctypes.c_int64), _vp],
                           ctypes.c_int),
    "ngb_unet_write_weights": ([ctypes.c_char_p, _vp, ctypes.c_int64], ctypes.c_int),
    "ngb_unet_read_weights": ([ctypes.c_char_p, _vp, ctypes.c_int64], ctypes.c_int),
    "ngb_learned_create": ([_i32, _i32, _vp, ctypes.c_int64, ctypes.POINTER(ctypes.c_void_p)], ctypes.c_int),
    "ngb_learned_destroy": ([_vp], ctypes.c_int),
    "ngb_learned_precondition": ([_vp, _vp, _vp, _vp], ctypes.c_int),
    "ngb_learned_solve": ([_vp, _vp, _vp, _vp, _vp, _vp], ctypes.c_int),
}


class LearnedParams(ctypes.Structure):
    _fields_ = [("tol", ctypes.c_double), ("max_iter", ctypes.c_int32), ("refresh_every", ctypes.c_int32),
                ("stall", ctypes.c_int32), ("fallback", ctypes.c_int32)]


class LearnedResult(ctypes.Structure):
    _fields_ = [("iterations", ctypes.c_int32), ("fallback", ctypes.c_int32), ("fallback_iterations", ctypes.c_int32),
                ("converged", ctypes.c_int32), ("rel_residual", ctypes.c_double), ("seconds", ctypes.c_double)]


class PoissonDesc(ctypes.Structure):
    _fields_ = [("nx", ctypes.c_int32), ("ny", ctypes.c_int32), ("nz", ctypes.c_int32), ("field", ctypes.c_int32),
                ("h", ctypes.c_double), ("bd", ctypes.c_void_p)]


class CgParams(ctypes.Structure):
    _fields_ = [("tol", ctypes.c_double), ("max_iter", ctypes.c_int32), ("refresh_every", ctypes.c_int32),
                ("check_every", ctypes.c_int32), ("jacobi", ctypes.c_int32)]


class CgResult(ctypes.Structure):
    _fields_ = [("iterations", ctypes.c_int32), ("converged", ctypes.c_int32), ("refreshes", ctypes.c_int32),
                ("pad", ctypes.c_int32), ("rel_residual", ctypes.c_double), ("seconds", ctypes.c_double)]


_pd = ctypes.POINTER(PoissonDesc)
_EXTRA_SIGNATURES.update({
    "ngb_laplacian_apply": ([_pd, _vp, _vp, _vp], ctypes.c_int),
    "ngb_dot_scratch_doubles": ([ctypes.c_int64], ctypes.c_size_t),
    "ngb_dot": ([ctypes.c_int64, _i32, _vp, _vp, _vp, _vp, _vp], ctypes.c_int),
    "ngb_cg_workspace_bytes": ([_pd], ctypes.c_size_t),
    "ngb_cg_solve": ([_pd, _vp, _vp, _vp, ctypes.c_size_t, ctypes.POINTER(CgParams), ctypes.POINTER(CgResult), _vp],
                     ctypes.c_int),
    "ngb_cg_time_passes": ([_pd, _vp, _vp, _vp, ctypes.c_size_t, _i32, _vp, _vp], ctypes.c_int),
    "ngb_poisson_rhs": ([_pd, _vp, _vp, _dbl, _vp, _vp], ctypes.c_int),
    "ngb_gaussian_sources": ([_i32, _i32, _i32, ctypes.c_uint64, _vp, _vp], ctypes.c_int),
    "ngb_dot_noalloc": ([ctypes.c_int64, _i32, _vp, _vp, _vp, _vp], ctypes.c_int),
    "ngb_conv3d": ([_i32, _i32, _i32, _vp, _i32, _i32, _vp, _vp, _vp, _i32, _i32, _i32, _i32, _i32, _vp], ctypes.c_int),
    "ngb_conv3d_bwd_weight": ([_i32, _i32, _i32, _vp, _i32, _i32, _vp, _i32, _i32, _vp, _vp], ctypes.c_int),
    "ngb_relu_bwd": ([ctypes.c_int64, _i32, _vp, _i32, _vp, _i32, _vp, _i32, _vp], ctypes.c_int),
    "ngb_pool2": ([_i32, _i32, _i32, _i32, _vp, _i32, _vp, _i32, _vp], ctypes.c_int),
    "ngb_pool2_bwd": ([_i32, _i32, _i32, _i32, _vp, _i32, _vp, _i32, _i32, _vp], ctypes.c_int),
    "ngb_up2": ([_i32, _i32, _i32, _i32, _vp, _i32, _vp, _i32, _vp], ctypes.c_int),
    "ngb_up2_bwd": ([_i32, _i32, _i32, _i32, _vp, _i32, _vp, _i32, _vp], ctypes.c_int),
    "ngb_adam": ([ctypes.c_int64, _vp, _vp, _vp, _vp, ctypes.c_float, ctypes.c_float, ctypes.c_float, ctypes.c_float,
                  _i32, _vp, _vp], ctypes.c_int),
    "ngb_flip_weights": ([_i32, _i32, _vp, _vp, _vp], ctypes.c_int),
    "ngb_mg_jacobi": ([_pd, _vp, _vp, _vp, _dbl, _vp], ctypes.c_int),
    "ngb_unet_input": ([ctypes.c_int64, _vp, _vp, _vp, _i32, _vp], ctypes.c_int),
    "ngb_unet_output": ([_i32, _i32, _i32, _vp, _i32, _vp, _dbl, _vp, _vp], ctypes.c_int),
    "ngb_scale_by_ratio": ([ctypes.c_int64, _vp, _vp, _vp, _vp], ctypes.c_int),
    "ngb_fcg_scratch_doubles": ([ctypes.c_int64], ctypes.c_size_t),
    "ngb_fcg_direction": ([ctypes.c_int64, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp], ctypes.c_int),
    "ngb_fcg_update": ([ctypes.c_int64, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp], ctypes.c_int),
    "ngb_mg_residual": ([_pd, _vp, _vp, _vp, _vp], ctypes.c_int),
    "ngb_mg_apply": ([_pd, _vp, _vp, _vp], ctypes.c_int),
    "ngb_mg_restrict": ([_pd, _vp, _vp, _dbl, _vp], ctypes.c_int),
    "ngb_mg_prolong_add": ([_pd, _vp, _vp, _vp], ctypes.c_int),
    "ngb_conv3d_tc_supported": ([_i32, _i32, _i32, _i32, _i32, _i32, _i32], ctypes.c_int),
    "ngb_conv3d_pack": ([_i32, _i32, _vp, _vp, _vp], ctypes.c_int),
    "ngb_conv3d_tc": ([_i32, _i32, _i32, _vp, _i32, _i32, _vp, _vp, _vp, _i32, _i32, _i32, _i32, _i32, _vp], ctypes.c_int),
    "ngb_conv3d_tc_check": ([_vp], ctypes.c_int),
    "ngb_conv3d_bwd_weight_tc_supported": ([ctypes.c_int32] * 7, ctypes.c_int),
    "ngb_conv3d_bwd_weight_tc": ([ctypes.c_int32] * 3 + [_vp, ctypes.c_int32, ctypes.c_int32, _vp, ctypes.c_int32, ctypes.c_int32, _vp, _vp],
                                 ctypes.c_int),
    "ngb_conv3d_bwd_weight_mma": ([ctypes.c_int32] * 3 + [_vp, ctypes.c_int32, ctypes.c_int32, _vp, ctypes.c_int32, ctypes.c_int32, _vp, _vp],
                                  ctypes.c_int),
    "ngb_conv3d_tc_wait_selftest": ([ctypes.c_int32, _vp], ctypes.c_int),
})


def check(rc):
    if rc != NGB_OK:
        raise NeonError("neon_gb300 error %d: %s" % (rc, lib().ngb_last_error().decode()))
    return rc


# ----------------------------------------------------------------------------- lattices
W19 = [1 / 18] * 3 + [1 / 36] * 6 + [1 / 3] + [1 / 18] * 3 + [1 / 36] * 6
C19 = [(-1, 0, 0), (0, -1, 0), (0, 0, -1), (-1, -1, 0), (-1, 1, 0), (-1, 0, -1), (-1, 0, 1), (0, -1, -1), (0, -1, 1),
       (0, 0, 0),
       (1, 0, 0), (0, 1, 0), (0, 0, 1), (1, 1, 0), (1, -1, 0), (1, 0, 1), (1, 0, -1), (0, 1, 1), (0, 1, -1)]


def _d27(d):
    return 0 if d == 0 else (-1 if d == 1 else 1)


C27 = [(_d27(q // 9), _d27((q // 3) % 3), _d27(q % 3)) for q in range(27)]
W27 = [{0: 8 / 27, 1: 2 / 27, 2: 1 / 54, 3: 1 / 216}[sum(c != 0 for c in v)] for v in C27]


def lattice(q):
    return (C19, W19) if q == 19 else (C27, W27)


def cavity_omega(n, ulb, re):
    """omega = 1 / (3 nu + 0.5) with nu = ulb (N - 2) / Re (Config.cpp:105-111)."""
    nu = ulb * (n - 2) / re
    return 1.0 / (3.0 * nu + 0.5)


def lid_wall_terms(q, ulb, ulid=(1.0, 0.0, 0.0)):
    """Populations held by moving-wall nodes: -6 w_k ulb (c_k . ulid) (RunCavityTwoPop.cu:177-185)."""
    c, w = lattice(q)
    return [-6.0 * w[k] * ulb * (c[k][0] * ulid[0] + c[k][1] * ulid[1] + c[k][2] * ulid[2]) for k in range(q)]


def lbm_dense_desc(nx, ny, nz, q, storage, omega, moving_wall_terms=None, box_cavity=True, plane_stride=0,
                   bounce_back_terms=None, zouhe_rho=1.0, zouhe_u=(0.0, 0.0, 0.0), dither_seed=0):
    d = LbmDenseDesc()
    d.dither_seed = dither_seed
    d.zouhe_rho = zouhe_rho
    for a in range(3):
        d.zouhe_u[a] = zouhe_u[a]
    d.nx, d.ny, d.nz, d.q = nx, ny, nz, q
    d.storage = STORAGE_NAMES[storage] if isinstance(storage, str) else storage
    d.box_cavity = 1 if box_cavity else 0
    d.plane_stride = plane_stride
    d.omega = omega
    for k in range(27):
        d.wall_term[0][k] = bounce_back_terms[k] if bounce_back_terms and k < len(bounce_back_terms) else 0.0
        d.wall_term[1][k] = moving_wall_terms[k] if moving_wall_terms and k < len(moving_wall_terms) else 0.0
    return d


def _ptr(t):
    if t is None:
        return None
    if hasattr(t, "data_ptr"):
        return ctypes.c_void_p(t.data_ptr())
    return ctypes.c_void_p(int(t))


def _stream(stream):
    if stream is None:
        return None
    if hasattr(stream, "cuda_stream"):
        return ctypes.c_void_p(stream.cuda_stream)
    return ctypes.c_void_p(int(stream))


def lbm_dense_step(desc, fin, fout, flags=None, stream=None):
    return check(lib().ngb_lbm_dense_step(ctypes.byref(desc), _ptr(fin), _ptr(fout), _ptr(flags), _stream(stream)))


def lbm_dense_run(desc, fa, fb, nsteps, flags=None, stream=None):
    return check(lib().ngb_lbm_dense_run(ctypes.byref(desc), _ptr(fa), _ptr(fb), _ptr(flags), int(nsteps),
                                         _stream(stream)))


def lbm_dense_run_host(desc, host_in, host_out, fa, fb, nsteps, flags=None, stream=None):
    return check(lib().ngb_lbm_dense_run_host(ctypes.byref(desc), _ptr(host_in), _ptr(host_out), _ptr(fa), _ptr(fb),
                                              _ptr(flags), int(nsteps), _stream(stream)))


def lbm_dense_save(path, desc, f, step, stream=None):
    """Checkpoint of the population buffer f (the newest state) with its step number."""
    check(lib().ngb_lbm_dense_save(str(path).encode(), ctypes.byref(desc), _ptr(f), int(step), _stream(stream)))


def lbm_dense_load(path, desc, fa, fb=None, stream=None):
    """Resume: fills fa (and fb) with the checkpoint's state; returns its step number."""
    step = ctypes.c_int64(0)
    check(lib().ngb_lbm_dense_load(str(path).encode(), ctypes.byref(desc), _ptr(fa), _ptr(fb) if fb is not None else None,
                                   ctypes.byref(step), _stream(stream)))
    return step.value


def lbm_wall_mask(nx, ny, nz, q, flags, stream=None):
    return check(lib().ngb_lbm_wall_mask(nx, ny, nz, q, _ptr(flags), _stream(stream)))


def lbm_cavity_init(desc, ulb, fa, fb=None, flags=None, stream=None):
    return check(lib().ngb_lbm_cavity_init(ctypes.byref(desc), float(ulb), _ptr(fa), _ptr(fb), _ptr(flags),
                                           _stream(stream)))


def lbm_dense_macroscopic(desc, fin, rho=None, u=None, flags=None, stream=None):
    return check(lib().ngb_lbm_dense_macroscopic(ctypes.byref(desc), _ptr(fin), _ptr(flags), _ptr(rho), _ptr(u),
                                                 _stream(stream)))


def cavity_profiles(u, nx, ny, nz, ulid):
    """Centre-line velocity profiles of the lid-driven cavity, as
    RunCavityTwoPop.cu:110-148 writes them: u_x / ulid along y through
    (nx/2, nz/2) and u_y / ulid along x through (ny/2, nz/2), positions
    normalised by the grid size, sorted. `u` is the velocity of
    ngb_lbm_dense_macroscopic (3 planes of nx*ny*nz doubles, host or device).
    Returns (x_profile, y_profile) as lists of (position, value)."""
    import numpy as np
    uu = np.asarray(u.cpu() if hasattr(u, "cpu") else u, dtype=np.float64).reshape(3, nz, ny, nx)
    scale = 1.0 / ulid
    xc, yc, zc = nx // 2, ny // 2, nz // 2
    yprof = [(y / ny, float(uu[0, zc, y, xc]) * scale) for y in range(ny)]
    xprof = [(x / nx, float(uu[1, zc, yc, x]) * scale) for x in range(nx)]
    return xprof, yprof


def write_cavity_profiles(directory, iteration, xprof, yprof):
    """NeonUniformLBM_<iteration, 5 digits>_{X,Y}.dat with lines "position value"
    in the reference's default stream format (6 significant digits)."""
    import os
    tag = "%05d" % iteration if iteration < 100000 else str(iteration)
    paths = []
    for prof, axis in ((yprof, "Y"), (xprof, "X")):
        path = os.path.join(directory, "NeonUniformLBM_%s_%s.dat" % (tag, axis))
        with open(path, "w") as f:
            for pos, val in prof:
                f.write("%g %g\n" % (pos, val))
        paths.append(path)
    return paths


# ----------------------------------------------------------------------------- bGrid
class BGrid:
    """A block-sparse grid (8^3 blocks) built on the device from a dense byte
    activity map (torch uint8 tensor on cuda, nx*ny*nz, x fastest).
    Mirrors Neon::bGrid's construction (bGrid_imp.h:19-246) for one partition."""

    def __init__(self, nx, ny, nz, active, stream=None):
        import torch
        self.nx, self.ny, self.nz = nx, ny, nz
        self.bnx, self.bny, self.bnz = (nx + 7) // 8, (ny + 7) // 8, (nz + 7) // 8
        dev = active.device
        self.block_of = torch.empty(self.bnx * self.bny * self.bnz, dtype=torch.int32, device=dev)
        nb = torch.zeros(1, dtype=torch.int32, device=dev)
        check(lib().ngb_bgrid_count(nx, ny, nz, _ptr(active), _ptr(self.block_of), _ptr(nb), _stream(stream)))
        self.n_blocks = int(nb.item())
        n = max(self.n_blocks, 1)
        self.origin = torch.empty(3 * n, dtype=torch.int32, device=dev)
        self.mask = torch.empty(16 * n, dtype=torch.int32, device=dev)
        self.conn = torch.empty(27 * n, dtype=torch.int32, device=dev)
        cnt = torch.zeros(1, dtype=torch.int64, device=dev)
        check(lib().ngb_bgrid_fill(nx, ny, nz, _ptr(active), _ptr(self.block_of), _ptr(self.origin), _ptr(self.mask),
                                   _ptr(self.conn), _ptr(cnt), _stream(stream)))
        self.n_active_voxels = int(cnt.item())

    def desc(self, q=19, storage="f32", omega=1.0, moving_wall_terms=None, bounce_back_terms=None):
        d = BGridDesc()
        d.n_blocks, d.q = self.n_blocks, q
        d.storage = STORAGE_NAMES[storage] if isinstance(storage, str) else storage
        d.omega = omega
        for k in range(27):
            d.wall_term[0][k] = bounce_back_terms[k] if bounce_back_terms and k < len(bounce_back_terms) else 0.0
            d.wall_term[1][k] = moving_wall_terms[k] if moving_wall_terms and k < len(moving_wall_terms) else 0.0
        d.origin, d.mask, d.conn = self.origin.data_ptr(), self.mask.data_ptr(), self.conn.data_ptr()
        return d


def bgrid_wall_mask(desc, flags, stream=None):
    return check(lib().ngb_bgrid_wall_mask(ctypes.byref(desc), _ptr(flags), _stream(stream)))


def bgrid_lbm_step(desc, fin, fout, flags, stream=None):
    return check(lib().ngb_bgrid_lbm_step(ctypes.byref(desc), _ptr(fin), _ptr(fout), _ptr(flags), _stream(stream)))


def bgrid_drag(desc, fin, flags, partials, force, stream=None):
    return check(lib().ngb_bgrid_drag(ctypes.byref(desc), _ptr(fin), _ptr(flags), _ptr(partials), _ptr(force),
                                      _stream(stream)))


# ----------------------------------------------------------------------------- eGrid
class EGrid:
    """An element-sparse grid of one partition built on the device from a dense
    byte activity map (torch uint8 tensor on cuda, nx*ny*nz, x fastest) and a
    list of stencil offsets (Neon::eGrid's construction, eGrid_imp.h:8-129):
    `count` elements in z, y, x order, `origin` (3 x int32 per element) and
    `conn` (int32, conn[s*count + e] = neighbour element along points[s] or -1)."""

    def __init__(self, nx, ny, nz, active, points, stream=None):
        import numpy as np
        import torch
        self.nx, self.ny, self.nz = nx, ny, nz
        self.points = [tuple(int(v) for v in p) for p in points]
        dev = active.device
        V = nx * ny * nz
        self.elem_of = torch.empty(V, dtype=torch.int32, device=dev)
        scratch = torch.empty((V + 2047) // 2048 + 1, dtype=torch.int32, device=dev)
        cnt = torch.zeros(1, dtype=torch.int32, device=dev)
        check(lib().ngb_egrid_count(nx, ny, nz, _ptr(active), _ptr(self.elem_of), _ptr(scratch), _ptr(cnt), _stream(stream)))
        self.count = int(cnt.item())
        n = max(self.count, 1)
        self.origin = torch.empty(3 * n, dtype=torch.int32, device=dev)
        self.conn = torch.empty(max(len(self.points), 1) * n, dtype=torch.int32, device=dev)
        pts = np.array(self.points, dtype=np.int8).reshape(-1)
        check(lib().ngb_egrid_fill(nx, ny, nz, _ptr(self.elem_of), self.count,
                                   pts.ctypes.data_as(ctypes.c_void_p) if len(self.points) else None, len(self.points),
                                   _ptr(self.origin), _ptr(self.conn), _stream(stream)))


def bgrid_flags_from_dense(desc, nx, ny, nz, cls, flags, stream=None):
    return check(lib().ngb_bgrid_flags_from_dense(ctypes.byref(desc), nx, ny, nz, _ptr(cls), _ptr(flags),
                                                  _stream(stream)))


def bgrid_laplace_i64(desc, a, b, stream=None):
    return check(lib().ngb_bgrid_laplace_i64(ctypes.byref(desc), _ptr(a), _ptr(b), _stream(stream)))


def dense_laplace_i64(nx, ny, nz, a, b, stream=None):
    return check(lib().ngb_dense_laplace_i64(nx, ny, nz, _ptr(a), _ptr(b), _stream(stream)))


def sphere_tube(nx, ny, nz, sphere_c, sphere_r, band, tube_c, tube_r, tube_band, amplitude, ctrl_dx, seed):
    g = SphereTube()
    g.nx, g.ny, g.nz, g.ctrl_dx = nx, ny, nz, ctrl_dx
    for a in range(3):
        g.sphere_c[a] = sphere_c[a]
    g.sphere_r, g.band = sphere_r, band
    g.tube_c[0], g.tube_c[1] = tube_c
    g.tube_r, g.tube_band, g.amplitude, g.seed = tube_r, tube_band, amplitude, seed
    return g


def geometry_sphere_tube(g, active, cls, stream=None):
    return check(lib().ngb_geometry_sphere_tube(ctypes.byref(g), _ptr(active), _ptr(cls), _stream(stream)))


def sphere_config(scale=1):
    """The flow-over-sphere case, 512x256x256 box at scale 1 (sizes divided by
    `scale`): sphere r = 32 at (128,128,128); active within 48 voxels of the
    sphere surface or of a radius-40 tube along x whose axis wanders +-24
    voxels through control points every 64 voxels (seed 2024)."""
    s = scale
    return sphere_tube(512 // s, 256 // s, 256 // s, (128 / s, 128 / s, 128 / s), 32 / s, 48 / s, (128 / s, 128 / s),
                       40 / s, 48 / s, 24 / s, max(1, 64 // s), 2024)


# ----------------------------------------------------------------------------- Poisson
def poisson_desc(nx, ny, nz, field="f32", h=1.0, bd=None):
    d = PoissonDesc()
    d.nx, d.ny, d.nz = nx, ny, nz
    d.field = STORAGE_NAMES[field] if isinstance(field, str) else field
    d.h = h
    d.bd = bd.data_ptr() if bd is not None else None
    return d


def laplacian_apply(desc, u, out, stream=None):
    return check(lib().ngb_laplacian_apply(ctypes.byref(desc), _ptr(u), _ptr(out), _stream(stream)))


def lbm_dense_kernels_per_step(desc):
    """Kernel launches one ngb_lbm_dense_step of `desc` issues."""
    n = lib().ngb_lbm_dense_kernels_per_step(ctypes.byref(desc))
    if n < 0:
        check(n)
    return n


def mg_jacobi(desc, u, r, out, omega, stream=None):
    """out = u + omega h^2/6 (r - A u) on Free nodes; u None: two sweeps from zero."""
    return check(lib().ngb_mg_jacobi(ctypes.byref(desc), _ptr(u) if u is not None else None, _ptr(r), _ptr(out), omega,
                                     _stream(stream)))


def mg_apply(desc, u, out, stream=None):
    """out = A u on Free nodes, 0 on the box faces (FP32, box-face Dirichlet problem)."""
    return check(lib().ngb_mg_apply(ctypes.byref(desc), _ptr(u), _ptr(out), _stream(stream)))


def mg_residual(desc, u, r, out, stream=None):
    return check(lib().ngb_mg_residual(ctypes.byref(desc), _ptr(u) if u is not None else None, _ptr(r), _ptr(out),
                                       _stream(stream)))


def mg_restrict(fine_desc, res, rc, scale=1.0, stream=None):
    return check(lib().ngb_mg_restrict(ctypes.byref(fine_desc), _ptr(res), _ptr(rc), scale, _stream(stream)))


def mg_prolong_add(fine_desc, ec, u, stream=None):
    return check(lib().ngb_mg_prolong_add(ctypes.byref(fine_desc), _ptr(ec), _ptr(u), _stream(stream)))


def dot(a, b, result, scratch=None, stream=None):
    """result (1-element float64 cuda tensor) = <a, b> accumulated in FP64."""
    import torch
    n = a.numel()
    if scratch is None:
        scratch = torch.empty(lib().ngb_dot_scratch_doubles(n), dtype=torch.float64, device=a.device)
    field = STORE_F64 if a.dtype == torch.float64 else STORE_F32
    return check(lib().ngb_dot(n, field, _ptr(a), _ptr(b), _ptr(result), _ptr(scratch), _stream(stream)))


def cg_workspace(desc, device):
    import torch
    nbytes = lib().ngb_cg_workspace_bytes(ctypes.byref(desc))
    return torch.empty(nbytes, dtype=torch.uint8, device=device)


def cg_solve(desc, b, x, workspace, tol=1e-8, max_iter=10000, refresh_every=50, check_every=50, jacobi=True,
             stream=None):
    """Jacobi-PCG / CG on the device; x (float64 cuda tensor) is the initial guess and the solution."""
    p = CgParams()
    p.tol, p.max_iter, p.refresh_every, p.check_every, p.jacobi = tol, max_iter, refresh_every, check_every, int(jacobi)
    r = CgResult()
    check(lib().ngb_cg_solve(ctypes.byref(desc), _ptr(b), _ptr(x), _ptr(workspace), workspace.numel(),
                             ctypes.byref(p), ctypes.byref(r), _stream(stream)))
    return {"iterations": r.iterations, "converged": bool(r.converged), "refreshes": r.refreshes,
            "rel_residual": r.rel_residual, "seconds": r.seconds}


def cg_time_passes(desc, b, x, workspace, reps=20, stream=None):
    """CUDA-event milliseconds per launch of the CG passes A and B (measurement aid)."""
    ms = (ctypes.c_float * 2)()
    check(lib().ngb_cg_time_passes(ctypes.byref(desc), _ptr(b), _ptr(x), _ptr(workspace), workspace.numel(), int(reps),
                                   ctypes.cast(ms, ctypes.c_void_p), _stream(stream)))
    return float(ms[0]), float(ms[1])


def gaussian_sources(nx, ny, nz, seed):
    import numpy as np
    c = np.zeros(24)
    a = np.zeros(8)
    check(lib().ngb_gaussian_sources(nx, ny, nz, seed, c.ctypes.data_as(ctypes.c_void_p),
                                     a.ctypes.data_as(ctypes.c_void_p)))
    return c, a


def poisson_rhs(desc, centres, amps, sigma, f, stream=None):
    """centres/amps: float64 cuda tensors (24 and 8 values)."""
    return check(lib().ngb_poisson_rhs(ctypes.byref(desc), _ptr(centres), _ptr(amps), float(sigma), _ptr(f),
                                       _stream(stream)))


class LearnedSolver:
    """The learned-preconditioner Poisson solver of the C ABI (ngb_learned_*):
    FCG(1) with a V-cycle whose coarsest solve is the U-Net, FP64 true
    residual, Jacobi-PCG fallback. `weights`: a weight-file path or an FP32
    host tensor of ngb_unet_weight_count() values; None gives the same cycle
    without the network (no coarsest-level correction)."""

    def __init__(self, n, levels, weights):
        import torch
        L = lib()
        if isinstance(weights, (str, bytes, os.PathLike)):
            from .learned import read_weights
            weights = read_weights(weights)
        h = ctypes.c_void_p()
        if weights is None:
            self._keep = None
            check(L.ngb_learned_create(int(n), int(levels), None, 0, ctypes.byref(h)))
        else:
            w = weights.detach().to("cpu", torch.float32).contiguous()
            self._keep = w
            check(L.ngb_learned_create(int(n), int(levels), ctypes.c_void_p(w.data_ptr()), w.numel(), ctypes.byref(h)))
        self.handle, self.n, self.levels = h, n, levels

    def precondition(self, r, z, stream=None):
        check(lib().ngb_learned_precondition(self.handle, _ptr(r), _ptr(z), _stream(stream)))
        return z

    def solve(self, b, x, tol=1e-8, max_iter=2000, refresh_every=10, stall=30, fallback=True, stream=None):
        p = LearnedParams()
        p.tol, p.max_iter, p.refresh_every, p.stall, p.fallback = tol, max_iter, refresh_every, stall, int(fallback)
        r = LearnedResult()
        check(lib().ngb_learned_solve(self.handle, _ptr(b), _ptr(x), ctypes.byref(p), ctypes.byref(r), _stream(stream)))
        return {"iterations": r.iterations, "fallback": bool(r.fallback), "fallback_iterations": r.fallback_iterations,
                "converged": bool(r.converged), "rel_residual": r.rel_residual, "seconds": r.seconds}

    def close(self):
        if getattr(self, "handle", None):
            lib().ngb_learned_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
