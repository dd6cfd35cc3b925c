"""Shared helpers of the test-suite (numpy <-> ctypes plumbing, cavity set-ups)."""
import ctypes

import numpy as np

import neon_gb300 as ngb


def P(a):
    """ctypes pointer of a numpy array."""
    return a.ctypes.data_as(ctypes.c_void_p)


STORE_DTYPE = {0: np.float64, 1: np.float32, 2: np.uint16, 3: np.uint16, 4: np.uint16}


def wall_table(q, ulb, storage):
    """4 x 27 wall-term table for the oracle: index 1 = moving lid, rounded like the stored value."""
    t = np.zeros((4, 27))
    terms = ngb.lid_wall_terms(q, ulb)
    for k in range(q):
        v = terms[k]
        if storage != 0:
            v = float(np.float32(v))
        t[1, k] = v
    return t


def oracle_cavity(orc, n, q, storage, steps, ulb=0.1, re=100.0, mode=None, compute_float=None, threads=0):
    """Run the oracle cavity; returns (populations after `steps`, packed flags, omega)."""
    V = n ** 3
    flags = np.zeros(V, np.uint32)
    orc.orc_cavity_flags(n, n, n, q, P(flags))
    a = np.zeros(q * V, STORE_DTYPE[storage])
    orc.orc_cavity_init(n, n, n, q, storage, ulb, P(a))
    b = a.copy()
    omega = ngb.cavity_omega(n, ulb, re)
    if mode is None:
        mode = 0 if (q == 19 and storage in (0, 1)) else (2 if storage in (2, 3, 4) else 1)
    if compute_float is None:
        compute_float = 0 if storage == 0 else 1
    wt = wall_table(q, ulb, storage)
    rc = orc.orc_lbm_run(n, n, n, q, storage, mode, compute_float, omega, P(wt), P(flags), P(a), P(b), steps, threads)
    assert rc == 0
    return (a if steps % 2 == 0 else b), flags, omega


def oracle_velocity(orc, n, q, storage, flags, pop, ulb=0.1, rho=None):
    """Velocity field as computeRhoAndU (LbmTools.h:383-437): pulled populations on bulk cells."""
    u = np.zeros(3 * n ** 3)
    wt = wall_table(q, ulb, storage)
    orc.orc_velocity(n, n, n, q, storage, P(wt), P(flags), P(pop), P(rho) if rho is not None else None, P(u))
    return u


def rel_max(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))
