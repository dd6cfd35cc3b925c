"""CPU baselines of the hot path on the host cores (measurement infrastructure).

Times the oracle (the CPU restatement of the reference's per-cell arithmetic)
on the cases the GPU path is measured on, one thread and all threads:

* D3Q19 FP32 lid-driven cavity (the reference's unrolled BGK arithmetic),
  64^3 and 128^3, MLUPS = cells * steps / time (walls included, as Neon
  counts them);
* the flow-over-sphere geometry at 256x128x128 (half size), D3Q19 FP32
  shifted form through the oracle's bit-exact restatement (generic storage
  functors, slower than the cavity's dedicated loop), MLUPS over the active
  cells;
* Poisson Jacobi-PCG (FP32 fields, FP64 dot products, true residual every
  50 iterations) to 1e-8 at 64^3 and 128^3 (the oracle's CG is serial).

The reference's own CPU backend runs its grid loops serially, so the 1-thread
numbers are the reference-like ones. Prints one JSON object.

    python oracle/cpu_baselines.py [--quick]
"""
import ctypes
import json
import os
import platform
import sys
import time

import numpy as np

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
import oracle  # noqa: E402

P = lambda a: a.ctypes.data_as(ctypes.c_void_p)  # noqa: E731


def _omega(n, ulb=0.1, re=100.0):
    return 1.0 / (3.0 * ulb * (n - 2) / re + 0.5)


def lbm_cavity(L, n, threads, seconds):
    """MLUPS of the D3Q19 FP32 cavity at n^3 (reference arithmetic)."""
    V = n ** 3
    flags = np.zeros(V, np.uint32)
    L.orc_cavity_flags(n, n, n, 19, P(flags))
    a = np.zeros(19 * V, np.float32)
    L.orc_cavity_init(n, n, n, 19, 1, 0.1, P(a))
    b = a.copy()
    us = L.orc_time_d3q19_f32(n, n, n, 2, threads, _omega(n), P(flags), P(a), P(b))
    steps = max(2, int(seconds * 1e6 / max(us / 2, 1.0)) // 2 * 2)
    us = L.orc_time_d3q19_f32(n, n, n, steps, threads, _omega(n), P(flags), P(a), P(b))
    return {"n": n, "threads": threads, "steps": steps, "seconds": round(us / 1e6, 3), "mlups": round(V * steps / us, 2)}


def lbm_sphere(L, scale, threads, seconds):
    """Active-cell MLUPS of the flow-over-sphere geometry (shifted FP32 form)."""
    s = scale
    nx, ny, nz = 512 // s, 256 // s, 256 // s
    V = nx * ny * nz
    sc = np.array([128 / s] * 3)
    tc = np.array([128 / s] * 2)
    active = np.zeros(V, np.uint8)
    cls = np.zeros(V, np.uint8)
    L.orc_sphere_tube(nx, ny, nz, max(1, 64 // s), P(sc), ctypes.c_double(32 / s), ctypes.c_double(48 / s), P(tc),
                      ctypes.c_double(40 / s), ctypes.c_double(48 / s), ctypes.c_double(24 / s), ctypes.c_uint64(2024),
                      P(active), P(cls))
    flags = np.zeros(V, np.uint32)
    L.orc_flags_from_classes(nx, ny, nz, 19, P(cls), P(flags))
    nact = int(active.sum())
    w = np.array([1 / 18] * 3 + [1 / 36] * 6 + [1 / 3] + [1 / 18] * 3 + [1 / 36] * 6, np.float32)
    a = np.zeros((19, V), np.float32)
    a[:, cls == 2] = w[:, None]
    a = a.ravel()
    b = a.copy()
    wall = np.zeros((4, 27))
    omega = 1.0 / (3.0 * 0.05 * 2 * (32 / s) / 100.0 + 0.5)
    run = lambda k: L.orc_lbm_run(nx, ny, nz, 19, 1, 2, 1, ctypes.c_double(omega), P(wall), P(flags), P(a), P(b), k, threads)
    t0 = time.perf_counter()
    run(2)
    dt = (time.perf_counter() - t0) / 2
    steps = max(2, int(seconds / max(dt, 1e-6)) // 2 * 2)
    t0 = time.perf_counter()
    run(steps)
    dt = time.perf_counter() - t0
    return {"dims": [nx, ny, nz], "active_cells": nact, "threads": threads, "steps": steps, "seconds": round(dt, 3),
            "mlups_active": round(nact * steps / dt / 1e6, 2)}


def poisson_pcg(L, n):
    """Seconds and iterations of the oracle's Jacobi-PCG (FP32 fields, FP64 dots) to 1e-8."""
    V = n ** 3
    bd = np.zeros(V, np.int8)
    L.orc_box_boundary(n, n, n, P(bd))
    centres = np.zeros(24)
    amps = np.zeros(8)
    L.orc_gaussian_sources(n, n, n, ctypes.c_uint64(2024), P(centres), P(amps))
    c = centres.reshape(8, 3)
    g = np.arange(n, dtype=np.float64)
    z, y, x = np.meshgrid(g, g, g, indexing="ij")
    f = np.zeros((n, n, n))
    for k in range(8):
        f += amps[k] * np.exp(-((x - c[k, 0]) ** 2 + (y - c[k, 1]) ** 2 + (z - c[k, 2]) ** 2) / (2 * 8.0 ** 2))
    f = f.ravel()
    f[bd.astype(bool) == False] = 0.0  # noqa: E712 (Fixed rows carry 0)
    b = f.astype(np.float32)
    xs = np.zeros(V)
    res = np.zeros(4)
    t0 = time.perf_counter()
    L.orc_pcg_f32(n, n, n, ctypes.c_double(1.0), P(bd), P(b), P(xs), ctypes.c_double(1e-8), 20000, 50, P(res), 1)
    dt = time.perf_counter() - t0
    return {"n": n, "threads": 1, "iterations": int(res[0]), "converged": bool(res[1]), "rel_residual": float(res[2]),
            "seconds": round(dt, 3)}


def main(quick=False):
    L = oracle.lib()
    cores = int(L.orc_max_threads())
    secs = 0.5 if quick else 5.0
    out = {"host": platform.machine(), "cores": cores, "cpu_model": platform.processor() or platform.machine(),
           "implementation": "oracle restatement of the reference arithmetic (g++ -O2, OpenMP)"}
    sizes = (16,) if quick else (64, 128)
    out["lbm_d3q19_f32_cavity"] = [lbm_cavity(L, n, t, secs) for n in sizes for t in sorted({1, cores})]
    scale = 8 if quick else 2
    out["lbm_d3q19_f32_sphere"] = [lbm_sphere(L, scale, t, secs) for t in sorted({1, cores})]
    out["poisson_jacobi_pcg_f32"] = [poisson_pcg(L, n) for n in ((32,) if quick else (64, 128))]
    print(json.dumps(out), flush=True)
    return out


if __name__ == "__main__":
    main(quick="--quick" in sys.argv)
