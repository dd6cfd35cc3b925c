#!/usr/bin/env python3
"""Benchmark of the Neon grid-stencil hot path on GB300.

Default workload: D3Q19 BGK lid-driven cavity, dense grid 384^3, FP32
populations in SoA planes (the FP32 D3Q19 384^3 case of the cavity
benchmark, benchmarks/lbm-lid-driven-cavity-flow), lid u = 0.1 along +x,
Re = 100. A "step" is one pull stream-collide time step over the whole
lattice; MLUPS = N^3 * steps / time (walls counted, as Metrics.h:39-42).

Prints ONE JSON line. `value` is device-timed with inputs resident in HBM;
`e2e` is the same metric through the host-buffer C-ABI call
(ngb_lbm_dense_run_host: H2D of the populations, the steps, D2H of the
result, all inside the timed region).

`--impl reference` times the CPU restatement of the reference's per-cell
D3Q19 FP32 arithmetic (the oracle port; the reference cannot be built
here) on all host threads, on bounded z-slab samples of the same lattice.
"""
import argparse
import ctypes
import json
import math
import os
import re
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "D3Q19 LBM MLUPS"
UNIT = "MLUPS"
BYTES_PER_UPDATE = {("d3q19", "f32"): 152, ("d3q19", "f64"): 304, ("d3q19", "f16off"): 76, ("d3q19", "bf16off"): 76,
                    ("d3q27", "f32"): 216, ("d3q27", "f64"): 432, ("d3q27", "f16off"): 108, ("d3q27", "bf16off"): 108}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=None,
                    help="timed steps (default 200; poisson: repeated solves, default 3)")
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n", type=int, default=0, help="grid size (default: 384 for the LBM workloads, 512 for poisson/learned, 256 for unet)")
    ap.add_argument("--lattice", default="d3q19", choices=["d3q19", "d3q27"])
    ap.add_argument("--storage", default="f32", choices=["f64", "f32", "f16off", "bf16off"])
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--extra", action="store_true", help="also time the other storage/lattice forms")
    ap.add_argument("--profiles", default="", help="cavity: write the centre-line velocity profiles into this directory")
    ap.add_argument("--workload", default="cavity", choices=["cavity", "sphere", "poisson", "learned", "unet", "accuracy"],
                    help="cavity: dense LBM (default, the headline); sphere: bGrid flow over a sphere; "
                         "poisson: Jacobi-PCG to 1e-8; learned: U-Net-preconditioned FCG vs Jacobi-PCG to 1e-8; "
                         "unet: forward applications of the preconditioner network at --n; "
                         "accuracy: cavity velocity error of every storage form against FP64 after --sim-steps")
    ap.add_argument("--train-n", type=int, default=64,
                    help="learned: training grid size = the coarsest level of the V-cycle")
    ap.add_argument("--lr", type=float, default=3e-4, help="learned: Adam learning rate")
    ap.add_argument("--train-pairs", type=int, default=2000, help="learned: solver-generated training pairs")
    ap.add_argument("--epochs", type=int, default=2, help="learned: training epochs")
    ap.add_argument("--weights", default="", help="learned: load U-Net weights from this file instead of training")
    ap.add_argument("--save-weights", default="", help="learned: save the trained weights here")
    ap.add_argument("--scale", type=int, default=1, help="sphere case size divisor")
    ap.add_argument("--sim-steps", type=int, default=0, help="sphere: steps of the drag comparison run")
    args = ap.parse_args()
    if args.n <= 0:
        args.n = {"poisson": 512, "learned": 512, "unet": 256}.get(args.workload, 384)
    if args.steps is None:
        args.steps = 3 if args.workload == "poisson" else 200
    return args


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def max_over_ranks(ms, world, device):
    """Slowest rank's time: the whole job ends when the last replica ends."""
    if world <= 1:
        return ms
    import torch
    t = torch.tensor([ms], dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def whole_job_mlups(world, cells, steps, ms):
    """MLUPS of all replicas together (weak scaling: every rank updates `cells` per step)."""
    return world * cells * steps / (ms * 1e3)


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def profiled_traffic(name):
    """dram bytes per launch recorded by an ncu capture summarised under profiles/."""
    p = os.path.join(ROOT, "profiles", name)
    try:
        with open(p) as f:
            for line in f:
                m = re.match(r"\s*traffic_bytes_per_launch:\s*([0-9.eE+]+)", line)
                if m:
                    return float(m.group(1))
    except OSError:
        pass
    return None


class ClockSampler:
    """Samples nvidia-smi clocks and throttle reasons while the GPU runs the
    timed work. The GPU is selected by its UUID (nvidia-smi numbers GPUs
    its own way and ignores CUDA_VISIBLE_DEVICES); each sample carries
    nvidia-smi's own timestamp, so the summary can keep only the samples
    taken inside a window of host wall-clock time."""

    FIELDS = ("timestamp,index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device, period_ms=50):
        self.gpu = self.gpu_selector(device)
        self.period_ms = period_ms
        self.proc = None
        self.lines = []

    @staticmethod
    def gpu_selector(device):
        """nvidia-smi -i argument of a torch CUDA device: GPU-<uuid>, else the PCI bus id."""
        try:
            import torch
            p = torch.cuda.get_device_properties(device)
            u = str(getattr(p, "uuid", "") or "")
            if u:
                return u if u.startswith("GPU-") else "GPU-" + u
            return "%08x:%02x:%02x.0" % (p.pci_domain_id, p.pci_bus_id, p.pci_device_id)
        except Exception:
            return None

    def start(self):
        if self.gpu is None:
            return
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", self.gpu, "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", str(self.period_ms)],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self, window=None):
        """Summary of the samples whose timestamp lies in window = (t0, t1) (time.time() values)."""
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"], "samples": 0}
        time.sleep(2.0 * self.period_ms / 1000.0)  # let the last samples of the window arrive
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.t.join(timeout=2)
        out = self.summarise(self.lines, window)
        out["gpu"] = self.gpu
        return out

    @staticmethod
    def parse_time(stamp):
        """Seconds since the epoch of an nvidia-smi timestamp ("2026/12/04 14:01:02.123", local time)."""
        import datetime
        try:
            return datetime.datetime.strptime(stamp.strip(), "%Y/%m/%d %H:%M:%S.%f").timestamp()
        except ValueError:
            return None

    @staticmethod
    def summarise(lines, window=None):
        """Median SM clock over the samples (inside `window` when given), the
        maximum clock, and the throttle reasons active in any of them."""
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in lines:
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 10:
                continue
            if window is not None:
                t = ClockSampler.parse_time(parts[0])
                if t is None or not (window[0] <= t <= window[1]):
                    continue
            try:
                clk = float(parts[2])
                smax = float(parts[3])
            except ValueError:
                continue
            sm.append(clk)
            for nm, v in zip(names, parts[6:10]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        sm.sort()
        med = sm[len(sm) // 2] if sm else None
        return {"sm_mhz": med, "sm_max_mhz": smax, "reasons": sorted(reasons), "samples": len(sm)}


def cpu_sample(n, seconds=12.0, threads=0):
    """Oracle port of the reference's D3Q19 FP32 per-cell arithmetic on a z-slab sample of the n^3 lattice."""
    import numpy as np
    import oracle
    import neon_gb300 as ngb
    L = oracle.lib()
    threads = threads or L.orc_max_threads()
    ulb = 0.1
    omega = ngb.cavity_omega(n, ulb, 100.0)
    # a slab of the full lattice: all of x and y, a few z planes (+2 walls)
    nz = max(3, min(n, 2 + int(threads) * 2))
    V = n * n * nz
    flags = np.zeros(V, np.uint32)
    L.orc_cavity_flags(n, n, nz, 19, flags.ctypes.data_as(ctypes.c_void_p))
    a = np.zeros(19 * V, np.float32)
    L.orc_cavity_init(n, n, nz, 19, 1, ulb, a.ctypes.data_as(ctypes.c_void_p))
    b = a.copy()
    P = lambda x: x.ctypes.data_as(ctypes.c_void_p)
    us = L.orc_time_d3q19_f32(n, n, nz, 1, threads, omega, P(flags), P(a), P(b))
    steps = max(1, int(seconds * 1e6 / max(us, 1.0)))
    us = L.orc_time_d3q19_f32(n, n, nz, steps, threads, omega, P(flags), P(a), P(b))
    mlups = V * steps / us
    return mlups, threads, "D3Q19 FP32 reference arithmetic, %dx%dx%d slab of the %d^3 lattice, %d steps (%.1f s)" % (
        n, n, nz, n, steps, us / 1e6)


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    import oracle
    L = oracle.lib()
    threads = L.orc_max_threads()
    # each step: one timed slab sample (~1 s) of the same workload
    samples = []
    for i in range(args.warmup + args.steps):
        mlups, thr, desc = cpu_sample(args.n, seconds=0.5 if i < args.warmup else 1.0, threads=threads)
        if i >= args.warmup:
            samples.append(mlups)
        if len(samples) >= min(args.steps, 20):
            break
    value = sum(samples) / len(samples)
    line = {"metric": METRIC, "value": round(value, 2), "unit": UNIT, "n_gpus": args.gpus, "steps": len(samples),
            "warmup": args.warmup, "ms_per_step": None, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (lid-driven cavity set-up)",
            "impl": "reference",
            "config": {"workload": "D3Q19 BGK lid-driven cavity, dense %d^3, FP32 SoA" % args.n,
                       "lattice": "d3q19", "storage": "f32", "n": args.n},
            "cpu_baseline": {"value": round(value, 2), "unit": UNIT, "cores": thr, "kind": "port",
                             "sample": desc + "; reference not buildable here (needs spdlog/rapidjson/cmake)"},
            "e2e": {"value": round(value, 2), "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_ours(args):
    import torch
    import neon_gb300 as ngb
    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=dev)
    ngb.lib()
    n, lat, st = args.n, args.lattice, args.storage
    q = 19 if lat == "d3q19" else 27
    ulb, re_ = 0.1, 100.0
    omega = ngb.cavity_omega(n, ulb, re_)
    desc = ngb.lbm_dense_desc(n, n, n, q, st, omega, ngb.lid_wall_terms(q, ulb), box_cavity=True)
    tdt = {"f64": torch.float64, "f32": torch.float32, "f16off": torch.float16, "bf16off": torch.bfloat16}[st]
    V = n ** 3
    fa = torch.empty(q * V, dtype=tdt, device=dev)
    fb = torch.empty_like(fa)
    stream = torch.cuda.current_stream(dev)
    ngb.lbm_cavity_init(desc, ulb, fa, fb, None, stream=stream)
    ngb.lbm_dense_run(desc, fa, fb, args.warmup + (args.warmup % 2), stream=stream)
    torch.cuda.synchronize()

    def barrier():
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    # ---------------- device-resident timing (CUDA events on the launching stream)
    sampler = ClockSampler(local)
    barrier()
    sampler.start()
    time.sleep(0.3)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    ngb.lbm_dense_run(desc, fa, fb, args.steps, stream=stream)
    e1.record(stream)
    e1.synchronize()
    barrier()
    clocks = sampler.stop()
    ms = max_over_ranks(e0.elapsed_time(e1), world, dev)
    per_step_ms = ms / args.steps
    value = whole_job_mlups(world, V, args.steps, ms)
    bpu = BYTES_PER_UPDATE[(lat, st)]
    peak, peak_kind = measured_peaks()
    # algorithmic bytes of the cells a step updates (the (n-2)^3 bulk cells; walls are not moved)
    achieved = bpu * (n - 2) ** 3 / (per_step_ms * 1e-3) / 1e9
    traffic = profiled_traffic("lbm_%s_%s_dense_%d.md" % (lat, st, n))

    # ---------------- centre-line velocity profiles (RunCavityTwoPop.cu:110-148)
    if args.profiles and rank == 0:
        done = args.warmup + (args.warmup % 2) + args.steps
        u = torch.zeros(3 * V, dtype=torch.float64, device=dev)
        ngb.lbm_dense_macroscopic(desc, fa if args.steps % 2 == 0 else fb, None, u, stream=stream)
        os.makedirs(args.profiles, exist_ok=True)
        ngb.write_cavity_profiles(args.profiles, done, *ngb.cavity_profiles(u, n, n, n, ulb))
        del u

    # ---------------- end to end through the host-buffer C-ABI call
    e2e = None
    if not args.no_e2e:
        host_in = torch.empty(q * V, dtype=tdt, pin_memory=True)
        host_out = torch.empty_like(host_in)
        host_in.copy_(fa.cpu())
        ngb.lbm_dense_run_host(desc, host_in, host_out, fa, fb, 2, stream=stream)  # warm the path
        barrier()
        h0, h1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        h0.record(stream)
        ngb.lbm_dense_run_host(desc, host_in, host_out, fa, fb, args.steps, stream=stream)
        h1.record(stream)
        h1.synchronize()
        barrier()
        ems = max_over_ranks(h0.elapsed_time(h1), world, dev)
        nbytes = q * V * host_in.element_size()
        e2e = {"value": round(whole_job_mlups(world, V, args.steps, ems), 2), "unit": UNIT,
               "h2d_bytes_per_step": nbytes // args.steps, "d2h_bytes_per_step": nbytes // args.steps,
               "note": "one H2D of the populations, %d steps, one D2H of the result per timed call" % args.steps}

    extra = {}
    if args.extra and rank == 0:
        for (l2, s2) in [("d3q19", "f16off"), ("d3q19", "bf16off"), ("d3q27", "f32"), ("d3q27", "f16off"),
                         ("d3q19", "f64")]:
            extra["%s_%s" % (l2, s2)] = time_variant(ngb, torch, dev, n if s2 != "f64" else 256, l2, s2, args)

    if rank == 0:
        cpu = None
        if not args.no_cpu:
            mlups, thr, sample = cpu_sample(n)
            cpu = {"value": round(mlups, 2), "unit": UNIT, "cores": thr, "kind": "port", "sample": sample}
        line = {"metric": METRIC, "value": round(value, 2), "unit": UNIT, "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": round(per_step_ms, 4), "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32" if st != "f64" else "f64",
                "data": "synthetic (lid-driven cavity set-up, equilibrium start)",
                "config": {"workload": "%s BGK lid-driven cavity, dense %d^3, %s SoA populations" % (lat.upper(), n, st),
                           "lattice": lat, "storage": st, "n": n, "lid_u": ulb, "Re": re_,
                           "l2": "inputs larger than L2 (2 x %.1f GB population buffers)" % (q * V * fa.element_size() / 1e9),
                           "parallelism": "replicas" if world > 1 else "single GPU"},
                "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                             "frac": round(achieved / peak, 4), "traffic": traffic,
                             "peak_kind": peak_kind, "bytes_per_update": bpu, "updated_cells": (n - 2) ** 3,
                             "launches_per_step": ngb.lbm_dense_kernels_per_step(desc),
                             "frac_of_nominal_8TBs": round(achieved / 8000.0, 4)},
                "cpu_baseline": cpu, "e2e": e2e, "gpu_launches": args.steps * ngb.lbm_dense_kernels_per_step(desc),
                "clocks": clocks}
        if extra:
            line["variants"] = extra
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def run_sphere(args):
    """Flow over a sphere on bGrid (8^3 blocks), 512x256x256 box: MLUPS per
    active cell for the chosen storage, and the drag coefficient after
    `--sim-steps` steps against an FP64 run of the same case."""
    import torch
    import neon_gb300 as ngb
    dev = torch.device("cuda", 0)
    ngb.lib()
    g = ngb.sphere_config(args.scale)
    V = g.nx * g.ny * g.nz
    act = torch.zeros(V, dtype=torch.uint8, device=dev)
    cls = torch.zeros_like(act)
    ngb.geometry_sphere_tube(g, act, cls)
    grid = ngb.BGrid(g.nx, g.ny, g.nz, act)
    u_in, re_ = 0.05, 100.0
    nu = u_in * 2 * g.sphere_r / re_
    omega = 1.0 / (3.0 * nu + 0.5)
    q = 19 if args.lattice == "d3q19" else 27
    terms = ngb.lid_wall_terms(q, u_in)
    w = ngb.lattice(q)[1]
    nb = grid.n_blocks
    flags = torch.zeros(nb * 512, dtype=torch.int32, device=dev)
    d0 = grid.desc(q, args.storage, omega, moving_wall_terms=terms)
    ngb.bgrid_flags_from_dense(d0, g.nx, g.ny, g.nz, cls, flags)
    ngb.bgrid_wall_mask(d0, flags)

    def simulate(storage, steps, timed):
        d = grid.desc(q, storage, omega, moving_wall_terms=terms)
        tdt = {"f64": torch.float64, "f32": torch.float32, "f16off": torch.float16, "bf16off": torch.bfloat16}[storage]
        f = torch.zeros(nb, q, 512, dtype=tdt, device=dev)
        if storage in ("f64", "f32"):
            f += torch.tensor(w, dtype=tdt, device=dev)[None, :, None]
        a, b = f.reshape(-1), f.clone().reshape(-1)
        ms = None
        if timed:
            for s in range(args.warmup):
                ngb.bgrid_lbm_step(d, a, b, flags)
                a, b = b, a
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            for s in range(steps):
                ngb.bgrid_lbm_step(d, a, b, flags)
                a, b = b, a
            e1.record()
            e1.synchronize()
            ms = e0.elapsed_time(e1) / steps
        else:
            for s in range(steps):
                ngb.bgrid_lbm_step(d, a, b, flags)
                a, b = b, a
        partials = torch.zeros(3 * nb, dtype=torch.float64, device=dev)
        force = torch.zeros(3, dtype=torch.float64, device=dev)
        ngb.bgrid_drag(d, a, flags, partials, force)
        torch.cuda.synchronize()
        cd = 2.0 * force[0].item() / (u_in ** 2 * 3.141592653589793 * g.sphere_r ** 2)
        return ms, cd

    ms, _ = simulate(args.storage, args.steps, True)
    cd, cd64 = None, None
    if args.sim_steps > 0:
        _, cd = simulate(args.storage, args.sim_steps, False)
        _, cd64 = simulate("f64", args.sim_steps, False)
    n_act = grid.n_active_voxels
    bpu = BYTES_PER_UPDATE[(args.lattice, args.storage)]
    peak, kind = measured_peaks()
    achieved = bpu * n_act / (ms * 1e-3) / 1e9
    line = {"metric": "bGrid %s LBM MLUPS (active cells)" % args.lattice.upper(), "value": round(n_act / (ms * 1e3), 2),
            "unit": "MLUPS", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms, 4),
            "higher_is_better": True, "dtype": "f32", "data": "synthetic (sphere + seeded tube geometry)",
            "config": {"workload": "flow over a sphere, bGrid 8^3 blocks, %dx%dx%d, %s storage" % (g.nx, g.ny, g.nz,
                                                                                                args.storage),
                       "active_blocks": nb, "candidate_blocks": grid.bnx * grid.bny * grid.bnz,
                       "block_occupancy": round(nb / (grid.bnx * grid.bny * grid.bnz), 4),
                       "active_voxels": n_act, "u_in": u_in, "Re_D": re_, "omega": omega},
            "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                         "frac": round(achieved / peak, 4), "peak_kind": kind, "bytes_per_update": bpu,
                         "note": "algorithmic bytes exclude the 4-byte flag and block metadata"},
            "drag": {"steps": args.sim_steps, "cd": cd, "cd_f64": cd64,
                     "rel_err": (abs(cd - cd64) / abs(cd64)) if cd is not None and cd64 else None},
            "gpu_launches": args.steps}
    print(json.dumps(line), flush=True)


def run_poisson(args):
    """Poisson -lap(u) = f, zero Dirichlet box, 8 seeded Gaussians (sigma 8):
    seconds and iterations of the device Jacobi-PCG (FP32 fields, FP64
    reductions and solution, true residual every 50 iterations) to 1e-8."""
    import torch
    import neon_gb300 as ngb
    dev = torch.device("cuda", 0)
    ngb.lib()
    n = args.n
    d = ngb.poisson_desc(n, n, n, "f32", 1.0)
    c, a = ngb.gaussian_sources(n, n, n, 2024)
    b = torch.empty(n ** 3, dtype=torch.float32, device=dev)
    ngb.poisson_rhs(d, torch.from_numpy(c).to(dev), torch.from_numpy(a).to(dev), 8.0, b)
    ws = ngb.cg_workspace(d, dev)
    results = []
    for rep in range(max(1, args.steps)):
        x = torch.zeros(n ** 3, dtype=torch.float64, device=dev)
        torch.cuda.synchronize()
        r = ngb.cg_solve(d, b, x, ws, tol=1e-8, max_iter=20000, refresh_every=50, check_every=50, jacobi=True)
        results.append(r)
    best = min(results, key=lambda r: r["seconds"])
    it = best["iterations"]
    peak, kind = measured_peaks()
    per_it = best["seconds"] / max(it, 1)
    achieved = 40.0 * n ** 3 / per_it / 1e9
    line = {"metric": "Poisson seconds to 1e-8 (Jacobi-PCG)", "value": round(best["seconds"], 4), "unit": "s",
            "n_gpus": 1, "steps": len(results), "warmup": 0, "higher_is_better": False, "dtype": "f32",
            "data": "synthetic (8 seeded Gaussians, sigma 8)",
            "config": {"workload": "Poisson 7-point, zero Dirichlet, %d^3, FP32 fields / FP64 reductions" % n,
                       "iterations": it, "rel_residual": best["rel_residual"], "refreshes": best["refreshes"],
                       "converged": best["converged"]},
            "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                         "frac": round(achieved / peak, 4), "peak_kind": kind,
                         "bytes_per_dof_iteration": 40,
                         "note": "whole-solve average incl. polls and refreshes"}}
    print(json.dumps(line), flush=True)


def run_learned(args):
    """Learned preconditioner: a 3-level U-Net (16/32/64 channels, BF16 tensor-core
    convolutions) trained on residual/error pairs that CG itself produces on
    seeded k^-2 Gaussian random fields at --train-n, then used inside flexible
    CG (with Jacobi-PCG fallback on stagnation) on the Gaussian-source Poisson
    problem at --n, against device Jacobi-PCG on the same problem; both to a
    1e-8 relative true residual. For --n > --train-n the network is the
    coarsest-level solve of a V-cycle (damped-Jacobi smoothing and
    full-weighting / trilinear transfers on the levels between --n and
    --train-n); the same cycle without the network is timed beside it. For
    --n == --train-n the network preconditions the fine grid directly.
    `value` is the FCG solve time (seconds)."""
    import torch
    import neon_gb300 as ngb
    from neon_gb300 import fcg
    from neon_gb300.learned import UNet
    dev = torch.device("cuda", 0)
    ngb.lib()
    n = args.n
    # --- training (or loading) the network
    net = UNet(seed=0, device=dev)
    train = {"pairs": 0, "seconds": 0.0, "loss_first": None, "loss_last": None}
    if args.weights:
        net.load_state_dict(torch.load(args.weights))
        train["weights"] = os.path.basename(args.weights)
    else:
        captures = (2, 5, 10, 20, 40, 80, 120, 160, 200, 250)
        systems = max(1, args.train_pairs // len(captures))
        t0 = time.perf_counter()
        pairs = fcg.make_training_set(args.train_n, systems, captures, seed=2024, device=dev)
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        losses = fcg.train(net, pairs, epochs=args.epochs, lr=args.lr)
        torch.cuda.synchronize()
        t2 = time.perf_counter()
        k = max(1, len(losses) // 10)
        train.update(pairs=len(pairs), seconds=round(t2 - t0, 1), data_seconds=round(t1 - t0, 1),
                     loss_first=round(sum(losses[:k]) / k, 4), loss_last=round(sum(losses[-k:]) / k, 4))
        del pairs
        torch.cuda.empty_cache()
        if args.save_weights:
            torch.save({k2: v.cpu() for k2, v in net.w.items()}, args.save_weights)
    # --- the Poisson problem of the Jacobi-PCG benchmark
    d = ngb.poisson_desc(n, n, n, "f32", 1.0)
    c, a = ngb.gaussian_sources(n, n, n, 2024)
    b = torch.empty(n ** 3, dtype=torch.float32, device=dev)
    ngb.poisson_rhs(d, torch.from_numpy(c).to(dev), torch.from_numpy(a).to(dev), 8.0, b)
    ws = ngb.cg_workspace(d, dev)
    x = torch.zeros(n ** 3, dtype=torch.float64, device=dev)
    pcg = ngb.cg_solve(d, b, x, ws, tol=1e-8, max_iter=20000, refresh_every=50, check_every=50, jacobi=True)
    # FCG preconditioned by the V-cycle whose coarsest level (--train-n) is the network
    levels = max(0, int(round(math.log2(n / args.train_n))))
    if args.train_n << levels != n:
        raise SystemExit("learned: --n must be --train-n times a power of two")
    vc = fcg.VCycle(n, levels, net, device=dev) if levels > 0 else None
    if vc is not None:
        vc(b)  # warm-up (network buffers at the coarsest size)
        torch.cuda.synchronize()
        x2 = torch.zeros(n ** 3, dtype=torch.float64, device=dev)
        res = fcg.fcg_solve_vcycle(vc, b, x2, tol=1e-8, max_iter=2000, fallback=True, ws=ws)
        # the same cycle without the network (coarsest correction zero)
        x3 = torch.zeros(n ** 3, dtype=torch.float64, device=dev)
        plain = fcg.fcg_solve_vcycle(fcg.VCycle(n, levels, coarse="none", device=dev), b, x3, tol=1e-8, max_iter=4000,
                                     fallback=True, ws=ws)
    else:
        net.forward(b)
        torch.cuda.synchronize()
        x2 = torch.zeros(n ** 3, dtype=torch.float64, device=dev)
        res = fcg.fcg_solve(net, b, x2, tol=1e-8, max_iter=2000, fallback=True, ws=ws)
        plain = None
    agree = float((x2 - x).norm() / x.norm())
    # U-Net forward cost at the size it runs at (device time)
    nn_ = n >> levels
    rc = b[:nn_ ** 3].clone()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(3):
        net.forward(rc)
    e1.record()
    e1.synchronize()
    fwd_ms = e0.elapsed_time(e1) / 3
    cfg = {"workload": "Poisson 7-point, zero Dirichlet, %d^3; FCG(1) with a V-cycle of %d damped-Jacobi levels whose "
                       "coarsest (%d^3) solve is the U-Net 16/32/64 trained at %d^3" % (n, levels, nn_, args.train_n),
           "fcg_iterations": res["iterations"], "fcg_fallback": res["fallback"],
           "fallback_iterations": res["fallback_iterations"], "fcg_rel_residual": res["rel_residual"],
           "converged": res["converged"], "pcg_seconds": round(pcg["seconds"], 4),
           "pcg_iterations": pcg["iterations"], "speedup_vs_pcg": round(pcg["seconds"] / res["seconds"], 3),
           "solution_rel_diff": agree, "unet_forward_ms": round(fwd_ms, 3),
           "unet_forward_tflops": round(net.flops_forward(nn_) / fwd_ms / 1e9, 1), "training": train}
    if plain is not None:
        cfg["without_network"] = {"seconds": round(plain["seconds"], 4), "iterations": plain["iterations"],
                                  "fallback": plain["fallback"], "fallback_iterations": plain["fallback_iterations"],
                                  "converged": plain["converged"]}
    line = {"metric": "Poisson seconds to 1e-8: learned FCG vs Jacobi-PCG", "value": round(res["seconds"], 4), "unit": "s",
            "n_gpus": 1, "steps": 1, "warmup": 1, "higher_is_better": False, "dtype": "bf16",
            "data": "synthetic (8 seeded Gaussians, sigma 8; training on seeded k^-2 fields)", "config": cfg}
    print(json.dumps(line), flush=True)


def bf16_peak():
    """Dense BF16 tensor peak (TFLOP/s, burst) measured on this machine, else the fallback."""
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["bf16_tflops"]), "measured"
    except Exception:
        return 1900.0, "fallback"


def run_unet(args):
    """Forward applications of the learned preconditioner's network (3-level
    U-Net, 16/32/64 channels, BF16 operands on the tcgen05 tensor cores, FP32
    accumulate) at --n^3 with seeded weights and a seeded input; a step is one
    application (10 convolutions, 2 pools, 2 upsamplings). `value` is TFLOP/s
    of the whole application; the roofline is the measured BF16 dense peak."""
    import torch
    import neon_gb300 as ngb
    from neon_gb300.learned import UNet
    dev = torch.device("cuda", 0)
    ngb.lib()
    n = args.n
    net = UNet(seed=0, device=dev)
    g = torch.Generator(device=dev)
    g.manual_seed(2024)
    r = torch.randn(n ** 3, device=dev, generator=g)
    s = torch.cuda.current_stream(dev)
    for _ in range(max(3, args.warmup)):
        net.forward(r)
    torch.cuda.synchronize()
    clk = ClockSampler(torch.cuda.current_device())
    clk.start()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(s)
    for _ in range(args.steps):
        net.forward(r)
    e1.record(s)
    e1.synchronize()
    clocks = clk.stop()
    ms = e0.elapsed_time(e1) / args.steps
    flops = net.flops_forward(n)
    tflops = flops / (ms * 1e-3) / 1e12
    peak, kind = bf16_peak()
    line = {"metric": "U-Net preconditioner forward TFLOP/s", "value": round(tflops, 1), "unit": "TFLOP/s", "n_gpus": 1,
            "steps": args.steps, "warmup": max(3, args.warmup), "ms_per_step": round(ms, 3), "higher_is_better": True,
            "scaling": "none", "vs_baseline": None, "dtype": "bf16", "data": "synthetic (seeded weights and input)",
            "config": {"workload": "U-Net 16/32/64, 3x3x3 convolutions, %d^3, one forward application per step" % n,
                       "flop_per_step": flops, "inputs_vs_l2": "activations of %.1f GB per application, larger than L2" % (
                           n ** 3 * 2 * (16 + 16 + 48 + 16) / 1e9)},
            "roofline": {"bound": "tensor", "achieved": round(tflops, 1), "peak": peak, "unit": "TFLOP/s",
                         "frac": round(tflops / peak, 4), "peak_kind": kind, "traffic": None},
            "clocks": clocks, "gpu_launches": 14 * args.steps}
    print(json.dumps(line), flush=True)


def run_accuracy(args):
    """Lid-driven cavity at --n for --sim-steps steps (default 2000) in every
    storage form of the lattice: MLUPS of each run and the relative L2 error of
    its velocity field (bulk cells) against the FP64 run."""
    import torch
    import neon_gb300 as ngb
    dev = torch.device("cuda", 0)
    ngb.lib()
    n, q = args.n, 19 if args.lattice == "d3q19" else 27
    steps = args.sim_steps or 2000
    ulb, re_ = 0.1, 100.0
    V = n ** 3
    tdts = {"f64": torch.float64, "f32": torch.float32, "f16off": torch.float16, "bf16off": torch.bfloat16}
    u_ref, out = None, {}
    for st in ("f64", "f32", "f16off", "bf16off"):
        desc = ngb.lbm_dense_desc(n, n, n, q, st, ngb.cavity_omega(n, ulb, re_), ngb.lid_wall_terms(q, ulb))
        fa = torch.empty(q * V, dtype=tdts[st], device=dev)
        fb = torch.empty_like(fa)
        ngb.lbm_cavity_init(desc, ulb, fa, fb)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        ngb.lbm_dense_run(desc, fa, fb, steps)
        e1.record()
        e1.synchronize()
        ms = e0.elapsed_time(e1) / steps
        fin = fa if steps % 2 == 0 else fb
        u = torch.zeros(3 * V, dtype=torch.float64, device=dev)
        ngb.lbm_dense_macroscopic(desc, fin, None, u)
        del fa, fb
        torch.cuda.empty_cache()
        if st == "f64":
            u_ref = u
            out[st] = {"mlups": round(V / (ms * 1e3), 1)}
        else:
            # bulk cells only (the interior; lid and wall cells carry identical set values)
            du = (u - u_ref).view(3, n, n, n)[:, 1:-1, 1:-1, 1:-1]
            err = float(du.norm() / u_ref.view(3, n, n, n)[:, 1:-1, 1:-1, 1:-1].norm())
            out[st] = {"mlups": round(V / (ms * 1e3), 1), "velocity_l2_rel_err_vs_f64": err}
            del u
    line = {"metric": "%s cavity velocity L2 error vs FP64" % args.lattice.upper(), "value": out["f16off"]["velocity_l2_rel_err_vs_f64"],
            "unit": "relative L2", "n_gpus": 1, "steps": steps, "warmup": 0, "higher_is_better": False, "dtype": "f32",
            "data": "synthetic (lid-driven cavity set-up, equilibrium start)",
            "config": {"workload": "%s BGK lid-driven cavity, dense %d^3, %d steps" % (args.lattice.upper(), n, steps),
                       "lid_u": ulb, "Re": re_, "forms": out,
                       "f16_speedup_vs_f32": round(out["f16off"]["mlups"] / out["f32"]["mlups"], 3)}}
    print(json.dumps(line), flush=True)


def time_variant(ngb, torch, dev, n, lat, st, args):
    q = 19 if lat == "d3q19" else 27
    ulb = 0.1
    desc = ngb.lbm_dense_desc(n, n, n, q, st, ngb.cavity_omega(n, ulb, 100.0), ngb.lid_wall_terms(q, ulb))
    tdt = {"f64": torch.float64, "f32": torch.float32, "f16off": torch.float16, "bf16off": torch.bfloat16}[st]
    V = n ** 3
    fa = torch.empty(q * V, dtype=tdt, device=dev)
    fb = torch.empty_like(fa)
    s = torch.cuda.current_stream(dev)
    ngb.lbm_cavity_init(desc, ulb, fa, fb, None, stream=s)
    ngb.lbm_dense_run(desc, fa, fb, 10, stream=s)
    steps = max(10, args.steps // 2 * 2)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(s)
    ngb.lbm_dense_run(desc, fa, fb, steps, stream=s)
    e1.record(s)
    e1.synchronize()
    ms = e0.elapsed_time(e1) / steps
    bpu = BYTES_PER_UPDATE[(lat, st)]
    del fa, fb
    torch.cuda.empty_cache()
    return {"n": n, "mlups": round(V / (ms * 1e3), 1), "ms_per_step": round(ms, 4),
            "achieved_gbs": round(bpu * (n - 2) ** 3 / (ms * 1e-3) / 1e9, 1), "bytes_per_update": bpu}


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == "sphere":
        run_sphere(args)
    elif args.workload == "poisson":
        run_poisson(args)
    elif args.workload == "learned":
        run_learned(args)
    elif args.workload == "unet":
        run_unet(args)
    elif args.workload == "accuracy":
        run_accuracy(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
