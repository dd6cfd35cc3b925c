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
result, all inside the timed region). The same line carries the second half
of the metric, Poisson seconds to 1e-8 at 512^3 (`poisson`: device
Jacobi-PCG with its per-pass roofline, and the learned preconditioner's FCG
with and without its network, training included), the 16-bit storage forms
of the cavity (`storage_16bit`) and the bGrid flow-over-sphere case
(`sphere`).

`--impl reference` times the CPU restatement of the reference's per-cell
D3Q19 FP32 arithmetic (the oracle port, bit-exact to the reference's own CPU
backend where that is built) on all host threads, on the full lattice of the
same configuration.
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
                    ("d3q19", "f16sr"): 76, ("d3q27", "f32"): 216, ("d3q27", "f64"): 432, ("d3q27", "f16off"): 108,
                    ("d3q27", "bf16off"): 108, ("d3q27", "f16sr"): 108}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=None,
                    help="timed steps (default 200; poisson: repeated solves, default 3)")
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n", type=int, default=0, help="grid size (default: 384 for the LBM workloads, 512 for poisson/learned, 256 for unet)")
    ap.add_argument("--lattice", default="d3q19", choices=["d3q19", "d3q27"])
    ap.add_argument("--storage", default="f32", choices=["f64", "f32", "f16off", "bf16off", "f16sr"])
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--extra", action="store_true", help="also time the other storage/lattice forms")
    ap.add_argument("--no-sections", action="store_true",
                    help="cavity: leave out the poisson, storage_16bit, sphere and unet sections of the line")
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
    ap.add_argument("--epochs", type=int, default=3, help="learned: training epochs")
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


def cavity_config(n, lat, st, q, esz, world):
    """The `config` object of the cavity line (identical for both arms)."""
    return {"workload": "%s BGK lid-driven cavity, dense %d^3, %s SoA populations" % (lat.upper(), n, st),
            "lattice": lat, "storage": st, "n": n, "lid_u": 0.1, "Re": 100.0,
            "l2": "inputs larger than L2 (2 x %.1f GB population buffers)" % (q * n ** 3 * esz / 1e9),
            "parallelism": "replicas" if world > 1 else "single GPU"}


class OracleCavity:
    """The oracle port of the reference's D3Q19 FP32 per-cell arithmetic on
    the full n^3 lattice (host buffers, all host threads)."""

    def __init__(self, n, threads=0):
        import numpy as np
        import oracle
        import neon_gb300 as ngb
        self.L = oracle.lib()
        self.n = n
        self.threads = threads or self.L.orc_max_threads()
        self.omega = ngb.cavity_omega(n, 0.1, 100.0)
        V = n ** 3
        self.flags = np.zeros(V, np.uint32)
        self.L.orc_cavity_flags(n, n, n, 19, self.flags.ctypes.data_as(ctypes.c_void_p))
        self.a = np.zeros(19 * V, np.float32)
        self.L.orc_cavity_init(n, n, n, 19, 1, 0.1, self.a.ctypes.data_as(ctypes.c_void_p))
        self.b = self.a.copy()

    def steps(self, k):
        """Runs k steps; returns MLUPS (N^3 per step, as Metrics.h)."""
        P = lambda x: x.ctypes.data_as(ctypes.c_void_p)  # noqa: E731
        n = self.n
        us = self.L.orc_time_d3q19_f32(n, n, n, k, self.threads, self.omega, P(self.flags), P(self.a), P(self.b))
        if k % 2:
            self.a, self.b = self.b, self.a
        return n ** 3 * k / us, us / 1e6


def cpu_sample(n, steps=6):
    """cpu_baseline of the cavity line: `steps` full-lattice steps of the oracle port."""
    oc = OracleCavity(n)
    oc.steps(2)  # warm-up (first touch of the buffers)
    mlups, sec = oc.steps(steps)
    return mlups, oc.threads, "D3Q19 FP32 reference arithmetic, full %d^3 lattice, %d steps (%.1f s)" % (n, steps, sec)


def run_reference(args):
    """The reference arm: the oracle port of the reference's D3Q19 FP32 step
    (bit-exact to the reference's CPU backend where that is built from its
    sources) on all host threads, the full lattice of the same config; each
    of --steps timed steps is one full-lattice step."""
    rank, world, _ = dist_env()
    if rank != 0:
        return
    n = args.n
    oc = OracleCavity(n)
    oc.steps(max(1, args.warmup))
    per = []
    for _ in range(args.steps):
        mlups, sec = oc.steps(1)
        per.append(sec)
    total = sum(per)
    value = n ** 3 * len(per) / (total * 1e6)
    line = {"metric": METRIC, "value": round(value, 2), "unit": UNIT, "n_gpus": args.gpus, "steps": len(per),
            "warmup": args.warmup, "ms_per_step": round(1e3 * total / len(per), 2), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (lid-driven cavity set-up, equilibrium start)", "impl": "reference",
            "config": cavity_config(n, "d3q19", "f32", 19, 4, world),
            "cpu_baseline": {"value": round(value, 2), "unit": UNIT, "cores": oc.threads, "kind": "port",
                             "sample": "D3Q19 FP32 reference arithmetic, full %d^3 lattice, %d timed steps (%.1f s); "
                                       "the oracle port equals the reference's own CPU backend bit for bit, but that "
                                       "build needs the reference sources, which are not on this machine" % (
                                           n, len(per), total)},
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
    tdt = TORCH_DTYPES[st](torch)
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
    # The timed steps sit inside a clock window: the same step graph runs for
    # about a second before and half a second after them, while nvidia-smi
    # samples the GPU every 50 ms; the clocks record keeps the samples of
    # that window (the timed region alone is a few milliseconds).
    sampler = ClockSampler(dev)
    barrier()
    sampler.start()
    time.sleep(0.2)
    ms_step_est = max(0.05, 152.0 * V / 6.0e12 * 1e3)
    load_steps = 2 * max(1, int(1000.0 / ms_step_est) // 2)
    w0 = time.time()
    ngb.lbm_dense_run(desc, fa, fb, load_steps, stream=stream)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    ngb.lbm_dense_run(desc, fa, fb, args.steps, stream=stream)
    e1.record(stream)
    ngb.lbm_dense_run(desc, fa, fb, load_steps // 2 * 2, stream=stream)
    stream.synchronize()
    w1 = time.time()
    barrier()
    clocks = sampler.stop(window=(w0, w1))
    clocks["window"] = "the timed steps inside %.2f s of the same steps (%d before, %d after)" % (
        w1 - w0, load_steps, load_steps // 2 * 2)
    ms = max_over_ranks(e0.elapsed_time(e1), world, dev)
    per_step_ms = ms / args.steps
    value = whole_job_mlups(world, V, args.steps, ms)
    bpu = BYTES_PER_UPDATE[(lat, st)]
    peak, peak_kind = measured_peaks()
    # algorithmic bytes of the cells a step updates (the (n-2)^3 bulk cells; walls are not moved)
    achieved = bpu * (n - 2) ** 3 / (per_step_ms * 1e-3) / 1e9
    traffic = profiled_traffic("lbm_%s_%s_dense_%d.md" % (lat, st, n))
    done_steps = args.warmup + (args.warmup % 2) + load_steps + args.steps + load_steps // 2 * 2

    # ---------------- centre-line velocity profiles (RunCavityTwoPop.cu:110-148)
    if args.profiles and rank == 0:
        u = torch.zeros(3 * V, dtype=torch.float64, device=dev)
        ngb.lbm_dense_macroscopic(desc, fa if done_steps % 2 == 0 else fb, None, u, stream=stream)
        os.makedirs(args.profiles, exist_ok=True)
        ngb.write_cavity_profiles(args.profiles, done_steps, *ngb.cavity_profiles(u, n, n, n, ulb))
        del u

    # ---------------- end to end through the host-buffer C-ABI call
    e2e = None
    if not args.no_e2e:
        host_in = torch.empty(q * V, dtype=tdt, pin_memory=True)
        host_out = torch.empty(q * V, dtype=tdt, pin_memory=True)  # empty_like would drop the pinning
        host_in.copy_(fa.cpu())
        ngb.lbm_dense_run_host(desc, host_in, host_out, fa, fb, 2, stream=stream)  # warm the path
        # three timed calls (host-link throughput varies between calls); the median is the value
        calls = []
        for _ in range(3):
            barrier()
            h0, h1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            h0.record(stream)
            ngb.lbm_dense_run_host(desc, host_in, host_out, fa, fb, args.steps, stream=stream)
            h1.record(stream)
            h1.synchronize()
            barrier()
            calls.append(max_over_ranks(h0.elapsed_time(h1), world, dev))
        ems = sorted(calls)[1]
        nbytes = q * V * host_in.element_size()
        # the host link alone (one H2D and one D2H of the populations), for the record
        c0, c1, c2 = (torch.cuda.Event(enable_timing=True) for _ in range(3))
        c0.record(stream)
        fa.copy_(host_in, non_blocking=True)
        c1.record(stream)
        host_out.copy_(fa, non_blocking=True)
        c2.record(stream)
        c2.synchronize()
        link = {"h2d_gbs": round(nbytes / (c0.elapsed_time(c1) * 1e-3) / 1e9, 1),
                "d2h_gbs": round(nbytes / (c1.elapsed_time(c2) * 1e-3) / 1e9, 1)}
        e2e = {"value": round(whole_job_mlups(world, V, args.steps, ems), 2), "unit": UNIT,
               "h2d_bytes_per_step": nbytes // args.steps, "d2h_bytes_per_step": nbytes // args.steps,
               "calls_ms": [round(c, 2) for c in calls], "host_link": link,
               "note": "one H2D of the populations, %d steps, one D2H of the result per timed call; median of "
                       "three calls" % args.steps}
        del host_in, host_out

    launches = args.steps * ngb.lbm_dense_kernels_per_step(desc)
    del fa, fb
    torch.cuda.empty_cache()

    extra = {}
    if args.extra and rank == 0:
        for (l2, s2) in [("d3q19", "bf16off"), ("d3q27", "f32"), ("d3q27", "f16off"), ("d3q19", "f64")]:
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
                "config": cavity_config(n, lat, st, q, TORCH_ITEMSIZE[st], world),
                "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                             "frac": round(achieved / peak, 4), "traffic": traffic,
                             "peak_kind": peak_kind, "bytes_per_update": bpu, "updated_cells": (n - 2) ** 3,
                             "launches_per_step": ngb.lbm_dense_kernels_per_step(desc),
                             "frac_of_nominal_8TBs": round(achieved / 8000.0, 4)},
                "cpu_baseline": cpu, "e2e": e2e, "gpu_launches": launches, "clocks": clocks}
        if not args.no_sections and lat == "d3q19" and st == "f32":
            line["storage_16bit"] = storage_16bit_section(ngb, torch, dev, n, args, per_step_ms)
            line["poisson"] = poisson_section(args)
            line["sphere"] = sphere_section(args)
            line["unet"] = unet_section(args)
        if extra:
            line["variants"] = extra
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


TORCH_DTYPES = {"f64": lambda t: t.float64, "f32": lambda t: t.float32, "f16off": lambda t: t.float16,
                "bf16off": lambda t: t.bfloat16, "f16sr": lambda t: t.float16}
TORCH_ITEMSIZE = {"f64": 8, "f32": 4, "f16off": 2, "bf16off": 2, "f16sr": 2}


def storage_16bit_section(ngb, torch, dev, n, args, f32_ms):
    """The 16-bit offset storage forms of the same cavity (g = f - w stored in
    16 bits, FP32 collision): MLUPS, ratio to the FP32 step timed above, and
    their roofline (76 B per update). f16sr stores with stochastic rounding
    (the form that meets the accuracy target), f16off rounds to nearest."""
    out = {}
    peak, kind = measured_peaks()
    for st in ("f16sr", "f16off"):
        v = time_variant(ngb, torch, dev, n, "d3q19", st, args)
        v["speedup_vs_f32"] = round(f32_ms / v["ms_per_step"], 3)
        v["roofline_frac"] = round(v["achieved_gbs"] / peak, 4)
        out[st] = v
    out["peak_kind"] = kind
    out["target"] = ">= 1.7x the FP32 MLUPS at <= 1e-3 velocity error vs FP64 (accuracy: --workload accuracy)"
    return out


def run_sphere(args, emit=True):
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
    del grid, flags, act, cls
    torch.cuda.empty_cache()
    if not emit:
        return line
    print(json.dumps(line), flush=True)


def poisson_problem(n, dev):
    """Config 3's Poisson case at n^3: zero Dirichlet box, f = 8 seeded Gaussians (sigma 8), FP32 fields."""
    import torch
    import neon_gb300 as ngb
    d = ngb.poisson_desc(n, n, n, "f32", 1.0)
    c, a = ngb.gaussian_sources(n, n, n, 2024)
    b = torch.empty(n ** 3, dtype=torch.float32, device=dev)
    ngb.poisson_rhs(d, torch.from_numpy(c).to(dev), torch.from_numpy(a).to(dev), 8.0, b)
    return d, b


def jacobi_pcg_run(d, b, n, dev, reps=1):
    """Device Jacobi-PCG to 1e-8 (FP32 fields, FP64 reductions and solution,
    true residual every 50 iterations): the best of `reps` solves, with the
    per-pass roofline (pass A 16 B/DOF, pass B 24 B/DOF per launch) from
    CUDA events on 20 launches of each pass."""
    import torch
    import neon_gb300 as ngb
    ws = ngb.cg_workspace(d, dev)
    results = []
    for _ in range(max(1, reps)):
        x = torch.zeros(n ** 3, dtype=torch.float64, device=dev)
        torch.cuda.synchronize()
        results.append(ngb.cg_solve(d, b, x, ws, tol=1e-8, max_iter=20000, refresh_every=50, check_every=50,
                                    jacobi=True))
    best = min(results, key=lambda r: r["seconds"])
    x0 = torch.zeros(n ** 3, dtype=torch.float64, device=dev)
    ms_a, ms_b = ngb.cg_time_passes(d, b, x0, ws, reps=20)
    peak, kind = measured_peaks()
    it = best["iterations"]
    whole = 40.0 * n ** 3 * it / best["seconds"] / 1e9
    passes = {"pass_a": {"ms": round(ms_a, 4), "bytes_per_dof": 16,
                         "achieved_gbs": round(16.0 * n ** 3 / (ms_a * 1e-3) / 1e9, 1)},
              "pass_b": {"ms": round(ms_b, 4), "bytes_per_dof": 24,
                         "achieved_gbs": round(24.0 * n ** 3 / (ms_b * 1e-3) / 1e9, 1)}}
    for v in passes.values():
        v["frac"] = round(v["achieved_gbs"] / peak, 4)
    out = {"seconds": round(best["seconds"], 4), "iterations": it, "rel_residual": best["rel_residual"],
           "converged": best["converged"], "refreshes": best["refreshes"], "solves": len(results),
           "roofline": {"bound": "hbm", "peak": peak, "peak_kind": kind, "unit": "GB/s",
                        "whole_solve_achieved": round(whole, 1), "whole_solve_frac": round(whole / peak, 4),
                        "bytes_per_dof_iteration": 40, **passes},
           "gpu_launches_per_iteration": 2, "launches_per_refresh": 2}
    return out, ws


def learned_fcg_run(args, n, dev, b, ws, pcg_seconds):
    """Learned preconditioner: a 3-level U-Net (16/32/64 channels, BF16
    tensor-core convolutions) trained on residual/error pairs that CG itself
    produces on seeded k^-2 Gaussian random fields at --train-n, then used
    inside flexible CG (Jacobi-PCG fallback on stagnation) to a 1e-8 relative
    true residual. For n > --train-n the network is the coarsest-level solve
    of a V-cycle (damped-Jacobi smoothing, full-weighting / trilinear
    transfers); the same cycle without the network is timed beside it."""
    import torch
    import neon_gb300 as ngb
    from neon_gb300 import fcg
    from neon_gb300.learned import UNet
    net = UNet(seed=0, device=dev)
    train = {"pairs": 0, "seconds": 0.0, "loss_first": None, "loss_last": None}
    if args.weights:
        net.load_weights(args.weights)
        train["weights"] = os.path.basename(args.weights)
    else:
        captures = (2, 5, 10, 20, 40, 80, 120, 160, 200, 250)
        t0 = time.perf_counter()
        pairs = fcg.make_training_set(args.train_n, captures=captures, seed=2024, device=dev, count=args.train_pairs)
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        losses = fcg.train(net, pairs, epochs=args.epochs, lr=args.lr)
        torch.cuda.synchronize()
        t2 = time.perf_counter()
        k = max(1, len(losses) // 10)
        train.update(pairs=len(pairs), seconds=round(t2 - t0, 1), data_seconds=round(t1 - t0, 1),
                     train_n=args.train_n, epochs=args.epochs,
                     loss_first=round(sum(losses[:k]) / k, 4), loss_last=round(sum(losses[-k:]) / k, 4))
        del pairs
        torch.cuda.empty_cache()
        if args.save_weights:
            net.save_weights(args.save_weights)
    levels = max(0, int(round(math.log2(n / args.train_n))))
    if args.train_n << levels != n:
        raise SystemExit("learned: --n must be --train-n times a power of two")
    plain = None
    if levels > 0:
        # the solve through the C ABI (ngb_learned_solve): V-cycle, network, FCG and FP64 true residual in the library
        solver = ngb.LearnedSolver(n, levels, net.flat_weights())
        z = torch.empty_like(b)
        solver.precondition(b, z)  # warm-up (first launches of every kernel)
        torch.cuda.synchronize()
        del z
        x2 = torch.zeros(n ** 3, dtype=torch.float64, device=dev)
        res = solver.solve(b, x2, tol=1e-8, max_iter=2000, refresh_every=10, stall=30, fallback=True)
        solver.close()
        # the same cycle without the network, through the same C-ABI solve
        plain_solver = ngb.LearnedSolver(n, levels, None)
        z = torch.empty_like(b)
        plain_solver.precondition(b, z)
        torch.cuda.synchronize()
        del z
        x3 = torch.zeros(n ** 3, dtype=torch.float64, device=dev)
        plain = plain_solver.solve(b, x3, tol=1e-8, max_iter=4000, refresh_every=10, stall=30, fallback=True)
        plain_solver.close()
        del x3
    else:
        net.forward(b)
        torch.cuda.synchronize()
        x2 = torch.zeros(n ** 3, dtype=torch.float64, device=dev)
        res = fcg.fcg_solve(net, b, x2, tol=1e-8, max_iter=2000, fallback=True, ws=ws)
    nn_ = n >> levels
    rc = b[:nn_ ** 3].clone()
    net.forward(rc)  # warm-up: a network loaded from a file has not run yet
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(3):
        net.forward(rc)
    e1.record()
    e1.synchronize()
    fwd_ms = e0.elapsed_time(e1) / 3
    out = {"seconds": round(res["seconds"], 4), "iterations": res["iterations"], "fallback": res["fallback"],
           "fallback_iterations": res["fallback_iterations"], "rel_residual": res["rel_residual"],
           "converged": res["converged"], "speedup_vs_jacobi_pcg": round(pcg_seconds / res["seconds"], 3),
           "structure": "FCG(1) with a V-cycle of %d damped-Jacobi levels whose coarsest (%d^3) solve is the U-Net "
                        "16/32/64 trained at %d^3" % (levels, nn_, args.train_n),
           "path": "C ABI ngb_learned_solve" if levels > 0 else "Python orchestration of the library kernels",
           "unet_forward_ms": round(fwd_ms, 3),
           "unet_forward_tflops": round(net.flops_forward(nn_) / fwd_ms / 1e9, 1), "training": train}
    if plain is not None:
        out["without_network"] = {"seconds": round(plain["seconds"], 4), "iterations": plain["iterations"],
                                  "fallback": plain["fallback"], "converged": plain["converged"],
                                  "speedup_vs_jacobi_pcg": round(pcg_seconds / plain["seconds"], 3)}
        out["network_gain"] = round(plain["seconds"] / res["seconds"], 3)
    return out, x2


def poisson_cpu_baseline(n=128):
    """The oracle's Jacobi-PCG (FP32 fields, FP64 dots, true residual every
    50 iterations) to 1e-8 at n^3 on one host core (the reference's CPU
    backend runs its grid loops serially)."""
    from oracle import cpu_baselines
    import oracle
    r = cpu_baselines.poisson_pcg(oracle.lib(), n)
    return {"value": r["seconds"], "unit": "s", "cores": 1, "kind": "port",
            "sample": "Jacobi-PCG to 1e-8 at %d^3 (%d iterations), the oracle's CG restatement" % (n, r["iterations"])}


def poisson_section(args, n=512):
    """Poisson -lap(u) = f at n^3 to 1e-8: Jacobi-PCG and the learned FCG, both on the device."""
    import torch
    dev = torch.device("cuda", 0)
    d, b = poisson_problem(n, dev)
    pcg, ws = jacobi_pcg_run(d, b, n, dev, reps=1)
    learned, _ = learned_fcg_run(args, n, dev, b, ws, pcg["seconds"])
    del ws, b
    torch.cuda.empty_cache()
    out = {"metric": "Poisson seconds to 1e-8 (512^3, zero Dirichlet, 8 seeded Gaussians)", "n": n,
           "jacobi_pcg": pcg, "learned_fcg": learned,
           "speedup_learned_vs_jacobi_pcg": learned["speedup_vs_jacobi_pcg"]}
    if not args.no_cpu:
        out["cpu_baseline"] = poisson_cpu_baseline()
    return out


def run_poisson(args):
    """Standalone Jacobi-PCG line (config 3) at --n."""
    import torch
    import neon_gb300 as ngb
    dev = torch.device("cuda", 0)
    ngb.lib()
    n = args.n
    d, b = poisson_problem(n, dev)
    pcg, _ = jacobi_pcg_run(d, b, n, dev, reps=args.steps)
    line = {"metric": "Poisson seconds to 1e-8 (Jacobi-PCG)", "value": pcg["seconds"], "unit": "s",
            "n_gpus": 1, "steps": pcg["solves"], "warmup": 0, "higher_is_better": False, "dtype": "f32",
            "data": "synthetic (8 seeded Gaussians, sigma 8)",
            "config": {"workload": "Poisson 7-point, zero Dirichlet, %d^3, FP32 fields / FP64 reductions" % n},
            "jacobi_pcg": pcg, "roofline": pcg["roofline"]}
    print(json.dumps(line), flush=True)


def run_learned(args):
    """Standalone learned-preconditioner line (config 4) at --n; `value` is the FCG solve time."""
    import torch
    import neon_gb300 as ngb
    dev = torch.device("cuda", 0)
    ngb.lib()
    n = args.n
    d, b = poisson_problem(n, dev)
    pcg, ws = jacobi_pcg_run(d, b, n, dev, reps=1)
    learned, x2 = learned_fcg_run(args, n, dev, b, ws, pcg["seconds"])
    line = {"metric": "Poisson seconds to 1e-8: learned FCG vs Jacobi-PCG", "value": learned["seconds"], "unit": "s",
            "n_gpus": 1, "steps": 1, "warmup": 1, "higher_is_better": False, "dtype": "bf16",
            "data": "synthetic (8 seeded Gaussians, sigma 8; training on seeded k^-2 fields)",
            "config": {"workload": "Poisson 7-point, zero Dirichlet, %d^3" % n}, "jacobi_pcg": pcg,
            "learned_fcg": learned}
    print(json.dumps(line), flush=True)


def sphere_section(args):
    """Config 2 on bGrid (FP16 storage, the config's own): MLUPS over active cells and roofline."""
    import copy
    a2 = copy.copy(args)
    a2.storage, a2.lattice, a2.steps, a2.warmup, a2.sim_steps, a2.scale = "f16off", "d3q19", 200, 10, 0, 1
    return run_sphere(a2, emit=False)


def unet_section(args):
    """The learned preconditioner's network at 512^3 (config 4's tensor-core
    path): TFLOP/s of one forward application against the measured BF16 peak."""
    import copy
    a2 = copy.copy(args)
    a2.n, a2.steps, a2.warmup = 512, 10, 3
    try:
        line = run_unet(a2, emit=False)
    except Exception as e:  # the headline line must not depend on this section
        return {"error": "%s: %s" % (type(e).__name__, e)}
    return {k: line[k] for k in ("metric", "value", "unit", "ms_per_step", "config", "roofline", "clocks", "gpu_launches")}


def bf16_peak():
    """Dense BF16 tensor peak (TFLOP/s, burst) measured on this machine, else the fallback."""
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["bf16_tflops"]), "measured"
    except Exception:
        return 1900.0, "fallback"


def run_unet(args, emit=True):
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
    # the device path of the solver's preconditioner (net.apply: |r|^2, scaled BF16
    # input, the 14 network launches, scaled output), no host round trip
    e = torch.empty_like(r)
    rr = torch.zeros(1, dtype=torch.float64, device=dev)
    scratch = torch.empty(ngb.lib().ngb_dot_scratch_doubles(r.numel()), dtype=torch.float64, device=dev)
    for _ in range(max(3, args.warmup)):
        net.apply(r, e, 1.0, rr, scratch)
    net.check()
    torch.cuda.synchronize()
    clk = ClockSampler(torch.cuda.current_device())
    clk.start()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(s)
    for _ in range(args.steps):
        net.apply(r, e, 1.0, rr, scratch)
    e1.record(s)
    e1.synchronize()
    clocks = clk.stop()
    net.check()
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
            "clocks": clocks, "gpu_launches": 17 * args.steps}
    if emit:
        print(json.dumps(line), flush=True)
    return line


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
    tdts = {k: v(torch) for k, v in TORCH_DTYPES.items()}
    u_ref, out = None, {}
    for st in ("f64", "f32", "f16sr", "f16off", "bf16off"):
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
    line = {"metric": "%s cavity velocity L2 error vs FP64" % args.lattice.upper(), "value": out["f16sr"]["velocity_l2_rel_err_vs_f64"],
            "unit": "relative L2", "n_gpus": 1, "steps": steps, "warmup": 0, "higher_is_better": False, "dtype": "f32",
            "data": "synthetic (lid-driven cavity set-up, equilibrium start)",
            "config": {"workload": "%s BGK lid-driven cavity, dense %d^3, %d steps" % (args.lattice.upper(), n, steps),
                       "lid_u": ulb, "Re": re_, "forms": out,
                       "value_form": "f16sr (FP16 offsets, stochastic rounding)",
                       "f16_speedup_vs_f32": round(out["f16sr"]["mlups"] / out["f32"]["mlups"], 3)}}
    print(json.dumps(line), flush=True)


def time_variant(ngb, torch, dev, n, lat, st, args):
    q = 19 if lat == "d3q19" else 27
    ulb = 0.1
    desc = ngb.lbm_dense_desc(n, n, n, q, st, ngb.cavity_omega(n, ulb, 100.0), ngb.lid_wall_terms(q, ulb))
    tdt = TORCH_DTYPES[st](torch)
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
