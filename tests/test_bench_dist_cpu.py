"""Host logic of bench.py's multi-GPU path (replicas, one process per GPU):
the timed region ends with the slowest rank and the value aggregates every
rank's lattice updates. Run here as two gloo ranks on the CPU."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    import torch
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    ms = 100.0 + 25.0 * rank  # rank 1 is the slower replica
    got = bench.max_over_ranks(ms, world, torch.device("cpu"))
    q.put((rank, got, bench.whole_job_mlups(world, 384 ** 3, 200, got)))
    dist.destroy_process_group()


def test_two_gloo_ranks_take_the_slowest_time_and_sum_the_work():
    mp = pytest.importorskip("torch.multiprocessing")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, ms, mlups in res:
        assert ms == 125.0
        assert abs(mlups - 2 * 384 ** 3 * 200 / (125.0 * 1e3)) < 1e-6


def test_single_rank_needs_no_process_group():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(3.5, 1, None) == 3.5
    assert bench.whole_job_mlups(1, 10 ** 6, 10, 2.0) == 5000.0


def test_clock_summary_reads_nvidia_smi_samples():
    """The clocks record of the bench line: median SM clock, maximum, and the
    throttle reasons that were active in any sample (nvidia-smi csv lines,
    timestamp first); with a window, only the samples taken inside it."""
    sys.path.insert(0, ROOT)
    import bench
    lines = ["2026/12/04 14:00:01.000, 0, 2070, 2070, 900.1, 0x0, Not Active, Not Active, Not Active, Not Active",
             "2026/12/04 14:00:01.050, 0, 1980, 2070, 1390.0, 0x4, Not Active, Not Active, Not Active, Active",
             "2026/12/04 14:00:01.100, 0, 2070, 2070, 1200.0, 0x0, Not Active, Not Active, Not Active, Not Active",
             "2026/12/04 14:00:05.000, 0, 1200, 2070, 300.0, 0x0, Not Active, Active, Not Active, Not Active",
             "garbage line"]
    got = bench.ClockSampler.summarise(lines)
    assert got == {"sm_mhz": 2070.0, "sm_max_mhz": 2070.0, "reasons": ["hw_thermal_slowdown", "sw_power_cap"],
                   "samples": 4}
    t0 = bench.ClockSampler.parse_time("2026/12/04 14:00:01.000")
    got = bench.ClockSampler.summarise(lines, window=(t0 + 0.04, t0 + 0.2))
    assert got == {"sm_mhz": 2070.0, "sm_max_mhz": 2070.0, "reasons": ["sw_power_cap"], "samples": 2}
    assert bench.ClockSampler.summarise([])["sm_mhz"] is None
