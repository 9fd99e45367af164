"""bench.py's multi-GPU reporting, on CPU: replicas of the single-scene step,
one per rank, report the slowest rank's time and the whole job's units over
it (no data-path collective). Two gloo ranks on 127.0.0.1."""
import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def _rank(rank, world, port, times, out):
    sys.path.insert(0, str(ROOT))
    import torch.distributed as dist

    import bench

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    t = bench.max_over_ranks(dist, times[rank], "cpu")
    dist.barrier()
    dist.destroy_process_group()
    out.put((rank, t, bench.job_rate(1000, world, t)))


def test_two_ranks_report_the_slowest_time_and_the_job_rate():
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    out = ctx.Queue()
    port = 29500 + os.getpid() % 1000
    times = [0.25, 0.5]
    procs = [ctx.Process(target=_rank, args=(r, 2, port, times, out)) for r in range(2)]
    for p in procs:
        p.start()
    got = sorted(out.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [g[1] for g in got] == [0.5, 0.5]      # every rank sees the max
    assert [g[2] for g in got] == [4000.0, 4000.0]  # 2 ranks x 1000 units / 0.5 s


def test_single_process_passes_values_through():
    sys.path.insert(0, str(ROOT))
    import bench

    assert bench.max_over_ranks(None, 1.5, "cpu") == 1.5
    assert bench.job_rate(10, 1, 2.0) == 5.0


def test_clock_summary_keeps_the_timed_region_and_names_throttle_reasons():
    """The clock record the JSON line carries: median SM clock and maximum over
    the samples inside the timed region, and the throttle reasons seen there."""
    import datetime

    sys.path.insert(0, str(ROOT))
    import bench

    t0 = datetime.datetime(2026, 1, 2, 3, 4, 5)
    rows = []
    for i, (mhz, reasons) in enumerate([(1500, "Not Active,Not Active,Not Active,Not Active"),
                                        (2070, "Not Active,Not Active,Not Active,Active"),
                                        (2070, "Not Active,Not Active,Not Active,Not Active"),
                                        (2055, "Active,Not Active,Not Active,Not Active"),
                                        (900, "Not Active,Not Active,Not Active,Not Active")]):
        ts = (t0 + datetime.timedelta(milliseconds=100 * i)).strftime("%Y/%m/%d %H:%M:%S.%f")[:-3]
        rows.append(f"{ts}, 0, {mhz}, 2070, 900.0, 0x0, {reasons}")
    s = bench.ClockSampler(0)
    s.out = "\n".join(rows)
    base = t0.timestamp()
    s.mark(base + 0.1, base + 0.3)  # samples 1..3
    c = s.summary()
    assert c["samples"] == 3 and c["sm_mhz"] == 2070 and c["sm_max_mhz"] == 2070
    assert c["reasons"] == ["hw_slowdown", "sw_power_cap"]
    s.mark(base + 0.41, base + 0.42)  # shorter than the period: the nearest sample
    c = s.summary()
    assert c["samples"] == 1 and c["sm_mhz"] == 900 and c["reasons"] == []
    s.out = ""
    assert bench.ClockSampler(0).summary()["reasons"] == ["unavailable"]


def test_committed_profiles_feed_the_bench_line():
    """The roofline's traffic comes from the committed ncu figures, and every
    profile summary states the ncu command that made it (clocks left alone)."""
    sys.path.insert(0, str(ROOT))
    import bench

    t = bench.ncu_traffic("sweep", "crumpled16x250")
    assert isinstance(t, int) and t > 977_114_680  # at least the algorithmic bytes
    summaries = sorted((ROOT / "profiles").glob("*.md"))
    assert len(summaries) >= 3
    for p in summaries:
        text = p.read_text()
        assert "ncu " in text and "--clock-control none" in text, p.name
