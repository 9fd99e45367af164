#!/usr/bin/env python3
"""Benchmark of the GB300 STQ broad phase: boxes/s and pairs/s.

Default workload: the large single scene, 16 interpenetrating crumpled sheets
of 250 x 250 vertices (5,968,048 vertex/edge/face boxes), synthetic and
seeded (the reference's external mesh benchmarks are not distributed).

One step = device box build from fp64 trajectories -> sweep-axis choice ->
radix sort -> STQ sweep -> all pairs in HBM. `value` times the step with its
inputs resident in HBM (CUDA events on the library's stream, L2 flushed
between steps); `e2e` times the same step through the C ABI on host buffers
(stq_broadphase_host: H2D mesh copy, pipeline, D2H pair copy).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl stq|reference]

--impl reference times the reference's CPU sort + sweep on the host cores: the
oracle restatement of src/cpu (checked bit for bit against the reference's own
src/cpu compiled unchanged, where its source tree is present), each step a
bounded sample of the same scene (all boxes sorted, every k-th start box swept).
Under torchrun (N > 1) every rank runs an independent replica (the path does
not shard on one scene); rank 0 prints the JSON line.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

WORKLOADS = {
    "crumpled16x250": dict(kind="crumpled", sheets=16, g=250, amp=0.05, sigma=0.005, seed=1),
    "crumpled16x290": dict(kind="crumpled", sheets=16, g=290, amp=0.05, sigma=0.005, seed=1),
    "cloth200": dict(kind="cloth", g=200, z_offset=0.01, sigma=0.003, seed=0),
}
L2_FLUSH_BYTES = 512 << 20  # > 129 MB L2
FALLBACK_HBM_GBS = 6800.0


def make_mesh(stq, w):
    if w["kind"] == "crumpled":
        return stq.crumpled_sheets(w["sheets"], w["g"], w["amp"], w["sigma"], w["seed"])
    return stq.cloth_pair(g=w["g"], z_offset=w["z_offset"], sigma=w["sigma"], seed=w["seed"])


def measured_peak():
    p = ROOT / "MEASURED_PEAKS.json"
    try:
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return FALLBACK_HBM_GBS, "fallback"


def ncu_traffic(kernel: str, workload: str):
    """DRAM bytes per launch of `kernel` from the committed ncu summary, if any."""
    p = ROOT / "profiles" / "traffic.txt"
    if not p.exists():
        return None
    for line in p.read_text().splitlines():
        parts = line.split()
        if len(parts) >= 3 and parts[0] == kernel and parts[1] == workload:
            try:
                return int(parts[2])
            except ValueError:
                return None
    return None


class ClockSampler:
    """nvidia-smi clocks and throttle reasons, sampled every 20 ms from before the
    warm-up (its start-up stays out of the timed region); the summary keeps the
    samples whose timestamps fall inside the marked timed region."""

    FIELDS = ("timestamp,index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.out = ""
        self.window = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "20"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            time.sleep(0.5)  # let it initialise before anything is timed
        except (FileNotFoundError, OSError):
            self.proc = None
        return self

    def mark(self, t0, t1):
        self.window = (t0, t1)

    def stop(self):
        if self.proc:
            time.sleep(0.05)
            self.proc.terminate()
            try:
                self.out, _ = self.proc.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                self.out, _ = self.proc.communicate()

    def summary(self):
        import datetime

        rows = []
        for line in (self.out or "").splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) >= 10:
                try:
                    ts = datetime.datetime.strptime(f[0], "%Y/%m/%d %H:%M:%S.%f").timestamp()
                    rows.append((ts, float(f[2]), float(f[3]), f[6:10]))
                except ValueError:
                    pass
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"], "samples": 0}
        inside = rows
        if self.window:
            t0, t1 = self.window
            inside = [r for r in rows if t0 - 0.02 <= r[0] <= t1 + 0.02]
            if not inside:  # region shorter than the sampling period: the nearest sample
                inside = [min(rows, key=lambda r: abs(r[0] - 0.5 * (t0 + t1)))]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for _, _, _, r in inside for i in range(4) if r[i].lower() == "active"})
        return {"sm_mhz": statistics.median(r[1] for r in inside), "sm_max_mhz": max(r[2] for r in inside),
                "reasons": reasons, "samples": len(inside)}


def max_over_ranks(dist, value: float, device) -> float:
    """The largest of the ranks' values (a timing): every rank gets it. With one
    process (dist None) the value itself."""
    if dist is None:
        return value
    import torch

    t = torch.tensor([value], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_rate(units_per_rank: int, world: int, seconds_max: float) -> float:
    """Whole-job throughput of replicas: every rank processed units_per_rank in
    its own time; the job took the slowest rank's time."""
    return world * units_per_rank / seconds_max


def pick_stride(orc, boxes, step_s: float, threads: int = 0) -> int:
    """Start-box stride of a CPU sample whose sweep takes about step_s seconds
    (a power of two, from a probe that sweeps every 256th start box)."""
    _, t_probe, _ = orc.time_sample(boxes, 256, threads)
    full = max(t_probe * 256, 1e-6)
    stride = 1
    while full / stride > step_s and stride < (1 << 20):
        stride *= 2
    return stride


def cpu_sample_steps(orc, boxes, stride: int, steps: int, warmup: int = 0, threads: int = 0) -> dict:
    """Times the reference's CPU sort + sweep (the oracle restatement of
    src/cpu/sweep.cpp) on a bounded sample of the scene: each step sorts all
    boxes (from an unsorted copy) and sweeps every stride-th start box of the
    sorted order in full. Throughput = start boxes swept / measured step time
    (no extrapolation to the whole scene)."""
    n = len(boxes)
    per_step = (n + stride - 1) // stride
    times, sorts = [], []
    for i in range(warmup + steps):
        t_sort, t_sweep, _ = orc.time_sample(boxes, stride, threads)
        if i >= warmup:
            times.append(t_sort + t_sweep)
            sorts.append(t_sort)
    th = threads if threads > 0 else orc.default_threads()
    total = sum(times)
    return dict(value=per_step * steps / total, unit="boxes/s", cores=th, kind="port",
                sample=(f"each step: sort of all {n} boxes ({1e3 * sum(sorts) / steps:.0f} ms) + full sweep of every "
                        f"{stride}-th start box of the sorted order ({per_step} start boxes), {th} threads; "
                        f"boxes/s = start boxes swept / measured step time"),
                ms_per_step=1e3 * total / steps, stride=stride, start_boxes_per_step=per_step)


def workload_config(name: str, nV: int, nE: int, nF: int) -> dict:
    """The `config` of both bench arms (identical by construction)."""
    return {"workload": name, "boxes": nV + nE + nF, "vertices": nV, "edges": nE, "faces": nF,
            "l2": "inputs and sorted scene exceed the 129 MB L2; GPU steps also flush L2 (512 MB write)"}


def bench_batched(stq, torch, dev, stream, local, steps, warmup, flush, tune=True, options="", loop=True):
    """256 cloth-pair scenes (box counts log-uniform in [1e3, 2e5]): the fused,
    graph-captured batch call against the per-scene plain launch loop
    (build + prepare + sweep with its host synchronisations, scene by scene),
    both with the settings the autotuner picks on this batch (untimed)."""
    meshes = stq.batch_scenes(256, 1e3, 2e5, seed=2)
    V0, V1, E, F, vo, eo, fo = stq.concat_meshes(meshes)
    d = [torch.from_numpy(x).to(dev) for x in (V0, V1, E, F)]
    N = int(sum(m.num_boxes for m in meshes))
    ctx = stq.Context(local, stream.cuda_stream)
    cap = 64 * N
    pairs = torch.empty((cap, 2), dtype=torch.int32, device=dev)
    r, per = ctx.batch_broadphase(d[0], d[1], vo, d[2], eo, d[3], fo, pairs, cap)
    total = r.total
    cap = int(total * 1.05) + 1024
    pairs = torch.empty((cap, 2), dtype=torch.int32, device=dev)
    tuned, tune_ms = context_options(stq, ctx, options) or "library defaults", None
    if tune:
        bboxes = torch.empty((N, 11), dtype=torch.int32, device=dev)
        bo = ctx.batch_build_boxes(d[0], d[1], vo, d[2], eo, d[3], fo, bboxes)
        tune_ms, tuned = ctx.autotune(bboxes, bo, pairs, cap)
        del bboxes

    def timed(fn):
        for _ in range(warmup):
            fn()
        ms = 0.0
        for i in range(steps):
            with torch.cuda.stream(stream):
                flush.fill_(i)
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            fn()
            b.record(stream)
            torch.cuda.synchronize(dev)
            ms += a.elapsed_time(b)
        return ms / steps

    launches0 = ctx.launches
    t_batch = timed(lambda: ctx.batch_broadphase(d[0], d[1], vo, d[2], eo, d[3], fo, pairs, cap))
    boxes = torch.empty((max(m.num_boxes for m in meshes), 11), dtype=torch.int32, device=dev)

    def plain_loop():
        found = 0
        for k, m in enumerate(meshes):
            v = slice(int(vo[k]), int(vo[k + 1]))
            ctx.build_boxes(d[0][v], d[1][v], d[2][int(eo[k]):int(eo[k + 1])],
                            d[3][int(fo[k]):int(fo[k + 1])], boxes)
            ctx.prepare(boxes, m.num_boxes, stq.AXIS_AUTO)
            found += ctx.sweep_prepared(pairs, cap).count
        assert found == total, (found, total)

    t_plain = timed(plain_loop) if loop else float("nan")
    ctx.close()
    return {"workload": "256 cloth-pair scenes, boxes log-uniform in [1e3, 2e5]", "boxes": N,
            "pairs": int(total), "batched_ms": t_batch, "plain_loop_ms": t_plain,
            "batched_boxes_per_s": N / (t_batch / 1e3), "plain_loop_boxes_per_s": N / (t_plain / 1e3),
            "batched_over_plain": t_plain / t_batch, "graph": True, "tuned": tuned,
            "tuned_prepare_sweep_ms": tune_ms}


def context_options(stq, ctx, spec: str) -> dict:
    """Applies `name=value,...` context options (cell_scale, shape, per_lane,
    lanes, queue, block, radix_bits); returns them as a dict."""
    names = {"cell_scale": stq.OPT_CELL_SCALE, "shape": stq.OPT_SWEEP_SHAPE, "per_lane": stq.OPT_PER_LANE,
             "lanes": stq.OPT_LANES, "queue": stq.OPT_QUEUE, "block": stq.OPT_BLOCK,
             "radix_bits": stq.OPT_RADIX_BITS, "run_cap": stq.OPT_RUN_CAP}
    out = {}
    for item in filter(None, spec.split(",")):
        k, v = item.split("=")
        ctx.set_option(names[k], int(v))
        out[k] = int(v)
    return out


def bench_skewed(stq, torch, dev, stream, local, steps, warmup, flush, tune=True, options=""):
    """64 scenes of 500,000 random boxes (95% small, lognormal extents around
    0.002; 5% slivers stretched 200x along a random axis), sweep axis x in half
    of the scenes and the largest-variance axis in the other half: the batched
    prepare + sweep against a per-scene loop of the same calls."""
    import numpy as np

    n_s, per = 64, 500_000
    scenes = [stq.random_boxes(per, sliver_frac=0.05, seed=1000 + k) for k in range(n_s)]
    allb = np.concatenate(scenes)
    allb["id"] = np.arange(len(allb), dtype=np.int32)
    box_off = np.arange(n_s + 1, dtype=np.int64) * per
    axes = [0 if k % 2 == 0 else stq.AXIS_AUTO for k in range(n_s)]
    boxes = torch.from_numpy(allb.view(np.int32).reshape(-1, 11).copy()).to(dev)
    ctx = stq.Context(local, stream.cuda_stream)
    cap = 8 * len(allb)
    pairs = torch.empty((cap, 2), dtype=torch.int32, device=dev)
    ctx.batch_prepare(boxes, box_off, axes=axes)
    total = ctx.sweep_prepared(pairs, cap).total
    cap = int(total * 1.05) + 1024
    pairs = torch.empty((cap, 2), dtype=torch.int32, device=dev)
    # settings tuned on the same batch (untimed; the tuner prepares with the
    # largest-variance axis in every scene, the timed runs use the axes above)
    tuned = context_options(stq, ctx, options) or "library defaults"
    if tune:
        tune_ms, tuned = ctx.autotune(boxes, box_off, pairs, cap)

    def timed(fn):
        for _ in range(warmup):
            fn()
        ms = 0.0
        for i in range(steps):
            with torch.cuda.stream(stream):
                flush.fill_(i)
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            fn()
            b.record(stream)
            torch.cuda.synchronize(dev)
            ms += a.elapsed_time(b)
        return ms / steps

    def batched():
        ctx.batch_prepare(boxes, box_off, axes=axes)
        r = ctx.sweep_prepared(pairs, cap)
        assert r.count == total

    def plain_loop():
        found = 0
        for k in range(n_s):
            ctx.prepare(boxes[k * per:(k + 1) * per], per, axes[k])
            found += ctx.sweep_prepared(pairs, cap).count
        assert found == total, (found, total)

    t_batch = timed(batched)
    t_plain = timed(plain_loop)
    ctx.close()
    n = len(allb)
    return {"workload": "64 x 500k random boxes, 5% slivers (200x), axis x / max-variance alternating",
            "boxes": n, "pairs": int(total), "batched_ms": t_batch, "plain_loop_ms": t_plain, "tuned": tuned,
            "batched_boxes_per_s": n / (t_batch / 1e3), "batched_pairs_per_s": total / (t_batch / 1e3),
            "batched_over_plain": t_plain / t_batch}


def bench_scene(stq, torch, dev, stream, local, steps, warmup, flush, workload):
    """Device-resident step (build, prepare, sweep) on another single scene."""
    mesh = make_mesh(stq, WORKLOADS[workload])
    n = mesh.num_boxes
    V0, V1, E, F = (torch.from_numpy(x).to(dev) for x in (mesh.V0, mesh.V1, mesh.E, mesh.F))
    boxes = torch.empty((n, 11), dtype=torch.int32, device=dev)
    ctx = stq.Context(local, stream.cuda_stream)
    ctx.build_boxes(V0, V1, E, F, boxes)
    ctx.prepare(boxes, n, stq.AXIS_AUTO)
    cap = 24 * n
    pairs = torch.empty((cap, 2), dtype=torch.int32, device=dev)
    total = ctx.sweep_prepared(pairs, cap).total
    cap = int(total * 1.05) + 1024
    pairs = torch.empty((cap, 2), dtype=torch.int32, device=dev)
    _, tuned = ctx.autotune(boxes, [0, n], pairs, cap)

    def step():
        ctx.build_boxes(V0, V1, E, F, boxes)
        ctx.prepare(boxes, n, stq.AXIS_AUTO)
        assert ctx.sweep_prepared(pairs, cap).count == total

    for _ in range(warmup):
        step()
    ms = 0.0
    for i in range(steps):
        with torch.cuda.stream(stream):
            flush.fill_(i)
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        step()
        b.record(stream)
        torch.cuda.synchronize(dev)
        ms += a.elapsed_time(b)
    ms /= steps
    ctx.close()
    return {"workload": workload, "boxes": n, "pairs": int(total), "ms_per_step": ms, "tuned": tuned,
            "boxes_per_s": n / (ms / 1e3), "pairs_per_s": total / (ms / 1e3),
            "pipeline_alg_frac": (60 * n + 8 * total) / (ms / 1e3) / 1e9 / measured_peak()[0]}


def bench_serving(stq, local, n_requests, rates, seed=4):
    """Poisson arrivals of time-stepped cloth-pair requests (boxes log-uniform
    in [1e4, 2e6], 1-20 steps, step noise 0.003, HBM budget 160 GB) at each
    rate: the continuous-batching server against the same server run one
    request at a time (serial). Latency = completion - arrival, split into the
    wait before the request's first tick (queue and admission; its upload
    overlaps the tick in flight) and the time from that tick's launch to
    completion (its steps, one per tick)."""
    import numpy as np

    rng = np.random.default_rng(seed)
    reqs = []
    for k in range(n_requests):
        n = float(np.exp(rng.uniform(np.log(1e4), np.log(2e6))))
        m = stq.cloth_pair(g=stq.cloth_pair_grid_for(int(n)), z_offset=float(rng.uniform(0.002, 0.05)),
                           sigma=float(rng.uniform(0.001, 0.01)), seed=stq.splitmix64(seed * 7919 + k))
        reqs.append((m, int(rng.integers(1, 21)), k))
    gaps = rng.exponential(1.0, n_requests)  # unit-rate gaps, scaled per rate
    box_steps = sum(m.num_boxes * s for m, s, _ in reqs)
    table = []
    for rate in rates:
        arrivals = np.cumsum(gaps / rate)
        row = {"rate_per_s": rate}
        for label, max_scenes in (("batched", 256), ("serial", 1)):
            sv = stq.Server(local, None, budget_bytes=160 << 30, max_boxes=1 << 25, max_scenes=max_scenes)
            t0 = time.perf_counter()
            i, arrive, done, tick_t = 0, {}, {}, []
            while len(done) < n_requests:
                now = time.perf_counter() - t0
                while i < n_requests and arrivals[i] <= now:
                    m, steps, sd = reqs[i]
                    arrive[sv.submit(m, steps, 0.003, sd)] = arrivals[i]
                    i += 1
                finished = sv.tick()
                t_tick = time.perf_counter() - t0
                for rid in finished:
                    done[rid] = t_tick
                st = sv.stats()
                while len(tick_t) < st["ticks"]:  # the tick just launched
                    tick_t.append(t_tick)
                if st["active"] == 0 and st["queued"] == 0 and i < n_requests:
                    time.sleep(max(0.0, min(0.002, arrivals[i] - (time.perf_counter() - t0))))
            elapsed = time.perf_counter() - t0
            lat, wait, serve, per_tick = [], [], [], []
            for r in done:
                first, last = sv.request_ticks(r)
                lat.append(done[r] - arrive[r])
                wait.append(max(0.0, tick_t[first] - arrive[r]))
                serve.append(done[r] - tick_t[first])
                per_tick.append((done[r] - tick_t[first]) / (last - first + 1))
            pairs = sum(int(sv.result(r)[0].sum()) for r in done)
            ms = lambda v, q: float(np.percentile(v, q) * 1e3)  # noqa: E731
            row[label] = {"p50_ms": ms(lat, 50), "p99_ms": ms(lat, 99),
                          "pairs_per_s": pairs / elapsed, "box_steps_per_s": box_steps / elapsed,
                          "seconds": elapsed, "ticks": sv.stats()["ticks"],
                          "wait_p50_ms": ms(wait, 50), "in_service_p50_ms": ms(serve, 50),
                          "tick_p50_ms": ms(per_tick, 50)}
            sv.close()
        table.append(row)
    return {"workload": f"{n_requests} Poisson requests per rate; cloth pairs, boxes log-uniform "
                        "in [1e4, 2e6], 1-20 steps, step noise 0.003; budget 160 GB",
            "latency_split": "wait = arrival to the launch of the request's first tick; in_service = "
                             "that launch to completion; tick = in_service / its ticks (one step each)",
            "rates": table}


def run_reference(args, w):
    """The reference's CPU path on the host cores (the oracle restatement of
    src/cpu: sort along x + sweep, app/main.cpp:138-156 scope), on the same
    scene as the GPU arm. A CPU-only process: it loads the oracle library only
    (which also holds the scene generators)."""
    import __graft_entry__ as entry

    orc = entry.load_oracle()
    orc.build()
    if w["kind"] == "crumpled":
        V0, V1, E, F = orc.crumpled_sheets(w["sheets"], w["g"], w["amp"], w["sigma"], w["seed"])
    else:
        V0, V1, E, F = orc.cloth_pair(w["g"], w["z_offset"], w["sigma"], w["seed"])
    boxes = orc.construct_boxes(V0, V1, E, F, orc.AABB_DTYPE)
    stride = pick_stride(orc, boxes, args.ref_step_s)
    cb = cpu_sample_steps(orc, boxes, stride, args.steps, args.warmup)
    value = cb["value"]
    line = {
        "metric": "boxes/s (STQ broad phase, one scene)", "value": value, "unit": "boxes/s",
        "impl": "reference", "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": cb["ms_per_step"], "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic (seeded crumpled-sheet trajectories)",
        "config": workload_config(args.workload, V0.shape[0], E.shape[0], F.shape[0]),
        "cpu_baseline": {k: cb[k] for k in ("value", "unit", "cores", "kind", "sample")},
        "e2e": {"value": value, "unit": "boxes/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="stq", choices=["stq", "reference"])
    ap.add_argument("--workload", default="crumpled16x250", choices=sorted(WORKLOADS))
    ap.add_argument("--cpu-step-s", type=float, default=3.0,
                    help="seconds of CPU sweep per sample step of the CPU baseline")
    ap.add_argument("--cpu-steps", type=int, default=3)
    ap.add_argument("--ref-step-s", type=float, default=3.0,
                    help="seconds of CPU sweep per step of the reference arm")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-parity", action="store_true",
                    help="skip the check of the main scene's pairs against the CPU oracle")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-batch", action="store_true")
    ap.add_argument("--no-serve", action="store_true")
    ap.add_argument("--no-extra", action="store_true",
                    help="skip the 8M-box scene and the skewed 64-scene batch")
    ap.add_argument("--no-tune", action="store_true",
                    help="skip the autotuner (use the library defaults), e.g. for profiling")
    ap.add_argument("--options", type=str, default="",
                    help="context options for the main scene, e.g. cell_scale=4,shape=2 (with --no-tune)")
    ap.add_argument("--only-skewed", action="store_true",
                    help="run the skewed 64-scene batch alone and print its figures (profiling runs)")
    ap.add_argument("--only-batched", action="store_true",
                    help="run the 256-scene batched call alone, without the per-scene loop (profiling runs)")
    ap.add_argument("--serve-requests", type=int, default=48)
    ap.add_argument("--serve-rates", type=str, default="50,200,500,1000,2000")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    w = WORKLOADS[args.workload]

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        if rank == 0:
            run_reference(args, w)
        return

    import numpy as np
    import torch

    import __graft_entry__ as entry

    pkg = entry.load_package()
    stq = pkg.stq
    torch.cuda.set_device(local)
    dev = torch.device(f"cuda:{local}")
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=dev)

    mesh = make_mesh(stq, w)
    nV, nE, nF = mesh.V0.shape[0], mesh.E.shape[0], mesh.F.shape[0]
    n = nV + nE + nF
    stream = torch.cuda.Stream(dev)
    V0 = torch.from_numpy(mesh.V0).to(dev)
    V1 = torch.from_numpy(mesh.V1).to(dev)
    E = torch.from_numpy(mesh.E).to(dev)
    F = torch.from_numpy(mesh.F).to(dev)
    boxes = torch.empty((n, 11), dtype=torch.int32, device=dev)
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.int32, device=dev)
    torch.cuda.synchronize(dev)
    if args.only_skewed:
        if rank == 0:
            print(json.dumps(bench_skewed(stq, torch, dev, stream, local, args.steps, args.warmup, flush,
                                          tune=not args.no_tune, options=args.options)), flush=True)
        return
    if args.only_batched:
        if rank == 0:
            print(json.dumps(bench_batched(stq, torch, dev, stream, local, args.steps, args.warmup, flush,
                                           tune=not args.no_tune, options=args.options, loop=False)),
                  flush=True)
        return

    ctx = stq.Context(local, stream.cuda_stream)
    # size the pair buffer from a first run
    cap = 24 * n
    pairs = torch.empty((cap, 2), dtype=torch.int32, device=dev)
    ctx.build_boxes(V0, V1, E, F, boxes)
    ctx.prepare(boxes, n, stq.AXIS_AUTO)
    r = ctx.sweep_prepared(pairs, cap)
    cap = int(r.total * 1.05) + 1024
    pairs = torch.empty((cap, 2), dtype=torch.int32, device=dev)
    # the project's autotuner picks cell scale, radix width, sweep shape,
    # lane-group width, queue depth and block size for this workload (not
    # timed); --no-tune with --options name=value,... sets them by hand instead
    # (profiling runs, which must not launch the tuner's trials)
    tuned = context_options(stq, ctx, args.options) or "library defaults"
    if not args.no_tune:
        tune_ms, tuned = ctx.autotune(boxes, [0, n], pairs, cap)

    def step():
        ctx.build_boxes(V0, V1, E, F, boxes)
        ctx.prepare(boxes, n, stq.AXIS_AUTO)
        res = ctx.sweep_prepared(pairs, cap)
        assert res.status == stq.STQ_OK, res
        return res.count

    clk = ClockSampler(local).start()
    for _ in range(args.warmup):
        flush.fill_(1)
        step()
    torch.cuda.synchronize(dev)
    ctx.enable_timing(True)
    launches0 = ctx.launches
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
           for _ in range(args.steps)]
    if dist:
        dist.barrier()
    torch.cuda.synchronize(dev)
    t_region = time.time()
    for i in range(args.steps):
        with torch.cuda.stream(stream):
            flush.fill_(i)  # evict the previous step's working set from L2
        evs[i][0].record(stream)
        npairs = step()
        evs[i][1].record(stream)
    torch.cuda.synchronize(dev)
    clk.mark(t_region, time.time())
    clk.stop()
    if dist:
        dist.barrier()
    step_ms = [a.elapsed_time(b) for a, b in evs]
    total_ms = max_over_ranks(dist, sum(step_ms), dev)
    launches = ctx.launches - launches0
    stages = ctx.stage_times()
    ctx.enable_timing(False)
    ms_per_step = total_ms / args.steps
    value = job_rate(n, world, ms_per_step / 1e3)

    # dominant kernel and its roofline (algorithmic bytes per launch / launch time)
    dom = max(stages.items(), key=lambda kv: kv[1][0])
    dom_name, (dom_ms, dom_calls) = dom
    alg_bytes = {
        "sweep": 40 * n + 8 * npairs,             # sorted records read once, pairs written once
        "sort": 16 * n,                           # key+index read once and written once
        "build": 24 * 2 * nV + 8 * nE + 12 * nF + 44 * n,
        "gather": 44 * n + 40 * n,
    }.get(dom_name)
    peak, peak_kind = measured_peak()
    per_launch_ms = dom_ms / max(dom_calls, 1)
    achieved = alg_bytes / (per_launch_ms / 1e3) / 1e9 if alg_bytes else None
    traffic = ncu_traffic(dom_name, args.workload)

    line = {
        "metric": "boxes/s (STQ broad phase, one scene)", "value": value, "unit": "boxes/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_per_step,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded crumpled-sheet trajectories; the reference's mesh benchmarks are not distributed)",
        "config": workload_config(args.workload, nV, nE, nF),
        "pairs": npairs, "axis": "max-variance", "parallelism": "replicas" if world > 1 else "single GPU",
        "tuned": tuned,
        "pairs_per_s": world * npairs / (ms_per_step / 1e3),
        "stage_ms_per_step": {k: v[0] / args.steps for k, v in stages.items() if v[1]},
        "gpu_launches": launches,
        "roofline": {"bound": "hbm", "kernel": dom_name, "achieved": achieved, "peak": peak,
                     "unit": "GB/s", "frac": (achieved / peak) if achieved else None,
                     "traffic": traffic, "peak_source": f"{peak_kind} hbm_gbs",
                     "alg_bytes_per_launch": alg_bytes, "launch_ms": per_launch_ms},
        "pipeline_alg_frac": (60 * n + 8 * npairs) / (ms_per_step / 1e3) / 1e9 / peak,
        "clocks": clk.summary(),
    }

    if not args.no_e2e:
        hmesh_t = [torch.from_numpy(a).pin_memory() for a in (mesh.V0, mesh.V1, mesh.E, mesh.F)]
        hmesh = stq.Mesh(*(t.numpy() for t in hmesh_t))
        hpairs_t = torch.empty((cap, 2), dtype=torch.int32).pin_memory()
        hpairs = hpairs_t.numpy()
        # the same (tuned) context, now through the host-memory call
        for _ in range(args.warmup):
            ctx.broadphase_host(hmesh, hpairs, stq.AXIS_AUTO)
        ts = []
        for _ in range(args.steps):
            torch.cuda.synchronize(dev)
            t0 = time.perf_counter()
            er = ctx.broadphase_host(hmesh, hpairs, stq.AXIS_AUTO)
            ts.append(time.perf_counter() - t0)
        assert er.status == stq.STQ_OK and er.count == npairs, er
        # for comparison: one copy of the whole pair list after the sweep
        ctx.set_option(stq.OPT_HOST_OVERLAP, 2)
        ctx.broadphase_host(hmesh, hpairs, stq.AXIS_AUTO)
        ts_staged = []
        for _ in range(args.steps):
            torch.cuda.synchronize(dev)
            t0 = time.perf_counter()
            ctx.broadphase_host(hmesh, hpairs, stq.AXIS_AUTO)
            ts_staged.append(time.perf_counter() - t0)
        ctx.set_option(stq.OPT_HOST_OVERLAP, 0)

        def link_ms(copy):  # the host link alone: the step's bytes, no compute
            lt = []
            for _ in range(args.warmup + args.steps):
                torch.cuda.synchronize(dev)
                t0 = time.perf_counter()
                with torch.cuda.stream(stream):
                    copy()
                stream.synchronize()
                lt.append(time.perf_counter() - t0)
            return 1e3 * float(np.median(lt[args.warmup:]))

        h2d_ms = link_ms(lambda: [d.copy_(h, non_blocking=True) for d, h in zip((V0, V1, E, F), hmesh_t)])
        d2h_ms = link_ms(lambda: hpairs_t[:npairs].copy_(pairs[:npairs], non_blocking=True))
        e2e_s = max_over_ranks(dist, sum(ts) / len(ts), dev)
        ts_sorted = sorted(ts)
        line["e2e"] = {"value": job_rate(n, world, e2e_s), "unit": "boxes/s",
                       "h2d_bytes_per_step": 48 * nV + 8 * nE + 12 * nF,
                       "d2h_bytes_per_step": 8 * er.count, "ms_per_step": e2e_s * 1e3,
                       "call": "stq_broadphase_host",
                       "pairs_out": "sweep windows, each copied while later ones are swept",
                       "ms_median": 1e3 * ts_sorted[len(ts) // 2], "ms_min": 1e3 * ts_sorted[0],
                       "ms_steps": [round(1e3 * t, 3) for t in ts],
                       "one_copy_after_sweep_ms_per_step": 1e3 * sum(ts_staged) / len(ts_staged),
                       "link_alone_ms": {"h2d_mesh": h2d_ms, "d2h_pairs": d2h_ms,
                                         "d2h_gbs": 8 * npairs / d2h_ms / 1e6}}

    if not args.no_batch:
        line["batched"] = bench_batched(stq, torch, dev, stream, local, args.steps, args.warmup, flush)

    if not args.no_extra:
        if args.workload != "crumpled16x290":
            line["scene_8m"] = bench_scene(stq, torch, dev, stream, local, args.steps, args.warmup, flush,
                                           "crumpled16x290")
        line["skewed"] = bench_skewed(stq, torch, dev, stream, local, args.steps, args.warmup, flush)

    if not args.no_serve and rank == 0:
        line["serve"] = bench_serving(stq, local, args.serve_requests,
                                      [float(x) for x in args.serve_rates.split(",")])

    if rank == 0 and world == 1 and not (args.no_cpu_baseline and args.no_parity):
        orc = entry.load_oracle()
        hb = orc.construct_boxes(mesh.V0, mesh.V1, mesh.E, mesh.F, stq.AABB_DTYPE)
        if not args.no_parity:
            # the timed step's output against the oracle (after all timing):
            # box bytes, and the whole sorted pair list
            step()
            ctx.sort_pairs(pairs, npairs)
            got = pairs[:npairs].cpu().numpy()
            t0 = time.perf_counter()
            want = orc.broadphase(hb)
            oracle_s = time.perf_counter() - t0
            line["parity"] = {"checked": "box bytes and the sorted pair list of one step against the CPU oracle",
                              "boxes_equal": boxes.cpu().numpy().tobytes() == hb.tobytes(),
                              "pairs_equal": bool(got.shape == want.shape and np.array_equal(got, want)),
                              "pairs": int(want.shape[0]), "oracle_s": oracle_s}
            del got, want
        if not args.no_cpu_baseline:
            cb = cpu_sample_steps(orc, hb, pick_stride(orc, hb, args.cpu_step_s), args.cpu_steps, 1)
            line["cpu_baseline"] = {k: cb[k] for k in ("value", "unit", "cores", "kind", "sample")}
    ctx.close()
    if dist:
        dist.destroy_process_group()
    if rank == 0:
        print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
