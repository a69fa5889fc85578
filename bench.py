"""Benchmark: ms/tick of a 1M-node 3D force layout (link + many-body + centre) on one GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--nodes N]

Workload (the metric's headline configuration): 3D, 1,000,000 nodes at the reference's
phyllotaxis start, 1,499,999 links (random tree + 500,000 distinct random pairs, the reference
benchmark's generator, LCG seed 42), forceLink(distance 30, strength 1/min(degree)) +
forceManyBody(-30, theta 0.9) + forceCenter(), alpha 1, alphaDecay 1 - 0.001^(1/300),
velocityDecay 0.4. A step is one tick. Synthetic, seeded data (no dataset is involved).

  value     ms per tick, device-timed with CUDA events on the engine's stream, state resident
  e2e       ms per tick through the C ABI with host buffers: each step uploads every position
            from pinned host memory (fl_update_positions_packed: x, y, z per node), queues the
            tick (fl_enqueue) and reads positions and velocities back into pinned host memory
            (fl_sync_packed: x, y, z each). The host link (~190-205 GB/s each way, measured)
            carries 3/4 of the bytes of the float4 calls, fl_update_positions and fl_sync
  e2e_float4  the same through those float4 calls (the reference's vec4 layout)
  roofline  the dominant kernel (the tree walk) against measured HBM bandwidth, and its FP32
            pipe view from interaction counts
  cpu_baseline  the oracle (FP64 C restatement of the reference's CPU simulation, one core) on
            a bounded sample: ticks of the same 1M-node layout
  batched, served  compact runs of the batched engine (256 graphs x 100 ticks against the plain
            engine one graph at a time) and of the layout server (40 jobs arriving at 2,000/s,
            continuous batching, against serial plain solves): layouts/s, p50/p99 latency

Timing: a pre-roll runs the warm-up and timed ticks twice from the start state and puts that
state back (fl_upload_all), so that every block of ticks has been captured as a CUDA graph;
then W warm-up ticks, then ticks W+1..W+K timed. The clock samples cover the pre-roll, the
warm-up and the timed region.

With --impl reference, the same workload and tick window run on the CPU implementation (the
oracle; the reference's own CPU code is JavaScript, and there is no Node.js on this machine).
Multi-GPU: the single simulation does not shard; N ranks run N independent replicas, and
`value` stays the ms per tick of one simulation (the slowest replica).
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

# before any CUDA context exists (torch's or the engine's): streams side by side (forcegpu)
os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "d3-force-3d-webgpu_gb300"))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

METRIC = "ms/tick at 1M nodes (3D link+charge+center)"
UNIT = "ms/tick"

# algorithmic bytes per node of one tick (link + charge + center, 1.5 links per node): state
# read + write 64, pins 4, charge 140, link 4 + 32 per link (48 at 1.5 links/node), centre 4
BYTES_PER_NODE_TICK = 64 + 4 + 140 + 4 + 48
# the walk's compulsory traffic per point: its sorted point (16) and permutation entry (4),
# the child slots of the tree read once (24 B x ~2 per point), the velocity read + write (32)
WALK_BYTES_PER_NODE = 16 + 4 + 48 + 32
# DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) of one walk launch of the default
# 1M-node workload, from an ncu capture of that launch: a profiler figure, not something this
# run can measure, so it is reported at that size only, with where it came from
WALK_DRAM_BYTES_1M = 74.4e6
WALK_DRAM_SOURCE = "ncu --set full capture of one k_walk launch, 1M-node workload"
FLOPS_PER_INTERACTION = 20  # FP32 ops per accepted cell or point interaction
FLOPS_PER_OPEN = 8          # per opened-cell test


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=20)
    p.add_argument("--warmup", type=int, default=5)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--nodes", type=int, default=1_000_000)
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--no-modes", action="store_true",
                   help="leave the compact batched and served measurements out of the line")
    p.add_argument("--block", type=int, default=50,
                   help="ticks queued per enqueue call (a block seen twice runs as a CUDA graph)")
    p.add_argument("--no-autotune", action="store_true",
                   help="keep the default tuning (else fl_autotune picks it before the warm-up)")
    p.add_argument("--mixed-charges", action="store_true",
                   help="many-body strengths +20 on every 4th node and -30 on the rest (the cell "
                        "recursion for strengths of both signs) instead of -30 everywhere")
    p.add_argument("--walk-group", type=int, default=0, choices=[0, 1, 16, 32],
                   help="points per tree-walk traversal (FL_TUNE_WALK_GROUP; 0 = by size)")
    p.add_argument("--precision", action="store_true",
                   help="print the many-body force accuracy report instead of the timing line")
    p.add_argument("--precision-ticks", type=int, default=100)
    p.add_argument("--batched", action="store_true",
                   help="print the batched-layout line (many graphs in one batch) instead")
    p.add_argument("--graphs", type=int, default=2048)
    p.add_argument("--serial-sample", type=int, default=48,
                   help="graphs laid out one at a time on the plain engine, for the comparison")
    p.add_argument("--served", action="store_true",
                   help="print the served-layout line (Poisson arrivals, continuous batching)")
    p.add_argument("--jobs", type=int, default=100)
    p.add_argument("--config2", action="store_true",
                   help="print the 100k-node line (link+charge+center+collide+radial, pins) with "
                        "per-force errors against the oracle")
    p.add_argument("--rate", type=float, default=50.0, help="job arrivals per second")
    return p.parse_args()


def workload(n):
    from forcegpu.graphs import benchmark_links, link_defaults, phyllotaxis
    src, dst = benchmark_links(n, n // 2, seed=42)
    bias, strength = link_defaults(n, src, dst)
    xyz = phyllotaxis(n, 3)
    return xyz, src, dst, bias, strength


def alphas(k, start=1.0):
    decay = 1 - 0.001 ** (1 / 300)
    out, a = [], start
    for _ in range(k):
        a += (0 - a) * decay
        out.append(a)
    return np.array(out), a


class Clocks:
    """nvidia-smi samples during the timed region (SM clock, max clock, throttle reasons)."""

    CMD = ["nvidia-smi", "--query-gpu=clocks.sm,clocks.max.sm,power.draw,"
           "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
           "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap",
           "--format=csv,noheader,nounits"]

    def __init__(self):
        self.rows, self.thread, self.done = [], None, threading.Event()

    def start(self):
        cmd = self.CMD + ["-i", os.environ.get("LOCAL_RANK", "0")]

        def poll():
            while not self.done.is_set():
                try:
                    out = subprocess.run(cmd, capture_output=True, text=True, timeout=5).stdout
                except (OSError, subprocess.TimeoutExpired):
                    return
                for line in out.splitlines():
                    self.rows.append([c.strip() for c in line.split(",")])
                self.done.wait(0.05)

        self.thread = threading.Thread(target=poll, daemon=True)
        self.thread.start()

    def stop(self):
        self.done.set()
        if self.thread:
            self.thread.join(timeout=6)
        sm = [float(r[0]) for r in self.rows if len(r) >= 7 and r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in self.rows if len(r) >= 7 and r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in self.rows if len(r) >= 7 for i in range(4)
                          if r[3 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons, "samples": len(sm)}


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f), "measured"
    except OSError:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


def cpu_baseline(xyz, src, dst, n, ticks=2, mixed=False):
    """The oracle (one core) on a bounded sample: 1 warm + `ticks` timed ticks at full size."""
    import oracle
    o = oracle.OracleSim(n, 3, xyz=xyz)
    o.link(src, dst, distance=30.0)
    o.manybody(charges(n, mixed), theta=0.9)
    o.center()
    o.tick(1)
    t0 = time.perf_counter()
    o.tick(ticks)
    dt = time.perf_counter() - t0
    return dt / ticks * 1e3, ticks


def plain_config(n, m):
    """The workload of the headline line, the same in both arms."""
    return {"workload": "3D layout, %d nodes, %d links, link+charge(theta 0.9)+center, "
                        "phyllotaxis start" % (n, m), "nodes": n, "links": m}


# seconds of timed CPU ticks the reference arm may spend (one 1M-node tick takes ~10 s on one core)
REFERENCE_BUDGET_S = 240.0


def run_reference(args):
    """--impl reference: the CPU implementation of the path (the oracle port of the reference's
    CPU simulation; the reference's own is JavaScript and there is no Node.js), rank 0 only.
    The same workload and tick window as the GPU arm: W untimed warm-up ticks, then ticks
    W+1..W+K timed one by one, stopping early only if they exceed REFERENCE_BUDGET_S. One thread:
    the reference's CPU force draws its jiggle from one sequential LCG stream, so its node loop
    cannot be split across threads without changing its results."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    n = args.nodes
    W, K = args.warmup, args.steps
    xyz, src, dst, _, _ = workload(n)
    import oracle
    o = oracle.OracleSim(n, 3, xyz=xyz)
    o.link(src, dst, distance=30.0)
    o.manybody(theta=0.9)
    o.center()
    if W:
        o.tick(W)
    times = []
    while len(times) < K and sum(times) < REFERENCE_BUDGET_S:
        t0 = time.perf_counter()
        o.tick(1)
        times.append(time.perf_counter() - t0)
    ms = sum(times) / len(times) * 1e3
    window = [W + 1, W + len(times)]
    line = {"metric": METRIC, "value": ms, "unit": UNIT, "impl": "reference", "n_gpus": args.gpus,
            "steps": len(times), "warmup": W, "ms_per_step": ms, "higher_is_better": False,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": plain_config(n, int(len(src))), "ticks_timed": window,
            "cpu_baseline": {"value": ms, "unit": UNIT, "cores": 1, "kind": "port",
                             "sample": "ticks %d-%d of the layout, full size, one thread" % tuple(window),
                             "host_cores": os.cpu_count()},
            "e2e": {"value": ms, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def rel_errors(got, ref):
    """Max over targets of |got - ref| / |ref| (vector norms), and the RMS relative error
    ||got - ref|| / ||ref|| over all targets."""
    diff = np.linalg.norm(got - ref, axis=1)
    norm = np.linalg.norm(ref, axis=1)
    ok = norm > 0
    return {"max_rel": float((diff[ok] / norm[ok]).max()) if ok.any() else 0.0,
            "rms_rel": float(np.sqrt((diff ** 2).sum()) / max(np.sqrt((norm ** 2).sum()), 1e-300))}


def gpu_manybody_dv(pos4, theta2, alpha, targets, cells, local=0, dmin2=1.0):
    """The velocity change the engine's many-body force gives the targets from positions pos4
    (velocities 0, decay 1: one tick's velocity is exactly the force's change)."""
    from forcegpu import Engine
    from forcegpu._lib import TUNE_CELL_SUMS, desc_from_gpu
    n = len(pos4)
    eng = Engine(local)
    eng.set_nodes(pos4, 3)
    d, keep = desc_from_gpu({"type": "manyBody", "version": 1, "strengths": np.full(n, -30.0),
                             "distanceMin2": dmin2, "distanceMax2": math.inf, "theta2": theta2}, 1, n)
    eng.set_forces([(d, keep)])
    eng.set_tuning(TUNE_CELL_SUMS, cells)
    eng.set_seed(12345)
    eng.enqueue(np.array([alpha]), 1.0)
    _, vel = eng.sync()
    eng.close()
    return vel[targets, :3].astype(np.float64)


def run_precision(args):
    """--precision: accuracy of the many-body force from one captured state of the layout.

    The 1M-node workload runs `--precision-ticks` ticks on the GPU; from that state (positions,
    the next tick's alpha) the many-body velocity change of 8,192 random target nodes is taken
    from the GPU (each cell-sum variant), from the oracle's d3 walk (the reference's CPU
    Barnes-Hut) and from the oracle's FP64 exact sum over all pairs, for theta 0.5 and 0.9; and
    for theta 0 (the exact path) on a 20,000-node layout. Prints one JSON line."""
    import oracle
    from forcegpu import Engine
    from forcegpu._lib import CELLS_AUTO, CELLS_FP32, CELLS_FP64_TOP, desc_from_gpu
    threads = os.cpu_count() or 1
    out = {"report": "many-body force accuracy", "targets": 8192, "host_threads": threads,
           "metric": "relative error of the velocity change vs the FP64 exact all-pairs sum",
           "cases": []}

    def layout_state(n, ticks):
        xyz, src, dst, bias, strength = workload(n)
        pos4 = np.zeros((n, 4), np.float32)
        pos4[:, :3] = xyz
        eng = Engine(0)
        eng.set_nodes(pos4, 3)
        links = {"type": "link", "version": 1, "source": src, "target": dst, "iterations": 1,
                 "strengths": strength, "distances": np.full(len(src), 30.0), "bias": bias}
        charge = {"type": "manyBody", "version": 1, "strengths": np.full(n, -30.0),
                  "distanceMin2": 1.0, "distanceMax2": math.inf, "theta2": 0.81}
        eng.set_forces([desc_from_gpu(links, 1, n), desc_from_gpu(charge, 2, n),
                        desc_from_gpu({"type": "center", "x": 0, "y": 0, "z": 0, "strength": 1.0}, 3, n)])
        eng.set_seed(12345)
        al, _ = alphas(ticks + 1)
        if ticks:
            eng.enqueue(al[:ticks], 0.6)
        pos, _ = eng.sync()
        eng.close()
        return pos, float(al[ticks])

    rng = np.random.default_rng(7)
    for n, thetas, ticks in ((args.nodes, (0.5, 0.9), args.precision_ticks), (20_000, (0.0,), args.precision_ticks)):
        pos, alpha = layout_state(n, ticks)
        targets = np.sort(rng.choice(n, min(8192, n), replace=False)).astype(np.int32)
        o = oracle.OracleSim(n, 3, xyz=pos[:, :3].astype(np.float64))
        o.manybody(theta=0.9)
        t0 = time.perf_counter()
        exact = o.manybody_probe(0, alpha, targets, oracle.MODE_EXACT, threads=threads)
        t_exact = time.perf_counter() - t0
        for theta in thetas:
            case = {"nodes": n, "theta": theta, "ticks": ticks, "alpha": alpha,
                    "exact_seconds": t_exact}
            if theta > 0:
                ot = oracle.OracleSim(n, 3, xyz=pos[:, :3].astype(np.float64))
                ot.manybody(theta=theta)
                d3 = ot.manybody_probe(0, alpha, targets, oracle.MODE_D3)
                case["cpu_barnes_hut_vs_exact"] = rel_errors(d3, exact)
                for name, cells in (("fixed_point", CELLS_AUTO), ("fp64_top", CELLS_FP64_TOP),
                                    ("fp32", CELLS_FP32)):
                    g = gpu_manybody_dv(pos, theta * theta, alpha, targets, cells)
                    case["gpu_%s_vs_exact" % name] = rel_errors(g, exact)
                    case["gpu_%s_vs_cpu_barnes_hut" % name] = rel_errors(g, d3)
            else:
                g = gpu_manybody_dv(pos, 0.0, alpha, targets, CELLS_AUTO)
                case["gpu_exact_path_vs_exact"] = rel_errors(g, exact)
            out["cases"].append(case)
            print(json.dumps(case), file=sys.stderr, flush=True)
    print(json.dumps(out), flush=True)


def batch_workload(graphs, seed=2024):
    """The batched configuration: `graphs` independent 3D graphs, sizes log-uniform in
    [100, 20000] (seeded), the reference benchmark's link generator at 1.5 links per node,
    phyllotaxis starts; link + charge (theta 0.9) + center, d3's defaults."""
    from forcegpu.batch import GraphSpec
    from forcegpu.graphs import benchmark_links, phyllotaxis
    rng = np.random.default_rng(seed)
    sizes = np.exp(rng.uniform(np.log(100), np.log(20000), graphs)).astype(np.int64)
    specs = []
    for i, n in enumerate(sizes):
        src, dst = benchmark_links(int(n), int(n) // 2, seed=1000 + i)
        specs.append(GraphSpec(xyz=phyllotaxis(int(n), 3), source=src, target=dst))
    return specs


def batched_measure(graphs, ticks, serial_sample, warmup, autotune, local=0):
    """Layouts per second of the batched engine on `graphs` graphs of the batched workload,
    `ticks` ticks each (every graph's own d3 alpha schedule), against the plain engine laying out
    a sample of the same graphs one at a time (the same work per graph). The batched figure is
    taken twice: device time of the queued ticks, and wall time from the graphs' upload to the
    positions read back (the like of the serial figure, which is wall time per graph)."""
    import torch
    from forcegpu import Engine
    from forcegpu.batch import Batch
    from forcegpu.graphs import link_defaults
    specs = batch_workload(graphs)
    nodes = int(sum(len(s.xyz) for s in specs))
    b = Batch(local)
    b.set_graphs(specs, ndim=3, seed=12345)
    tuning = b.autotune(ticks=3) if autotune else None
    stream = torch.cuda.ExternalStream(b.stream(), device=local)
    # warm-up on the schedule's first ticks, then the timed full layout from the start
    b.run(warmup)
    b.sync()
    clocks = Clocks()
    clocks.start()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    b.set_graphs(specs, ndim=3, seed=12345)
    sched = b.alpha_schedule(ticks)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    launches0 = b.launches()
    e0.record(stream)
    b.enqueue(sched)
    e1.record(stream)
    pos, _ = b.sync()
    wall = time.perf_counter() - t0
    clk = clocks.stop()
    dev_ms = e0.elapsed_time(e1)
    launches = b.launches() - launches0
    assert np.isfinite(pos).all()
    dev_bytes = b.device_bytes()
    b.close()
    # the plain engine, one graph after another (a sample, each a full layout of `ticks` ticks)
    rng = np.random.default_rng(99)
    sample = rng.choice(len(specs), min(serial_sample, len(specs)), replace=False)
    eng = Engine(local)
    sample_nodes = 0
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    for gi in sample:
        sp = specs[gi]
        n = len(sp.xyz)
        sample_nodes += n
        pos4 = np.zeros((n, 4), np.float32)
        pos4[:, :3] = sp.xyz
        eng.set_nodes(pos4, 3)
        bias, strength = link_defaults(n, sp.source, sp.target)
        eng.set_forces(plain_forces(n, sp.source, sp.target, bias, strength))
        al, _ = alphas(ticks)
        eng.enqueue(al, 0.6)
        eng.sync()
    serial_s = time.perf_counter() - t1
    eng.close()
    serial = len(sample) / serial_s
    return {"graphs": len(specs), "nodes": nodes, "ticks": ticks,
            "layouts_per_s": len(specs) / (dev_ms / 1e3),
            "layouts_per_s_wall": len(specs) / wall,
            "ms_per_tick": dev_ms / ticks,
            "serial_plain_layouts_per_s": serial, "serial_sample_graphs": len(sample),
            "serial_sample_nodes": sample_nodes,
            "speedup_vs_serial_plain": len(specs) / wall / serial,
            "gpu_launches": int(launches), "tuning": tuning, "clocks": clk,
            "device_bytes": dev_bytes,
            "workload": "%d 3D graphs, sizes log-uniform in [100, 20000] (seed 2024), 1.5 links/node, "
                        "link+charge(theta 0.9)+center, %d ticks each" % (len(specs), ticks)}


def batched_summary(args, local):
    """The compact batched measurement of the default line: 256 graphs x 100 ticks."""
    return batched_measure(256, 100, 16, 3, autotune=False, local=local)


def run_batched(args):
    """--batched: the batched configuration, 2,048 graphs x 300 ticks."""
    m = batched_measure(args.graphs, 300, args.serial_sample, args.warmup, not args.no_autotune)
    line = {"metric": "layouts/s, %d graphs x 300 ticks (batched)" % m["graphs"],
            "value": m["layouts_per_s"], "unit": "layouts/s", "n_gpus": 1, "steps": 300,
            "warmup": args.warmup, "ms_per_step": m["ms_per_tick"], "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": m["workload"], "graphs": m["graphs"], "nodes": m["nodes"],
                       "tuning": m["tuning"]},
            "e2e": {"value": m["layouts_per_s_wall"], "unit": "layouts/s",
                    "h2d_bytes_per_step": 8 * m["graphs"],
                    "d2h_bytes_per_step": 32 * m["nodes"] / 300},
            "serial_plain": {"value": m["serial_plain_layouts_per_s"], "unit": "layouts/s",
                             "sample_graphs": m["serial_sample_graphs"],
                             "sample_nodes": m["serial_sample_nodes"]},
            "speedup_vs_serial_plain": m["speedup_vs_serial_plain"],
            "gpu_launches": m["gpu_launches"], "clocks": m["clocks"],
            "device_bytes": m["device_bytes"]}
    print(json.dumps(line), flush=True)


def served_jobs(count, rate, seed=77):
    """The served configuration: Poisson arrivals at `rate` jobs/s; each job a 2D or 3D graph
    (50/50), size log-uniform in [500, 200000], the reference benchmark's link generator at 1 to
    3 links per node (uniform), link + charge + center, and in 30 % of jobs also collide with
    radii uniform in [1, 5]; tick count uniform in [100, 500]."""
    from forcegpu.graphs import benchmark_links, phyllotaxis
    from forcegpu.serve import Job
    rng = np.random.default_rng(seed)
    t = np.cumsum(rng.exponential(1.0 / rate, count))
    jobs = []
    for i in range(count):
        n = int(np.exp(rng.uniform(np.log(500), np.log(200_000))))
        dims = 2 if rng.random() < 0.5 else 3
        per = rng.uniform(1.0, 3.0)
        src, dst = benchmark_links(n, max(0, int(n * per) - (n - 1)), seed=5000 + i)
        radii = rng.uniform(1.0, 5.0, n) if rng.random() < 0.3 else None
        jobs.append(Job(xyz=phyllotaxis(n, dims)[:, :dims], source=src, target=dst,
                        ticks=int(rng.integers(100, 501)), radii=radii, arrival=float(t[i])))
    return jobs


def served_measure(count, rate, local=0):
    """The layout server under Poisson arrivals (continuous batching), and the same jobs solved
    one at a time on the plain engine, first come first served (each job's service time
    measured alone, the queue replayed against the same arrivals)."""
    import copy
    from forcegpu.serve import LayoutServer, latency_summary
    jobs = served_jobs(count, rate)
    work = copy.deepcopy(jobs)
    # the server, in real time: arrivals are offsets from the start
    srv = LayoutServer(device=local, hbm_budget=96 << 30, block=50).warmup()
    clocks = Clocks()
    clocks.start()
    t0 = time.perf_counter()
    for j in work:
        j.arrival = t0 + j.arrival
        srv.submit(j)
    srv.run_until_idle()
    makespan = time.perf_counter() - t0
    clk = clocks.stop()
    srv.close()
    assert all(j.result is not None and np.isfinite(j.result).all() for j in work)
    served = latency_summary(work)
    serial = copy.deepcopy(jobs)
    one = LayoutServer(device=local, hbm_budget=96 << 30, block=50, batching=False,
                       plain_graphs=True).warmup()
    service = []
    for j in serial:
        j.arrival = None
        one.submit(j)
        s0 = time.perf_counter()
        one.run_until_idle()
        service.append(time.perf_counter() - s0)
    one.close()
    finish, lat = 0.0, []
    for j, sv in zip(jobs, service):
        finish = max(finish, j.arrival) + sv
        lat.append(finish - j.arrival)
    lat = np.array(lat)
    node_ticks = sum(j.n * j.ticks for j in jobs)
    serial_lps = len(jobs) / max(finish - jobs[0].arrival, 1e-9)
    return {"jobs": len(jobs), "rate_per_s": rate, "layouts_per_s": len(jobs) / makespan,
            "makespan_s": makespan, "latency": served,
            "serial_plain": {"layouts_per_s": serial_lps,
                             "p50_s": float(np.percentile(lat, 50)),
                             "p99_s": float(np.percentile(lat, 99)),
                             "busy_seconds": float(sum(service))},
            "speedup_vs_serial_plain": len(jobs) / makespan / serial_lps,
            "node_ticks": int(node_ticks), "clocks": clk,
            "workload": "%d jobs, Poisson arrivals at %g/s, 2D/3D 50/50, sizes log-uniform "
                        "[500, 200000], 1-3 links/node, 30%% collide, ticks uniform [100, 500]"
                        % (len(jobs), rate)}


def served_summary(args, local):
    """The compact served measurement of the default line: 40 jobs arriving at 2,000/s."""
    return served_measure(40, 2000.0, local)


def run_served(args):
    """--served: the served configuration."""
    m = served_measure(args.jobs, args.rate)
    line = {"metric": "served layouts/s and p99 latency (continuous batching)",
            "value": m["layouts_per_s"], "unit": "layouts/s", "n_gpus": 1, "steps": m["jobs"],
            "warmup": 0, "ms_per_step": 1e3 * m["makespan_s"] / m["jobs"],
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic", "config": {"workload": m["workload"], "node_ticks": m["node_ticks"]},
            "latency": m["latency"], "serial_plain": m["serial_plain"],
            "speedup_vs_serial_plain": m["speedup_vs_serial_plain"], "clocks": m["clocks"]}
    print(json.dumps(line), flush=True)


def run_config2(args):
    """--config2: 100,000 nodes in 3D, the benchmark's link generator, link + charge (theta 0.9)
    + center + collide (radius uniform in [1, 5], 1 iteration, grid path) + radial (r 200,
    strength 0.05), every 10th node pinned at its start; 300 ticks timed. Then, from the state
    after those ticks, each force's velocity change on 4,096 random nodes against the oracle
    (link and collide in their Jacobi form, as the GPU applies them) and, for the many-body
    force, against the FP64 exact sum."""
    import torch
    import oracle
    from forcegpu import Engine
    from forcegpu._lib import desc_from_gpu
    n, ticks = 100_000, 300
    xyz, src, dst, bias, strength = workload(n)
    rng = np.random.default_rng(4)
    radii = rng.uniform(1.0, 5.0, n).astype(np.float32).astype(np.float64)
    pos4 = np.zeros((n, 4), np.float32)
    pos4[:, :3] = xyz
    fix4 = pos4.copy()
    mask = np.where(np.arange(n) % 10 == 0, 7, 0).astype(np.uint32)
    g = {
        "link": {"type": "link", "version": 1, "source": src, "target": dst, "iterations": 1,
                 "strengths": strength, "distances": np.full(len(src), 30.0), "bias": bias},
        "charge": {"type": "manyBody", "version": 1, "strengths": np.full(n, -30.0),
                   "distanceMin2": 1.0, "distanceMax2": math.inf, "theta2": 0.81},
        "center": {"type": "center", "x": 0, "y": 0, "z": 0, "strength": 1.0},
        "collide": {"type": "collide", "version": 1, "radii": radii, "strength": 1.0, "iterations": 1},
        "radial": {"type": "radial", "version": 1, "radiuses": np.full(n, 200.0),
                   "strengths": np.full(n, 0.05), "x": 0, "y": 0, "z": 0},
    }
    names = ["link", "charge", "center", "collide", "radial"]
    eng = Engine(0)
    eng.set_nodes(pos4, 3, None, fix4, mask)
    eng.set_forces([desc_from_gpu(g[k], i + 1, n) for i, k in enumerate(names)])
    eng.set_seed(12345)
    al, _ = alphas(ticks + args.warmup + 1)
    eng.enqueue(al[:args.warmup], 0.6)
    eng.idle()
    stream = torch.cuda.ExternalStream(eng.stream(), device=0)
    eng.profile(True)
    clocks = Clocks()
    clocks.start()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    eng.enqueue(al[args.warmup:args.warmup + ticks], 0.6)
    e1.record(stream)
    pos, vel = eng.sync()
    clk = clocks.stop()
    prof = eng.profile_read()
    eng.profile(False)
    eng.close()
    ms = e0.elapsed_time(e1) / ticks
    alpha = float(al[args.warmup + ticks])
    targets = np.sort(rng.choice(n, 4096, replace=False)).astype(np.int32)
    p64, v64 = pos[:, :3].astype(np.float64), vel[:, :3].astype(np.float64)

    def gpu_dv(name):
        e = Engine(0)
        e.set_nodes(pos, 3, vel)
        e.set_forces([desc_from_gpu(g[name], 1, n)])
        e.set_seed(777)
        e.enqueue(np.array([alpha]), 1.0)
        _, v2 = e.sync()
        e.close()
        return (v2[:, :3].astype(np.float64) - v64)[targets]

    def cpu_dv(add, probe_mode=None):
        o = oracle.OracleSim(n, 3, xyz=p64, vxyz=v64)
        add(o)
        if probe_mode is not None:
            return o.manybody_probe(0, alpha, targets, probe_mode, threads=os.cpu_count() or 1)
        o.apply_force(0, alpha)
        return (o.state()[1] - v64)[targets]

    errors = {}
    errors["link_vs_cpu_jacobi"] = rel_errors(
        gpu_dv("link"), cpu_dv(lambda o: o.link(src, dst, 30.0, strength, 1, oracle.MODE_JACOBI)))
    charge_gpu = gpu_dv("charge")
    errors["charge_vs_cpu_barnes_hut"] = rel_errors(
        charge_gpu, cpu_dv(lambda o: o.manybody(theta=0.9), oracle.MODE_D3))
    errors["charge_vs_fp64_exact"] = rel_errors(
        charge_gpu, cpu_dv(lambda o: o.manybody(theta=0.9), oracle.MODE_EXACT))
    errors["cpu_barnes_hut_vs_fp64_exact"] = rel_errors(
        cpu_dv(lambda o: o.manybody(theta=0.9), oracle.MODE_D3),
        cpu_dv(lambda o: o.manybody(theta=0.9), oracle.MODE_EXACT))
    errors["collide_vs_cpu_jacobi"] = rel_errors(
        gpu_dv("collide"), cpu_dv(lambda o: o.collide(radii, 1.0, 1, oracle.MODE_JACOBI)))
    errors["radial_vs_cpu"] = rel_errors(
        gpu_dv("radial"), cpu_dv(lambda o: o.radial(np.full(n, 200.0), 0.05)))
    line = {"metric": "ms/tick at 100k nodes (3D link+charge+center+collide+radial, pins)",
            "value": ms, "unit": "ms/tick", "n_gpus": 1, "steps": ticks, "warmup": args.warmup,
            "ms_per_step": ms, "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32", "data": "synthetic",
            "config": {"workload": "100,000 nodes, 149,999 links, collide r U[1,5] (grid), radial "
                                   "r 200 s 0.05, every 10th node pinned, 300 ticks", "nodes": n},
            "kernels": {k: {"ms_per_tick": v[0] / ticks, "launches": v[1]} for k, v in prof.items()},
            "force_errors_4096_targets": errors, "clocks": clk}
    print(json.dumps(line), flush=True)


def charges(n, mixed=False):
    """The many-body strengths: -30 (d3's default), or with mixed, +20 on every 4th node."""
    return np.where(np.arange(n) % 4 == 0, 20.0, -30.0) if mixed else np.full(n, -30.0)


def plain_forces(n, src, dst, bias, strength, mixed=False):
    """The benchmark's force list: link (distance 30, d3's default strength and bias), many-body
    (-30, or charges(n, mixed), theta 0.9), center."""
    from forcegpu._lib import desc_from_gpu
    links = {"type": "link", "version": 1, "source": src, "target": dst, "iterations": 1,
             "strengths": strength, "distances": np.full(len(src), 30.0), "bias": bias}
    charge = {"type": "manyBody", "version": 1, "strengths": charges(n, mixed), "distanceMin2": 1.0,
              "distanceMax2": math.inf, "theta2": 0.81}
    center = {"type": "center", "x": 0, "y": 0, "z": 0, "strength": 1.0}
    return [desc_from_gpu(links, 1, n), desc_from_gpu(charge, 2, n), desc_from_gpu(center, 3, n)]


def main():
    args = parse()
    if args.config2:
        run_config2(args)
        return
    if args.served:
        run_served(args)
        return
    if args.impl == "reference":
        run_reference(args)
        return
    if args.precision:
        run_precision(args)
        return
    if args.batched:
        run_batched(args)
        return
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    import torch
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    from forcegpu import Engine
    from forcegpu._lib import (Q_DEVICE_BYTES, Q_LAUNCHES, Q_WALK_APPLIES, Q_WALK_OPENS,
                               Q_WALK_RARE, Q_WALK_TESTS, Q_WALK_USEFUL, TUNE_WALK_GROUP)

    n = args.nodes
    W, K = args.warmup, args.steps
    xyz, src, dst, bias, strength = workload(n)
    pos4 = np.zeros((n, 4), np.float32)
    pos4[:, :3] = xyz
    eng = Engine(local)
    eng.set_nodes(pos4, 3)
    eng.set_forces(plain_forces(n, src, dst, bias, strength, args.mixed_charges))
    eng.set_seed(12345)
    eng.set_tuning(TUNE_WALK_GROUP, args.walk_group)
    decay = 0.6
    tuning = None
    if not args.no_autotune:  # outside the timed region, from the same start (state restored)
        tuning = eng.autotune(ticks=10, alpha=0.5, decay=decay)
    # ticks are queued in blocks of B, as an application queues a frame's or a batch's worth:
    # the engine runs a block it has seen before as one CUDA graph
    B = max(1, min(args.block, K))
    al, _ = alphas(W + K + 2 * K + B + 9)

    def run(first, count):
        k = first
        while k < first + count:
            c = min(B, first + count - k)
            eng.enqueue(al[k:k + c], decay)
            k += c

    stream = torch.cuda.ExternalStream(eng.stream(), device=local)
    clocks = Clocks()
    clocks.start()
    # pre-roll, outside the count of warm-up ticks: the same W + K ticks twice from the start
    # (fl_upload_all puts the start state back and keeps the captured blocks), so that every
    # block the warm-up and the timed region queue has been seen twice and runs as a CUDA graph
    for _ in range(2):
        run(0, W)
        run(W, K)
        eng.idle()
        eng.upload_all(pos4)
    run(0, W)  # the warm-up: ticks 1..W
    eng.idle()

    # timed region: ticks W+1..W+K, state resident, CUDA events on the engine's stream
    def barrier():
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    launches0 = eng.query(Q_LAUNCHES)
    barrier()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    run(W, K)
    e1.record(stream)
    eng.idle()
    barrier()
    clk = clocks.stop()
    ms_total = e0.elapsed_time(e1)
    launches = eng.query(Q_LAUNCHES) - launches0
    total = W + K
    # the per-kernel times: one more block, with the kernels timed one group at a time
    eng.profile(True)
    eng.enqueue(al[total:total + B], decay)
    eng.idle()
    prof = eng.profile_read()
    eng.profile(False)
    total += B
    if world > 1:  # the slowest replica
        t = torch.tensor([ms_total], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms_total = float(t.item())
    ms_tick = ms_total / K

    # the walk's counted work, from one more tick with the walk's counters on (outside the
    # timed region): FP32 operations per launch for the FP32-pipe view of the roofline
    eng.profile(2)
    eng.enqueue(al[total:total + 1], decay)
    eng.idle()
    walk_count = {k: eng.query(q) for k, q in (("tests", Q_WALK_TESTS), ("useful", Q_WALK_USEFUL),
                                              ("opens", Q_WALK_OPENS), ("applies", Q_WALK_APPLIES),
                                              ("rare_rounds", Q_WALK_RARE))}
    eng.profile(False)

    def max_over_ranks(v):
        if world > 1:
            t = torch.tensor([v], device="cuda")
            torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
            v = float(t.item())
        return v

    # e2e through the C ABI with pinned host buffers, K ticks from the state reached
    e2e = e2e_float4 = None
    if not args.no_e2e:
        hp = torch.empty((n, 3), dtype=torch.float32, pin_memory=True)
        hv = torch.empty((n, 3), dtype=torch.float32, pin_memory=True)
        eng.sync_packed_into(hp.data_ptr(), hv.data_ptr())
        hpn = hp.numpy()
        a2 = al[total + 1:total + 1 + K]
        barrier()
        t0 = time.perf_counter()
        for i in range(K):
            # the upload is queued, not waited for: the tick follows it on the stream with no
            # host round trip, and the readback's wait covers all three
            eng.update_positions_packed_async(0, hpn)
            eng.enqueue(a2[i:i + 1], decay)
            eng.sync_packed_into(hp.data_ptr(), hv.data_ptr())
        barrier()
        e2e_ms = max_over_ranks((time.perf_counter() - t0) * 1e3 / K)
        e2e = {"value": e2e_ms, "unit": UNIT, "h2d_bytes_per_step": 12 * n + 8,
               "d2h_bytes_per_step": 24 * n,
               "calls": "fl_update_positions_packed_async + fl_enqueue + fl_sync_packed"}
        # the same through the float4 calls: the reference's vec4 layout, 16 B per node each way
        hp4 = torch.empty((n, 4), dtype=torch.float32, pin_memory=True)
        hv4 = torch.empty((n, 4), dtype=torch.float32, pin_memory=True)
        eng.sync_into(hp4.data_ptr(), hv4.data_ptr())
        hp4n = hp4.numpy()
        a3 = al[total + 1 + K:total + 1 + 2 * K]
        barrier()
        t0 = time.perf_counter()
        for i in range(K):
            eng.update_positions(0, hp4n)
            eng.enqueue(a3[i:i + 1], decay)
            eng.sync_into(hp4.data_ptr(), hv4.data_ptr())
        barrier()
        ms4 = max_over_ranks((time.perf_counter() - t0) * 1e3 / K)
        e2e_float4 = {"value": ms4, "unit": UNIT, "h2d_bytes_per_step": 16 * n + 8,
                      "d2h_bytes_per_step": 32 * n, "calls": "fl_update_positions + fl_enqueue + fl_sync"}

    dev_bytes = eng.query(Q_DEVICE_BYTES)
    peaks, peak_kind = measured_peaks()
    walk_ms, walk_n = prof.get("walk", (0.0, 0))
    walk_avg = walk_ms / max(1, walk_n)
    walk_bytes = WALK_BYTES_PER_NODE * n
    achieved = walk_bytes / (walk_avg * 1e-3) / 1e9 if walk_avg else None
    roof = {"bound": "hbm", "kernel": "k_walk", "achieved": achieved, "peak": peaks["hbm_gbs"],
            "unit": "GB/s", "frac": (achieved / peaks["hbm_gbs"]) if achieved else None,
            "traffic": WALK_DRAM_BYTES_1M if n == 1_000_000 else None,
            "traffic_source": WALK_DRAM_SOURCE if n == 1_000_000 else None, "peak_kind": peak_kind,
            "algorithmic_bytes_per_launch": walk_bytes, "avg_launch_ms": walk_avg,
            "tick_bytes": BYTES_PER_NODE_TICK * n,
            "tick_hbm_frac": BYTES_PER_NODE_TICK * n / (ms_tick * 1e-3) / 1e9 / peaks["hbm_gbs"]}
    flops = FLOPS_PER_INTERACTION * walk_count["applies"] + FLOPS_PER_OPEN * walk_count["opens"]
    sms = torch.cuda.get_device_properties(local).multi_processor_count
    mhz = clk["sm_mhz"] or 2070.0
    fp32_peak = sms * 128 * 2 * mhz * 1e6 / 1e12  # TFLOP/s at the median sampled SM clock
    fp32_achieved = flops / (walk_avg * 1e-3) / 1e12 if walk_avg else None
    roof["fp32"] = {"achieved": fp32_achieved, "peak": fp32_peak, "unit": "TFLOP/s",
                    "frac": fp32_achieved / fp32_peak if fp32_achieved else None,
                    "flops_per_launch": flops, "sms": sms, "sm_mhz": mhz,
                    "per_point": {k: v / n for k, v in walk_count.items()}}
    kernels = {k: {"ms_per_tick": v[0] / B, "launches": v[1]} for k, v in prof.items()}

    line = {"metric": METRIC, "value": ms_tick, "unit": UNIT, "n_gpus": world, "steps": K,
            "warmup": W, "ms_per_step": ms_tick, "higher_is_better": False,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": dict(plain_config(n, len(src)),
                           **({"charges": "+20 on every 4th node, -30 elsewhere"}
                              if args.mixed_charges else {})),
            "ticks_timed": [W + 1, W + K],
            "preroll": "the same %d ticks twice before the warm-up, from the start state "
                       "(fl_upload_all), so that every tick block runs as a CUDA graph" % (W + K),
            "tick_block": B, "tuning": tuning,
            "l2": "working set %.0f MB > 126 MB L2 (no flush)" % (dev_bytes / 1e6),
            "gpu_launches": int(launches), "clocks": clk, "roofline": roof, "kernels": kernels}
    if world > 1:
        line["replicas"] = world
        line["aggregate_ticks_per_s"] = world * K / (ms_total * 1e-3)
        line["value_note"] = "ms per tick of one simulation (the slowest of %d independent replicas)" % world
    if e2e:
        line["e2e"] = e2e
        line["e2e_float4"] = e2e_float4
    eng.close()
    if not args.no_modes:
        line["batched"] = batched_summary(args, local)
        line["served"] = served_summary(args, local)
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        ms_cpu, t = cpu_baseline(xyz, src, dst, n, mixed=args.mixed_charges)
        line["cpu_baseline"] = {"value": ms_cpu, "unit": UNIT, "cores": 1, "kind": "port",
                                "sample": "ticks 2-%d of the same 1M-node layout (oracle, FP64, one core)" % (1 + t),
                                "host_cores": os.cpu_count()}
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
