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

With --impl reference, the same workload runs on the CPU implementation (the oracle; the
reference's own CPU code is JavaScript, and there is no Node.js on this machine).
Multi-GPU: the single simulation does not shard; N ranks run N independent replicas.
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
# DRAM bytes (read + write) of one walk launch at the default 1M-node workload, from ncu
# (profiles/walk_1m_3d.md); reported as the roofline's measured traffic at that size only
WALK_DRAM_BYTES_1M = 73.5e6
FLOPS_PER_INTERACTION = 20  # FP32 ops per accepted cell or point interaction
FLOPS_PER_OPEN = 8          # per opened-cell test


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=300)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--nodes", type=int, default=1_000_000)
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--block", type=int, default=50,
                   help="ticks queued per enqueue call (a block seen twice runs as a CUDA graph)")
    p.add_argument("--no-autotune", action="store_true",
                   help="keep the default tuning (else fl_autotune picks it before the warm-up)")
    p.add_argument("--walk-group", type=int, default=32, choices=[16, 32],
                   help="points per tree-walk traversal (FL_TUNE_WALK_GROUP)")
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


def cpu_baseline(xyz, src, dst, n, ticks=2):
    """The oracle (one core) on a bounded sample: 1 warm + `ticks` timed ticks at full size."""
    import oracle
    o = oracle.OracleSim(n, 3, xyz=xyz)
    o.link(src, dst, distance=30.0)
    o.manybody(theta=0.9)
    o.center()
    o.tick(1)
    t0 = time.perf_counter()
    o.tick(ticks)
    dt = time.perf_counter() - t0
    return dt / ticks * 1e3, ticks


def run_reference(args):
    """--impl reference: the CPU implementation of the path (the oracle port), rank 0 only."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    n = args.nodes
    xyz, src, dst, _, _ = workload(n)
    import oracle
    o = oracle.OracleSim(n, 3, xyz=xyz)
    o.link(src, dst, distance=30.0)
    o.manybody(theta=0.9)
    o.center()
    warm = max(1, min(args.warmup, 1))
    steps = max(1, min(args.steps, 5))
    o.tick(warm)
    t0 = time.perf_counter()
    o.tick(steps)
    ms = (time.perf_counter() - t0) / steps * 1e3
    line = {"metric": METRIC, "value": ms, "unit": UNIT, "impl": "reference", "n_gpus": args.gpus,
            "steps": steps, "warmup": warm, "ms_per_step": ms, "higher_is_better": False,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": "3D layout, %d nodes, %d links, link+charge(theta 0.9)+center"
                                   % (n, len(src)), "nodes": n, "links": int(len(src))},
            "cpu_baseline": {"value": ms, "unit": UNIT, "cores": 1, "kind": "port",
                             "sample": "ticks %d-%d of the layout, full size" % (warm + 1, warm + steps)},
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


def run_batched(args):
    """--batched: layouts per second of the batched engine on a batch of many graphs, 300 ticks
    each (every graph's own d3 alpha schedule), against the plain engine laying out a sample of
    the same graphs one at a time (the same work per graph; layouts/s of the sample)."""
    import torch
    from forcegpu import Engine
    from forcegpu._lib import desc_from_gpu
    from forcegpu.batch import Batch
    from forcegpu.graphs import link_defaults
    ticks = 300
    specs = batch_workload(args.graphs)
    nodes = int(sum(len(s.xyz) for s in specs))
    b = Batch(0)
    b.set_graphs(specs, ndim=3, seed=12345)
    tuning = None if args.no_autotune else b.autotune(ticks=3)
    stream = torch.cuda.ExternalStream(b.stream(), device=0)
    # warm-up on a copy of the schedule, then the timed full layout from the start
    b.run(args.warmup)
    b.sync()
    b.set_graphs(specs, ndim=3, seed=12345)
    sched = b.alpha_schedule(ticks)
    clocks = Clocks()
    clocks.start()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    launches0 = b.launches()
    t0 = time.perf_counter()
    e0.record(stream)
    b.enqueue(sched)
    e1.record(stream)
    pos, _ = b.sync()
    wall = time.perf_counter() - t0
    clk = clocks.stop()
    dev_ms = e0.elapsed_time(e1)
    launches = b.launches() - launches0
    assert np.isfinite(pos).all()
    batched = len(specs) / (dev_ms / 1e3)
    # the plain engine, one graph after another (a sample; each a full 300-tick layout)
    rng = np.random.default_rng(99)
    sample = rng.choice(len(specs), min(args.serial_sample, len(specs)), replace=False)
    eng = Engine(0)
    sample_nodes = 0
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    for gi in sample:
        s = specs[gi]
        n = len(s.xyz)
        sample_nodes += n
        pos4 = np.zeros((n, 4), np.float32)
        pos4[:, :3] = s.xyz
        eng.set_nodes(pos4, 3)
        bias, strength = link_defaults(n, s.source, s.target)
        ld = desc_from_gpu({"type": "link", "version": 1, "source": s.source, "target": s.target,
                            "iterations": 1, "strengths": strength,
                            "distances": np.full(len(s.source), 30.0), "bias": bias}, 1, n)
        cd = desc_from_gpu({"type": "manyBody", "version": 1, "strengths": np.full(n, -30.0),
                            "distanceMin2": 1.0, "distanceMax2": math.inf, "theta2": 0.81}, 2, n)
        xd = desc_from_gpu({"type": "center", "x": 0, "y": 0, "z": 0, "strength": 1.0}, 3, n)
        eng.set_forces([ld, cd, xd])
        al, _ = alphas(ticks)
        eng.enqueue(al, 0.6)
        eng.sync()
    serial_s = time.perf_counter() - t1
    eng.close()
    serial = len(sample) / serial_s
    line = {"metric": "layouts/s, 2048 graphs x 300 ticks (batched)", "value": batched,
            "unit": "layouts/s", "n_gpus": 1, "steps": ticks, "warmup": args.warmup,
            "ms_per_step": dev_ms / ticks, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": "%d 3D graphs, sizes log-uniform in [100, 20000] (seed 2024), "
                                   "1.5 links/node, link+charge(theta 0.9)+center, 300 ticks each"
                                   % len(specs), "graphs": len(specs), "nodes": nodes,
                       "tuning": tuning},
            "e2e": {"value": len(specs) / wall, "unit": "layouts/s",
                    "h2d_bytes_per_step": 8 * len(specs), "d2h_bytes_per_step": 32 * nodes / ticks},
            "serial_plain": {"value": serial, "unit": "layouts/s", "sample_graphs": len(sample),
                             "sample_nodes": sample_nodes, "seconds": serial_s},
            "speedup_vs_serial_plain": batched / serial,
            "gpu_launches": int(launches), "clocks": clk,
            "device_bytes": b.device_bytes()}
    print(json.dumps(line), flush=True)
    b.close()


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


def run_served(args):
    """--served: the layout server under Poisson arrivals (continuous batching), and the same
    jobs solved one at a time on the plain engine, first come first served."""
    import copy
    from forcegpu.serve import LayoutServer, latency_summary
    jobs = served_jobs(args.jobs, args.rate)
    work = copy.deepcopy(jobs)
    # the server, in real time: arrivals are offsets from the start
    srv = LayoutServer(hbm_budget=96 << 30, block=50).warmup()
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
    # serial plain solves, FIFO under the same arrivals: each job's service time measured alone
    serial = copy.deepcopy(jobs)
    one = LayoutServer(hbm_budget=96 << 30, block=50, batching=False, plain_graphs=True).warmup()
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
    line = {"metric": "served layouts/s and p99 latency (continuous batching)",
            "value": len(jobs) / makespan, "unit": "layouts/s", "n_gpus": 1, "steps": len(jobs),
            "warmup": 0, "ms_per_step": 1e3 * makespan / len(jobs), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": "%d jobs, Poisson arrivals at %g/s, 2D/3D 50/50, sizes "
                                   "log-uniform [500, 200000], 1-3 links/node, 30%% collide, "
                                   "ticks uniform [100, 500]" % (len(jobs), args.rate),
                       "node_ticks": int(node_ticks)},
            "latency": served,
            "serial_plain": {"layouts_per_s": len(jobs) / max(finish - jobs[0].arrival, 1e-9),
                             "p50_s": float(np.percentile(lat, 50)),
                             "p99_s": float(np.percentile(lat, 99)),
                             "busy_seconds": float(sum(service))},
            "clocks": clk}
    line["speedup_vs_serial_plain"] = line["value"] / line["serial_plain"]["layouts_per_s"]
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
    import forcegpu
    from forcegpu import Engine
    from forcegpu._lib import (Q_DEVICE_BYTES, Q_LAUNCHES, Q_WALK_APPLIES, Q_WALK_OPENS,
                               Q_WALK_RARE, Q_WALK_TESTS, Q_WALK_USEFUL, TUNE_WALK_GROUP,
                               desc_from_gpu)

    n = args.nodes
    xyz, src, dst, bias, strength = workload(n)
    pos4 = np.zeros((n, 4), np.float32)
    pos4[:, :3] = xyz
    eng = Engine(local)
    eng.set_nodes(pos4, 3)
    links = {"type": "link", "version": 1, "source": src, "target": dst, "iterations": 1,
             "strengths": strength, "distances": np.full(len(src), 30.0), "bias": bias}
    d_link, keep_l = desc_from_gpu(links, 1, n)
    charge = {"type": "manyBody", "version": 1, "strengths": np.full(n, -30.0), "distanceMin2": 1.0,
              "distanceMax2": math.inf, "theta2": 0.81}
    d_charge, keep_c = desc_from_gpu(charge, 2, n)
    d_center, keep_x = desc_from_gpu({"type": "center", "x": 0, "y": 0, "z": 0, "strength": 1.0}, 3, n)
    descs = [(d_link, keep_l), (d_charge, keep_c), (d_center, keep_x)]
    eng.set_forces(descs)
    eng.set_seed(12345)
    eng.set_tuning(TUNE_WALK_GROUP, args.walk_group)
    decay = 0.6
    tuning = None
    if not args.no_autotune:  # outside the timed region, from the same start
        tuning = eng.autotune(ticks=10, alpha=0.5, decay=decay)
    # ticks are queued in blocks of B, as an application queues a frame's or a batch's worth:
    # the engine runs a block it has seen before as one CUDA graph
    B = max(1, min(args.block, args.steps))
    warm = max(args.warmup, 2 * B)
    total = warm + args.steps
    al, _ = alphas(total + 2 * args.steps + B + 9)

    def run(first, count):
        k = first
        while k < first + count:
            c = min(B, first + count - k)
            eng.enqueue(al[k:k + c], decay)
            k += c

    stream = torch.cuda.ExternalStream(eng.stream(), device=local)
    run(0, warm)  # warm-up
    eng.idle()

    # timed region: K ticks, state resident, CUDA events on the engine's stream
    def barrier():
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    launches0 = eng.query(Q_LAUNCHES)
    clocks = Clocks()
    clocks.start()
    barrier()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    run(warm, args.steps)
    e1.record(stream)
    eng.idle()
    barrier()
    clk = clocks.stop()
    ms_total = e0.elapsed_time(e1)
    launches = eng.query(Q_LAUNCHES) - launches0
    # the per-kernel times: one more block, with the kernels timed one group at a time
    eng.profile(True)
    eng.enqueue(al[total:total + B], decay)
    eng.idle()
    prof = eng.profile_read()
    eng.profile(False)
    total += B
    if world > 1:
        t = torch.tensor([ms_total], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms_total = float(t.item())
    ms_tick = ms_total / args.steps
    value = ms_total / (args.steps * world)

    # the walk's counted work, from one more tick with the walk's counters on (outside the
    # timed region): FP32 operations per launch for the FP32-pipe view of the roofline
    eng.profile(2)
    eng.enqueue(al[total:total + 1], decay)
    eng.idle()
    walk_count = {k: eng.query(q) for k, q in (("tests", Q_WALK_TESTS), ("useful", Q_WALK_USEFUL),
                                              ("opens", Q_WALK_OPENS), ("applies", Q_WALK_APPLIES),
                                              ("rare_rounds", Q_WALK_RARE))}
    eng.profile(False)

    # e2e through the C ABI with pinned host buffers
    e2e = None
    if not args.no_e2e:
        hp = torch.empty((n, 3), dtype=torch.float32, pin_memory=True)
        hv = torch.empty((n, 3), dtype=torch.float32, pin_memory=True)
        eng.sync_packed_into(hp.data_ptr(), hv.data_ptr())
        hpn = hp.numpy()
        k = args.steps
        a2 = al[total + 1:total + 1 + k]
        barrier()
        t0 = time.perf_counter()
        for i in range(k):
            eng.update_positions_packed(0, hpn)
            eng.enqueue(a2[i:i + 1], decay)
            eng.sync_packed_into(hp.data_ptr(), hv.data_ptr())
        barrier()
        e2e_ms = (time.perf_counter() - t0) * 1e3 / k
        if world > 1:
            t = torch.tensor([e2e_ms], device="cuda")
            torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
            e2e_ms = float(t.item())
        e2e = {"value": e2e_ms / world, "unit": UNIT, "h2d_bytes_per_step": 12 * n + 8,
               "d2h_bytes_per_step": 24 * n,
               "calls": "fl_update_positions_packed + fl_enqueue + fl_sync_packed"}
        # the same through the float4 calls: the reference's vec4 layout, 16 B per node each way
        hp4 = torch.empty((n, 4), dtype=torch.float32, pin_memory=True)
        hv4 = torch.empty((n, 4), dtype=torch.float32, pin_memory=True)
        eng.sync_into(hp4.data_ptr(), hv4.data_ptr())
        hp4n = hp4.numpy()
        a3 = al[total + 1 + k:total + 1 + 2 * k]
        barrier()
        t0 = time.perf_counter()
        for i in range(k):
            eng.update_positions(0, hp4n)
            eng.enqueue(a3[i:i + 1], decay)
            eng.sync_into(hp4.data_ptr(), hv4.data_ptr())
        barrier()
        ms4 = (time.perf_counter() - t0) * 1e3 / k
        if world > 1:
            t = torch.tensor([ms4], device="cuda")
            torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
            ms4 = float(t.item())
        e2e_float4 = {"value": ms4 / world, "unit": UNIT, "h2d_bytes_per_step": 16 * n + 8,
                      "d2h_bytes_per_step": 32 * n, "calls": "fl_update_positions + fl_enqueue + fl_sync"}

    dev_bytes = eng.query(Q_DEVICE_BYTES)
    peaks, peak_kind = measured_peaks()
    walk_ms, walk_n = prof.get("walk", (0.0, 0))
    walk_avg = walk_ms / max(1, walk_n)
    walk_bytes = WALK_BYTES_PER_NODE * n
    achieved = walk_bytes / (walk_avg * 1e-3) / 1e9 if walk_avg else None
    roof = {"bound": "hbm", "kernel": "k_walk", "achieved": achieved, "peak": peaks["hbm_gbs"],
            "unit": "GB/s", "frac": (achieved / peaks["hbm_gbs"]) if achieved else None,
            "traffic": WALK_DRAM_BYTES_1M if n == 1_000_000 else None, "peak_kind": peak_kind,
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

    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": warm, "ms_per_step": ms_tick, "higher_is_better": False,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": "3D layout, %d nodes, %d links, link+charge(theta 0.9)+center, "
                                   "ticks %d-%d from the phyllotaxis start" % (n, len(src), warm + 1, warm + args.steps),
                       "tick_block": B, "tuning": tuning,
                       "nodes": n, "links": int(len(src)), "parallelism": "replicas" if world > 1 else "single",
                       "l2": "working set %.0f MB > 126 MB L2 (no flush)" % (dev_bytes / 1e6)},
            "gpu_launches": int(launches), "clocks": clk, "roofline": roof, "kernels": kernels}
    if e2e:
        line["e2e"] = e2e
        line["e2e_float4"] = e2e_float4
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        ms_cpu, t = cpu_baseline(xyz, src, dst, n)
        line["cpu_baseline"] = {"value": ms_cpu, "unit": UNIT, "cores": 1, "kind": "port",
                                "sample": "ticks 2-%d of the same 1M-node layout (oracle, FP64, one core)" % (1 + t),
                                "host_cores": os.cpu_count()}
    if rank == 0:
        print(json.dumps(line), flush=True)
    eng.close()
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
