"""A layout server: jobs (graph + forces + tick count) arrive at any time and are laid out with
continuous batching on one GPU.

    srv = LayoutServer(hbm_budget=64 << 30)
    job = srv.submit(Job(xyz, source, target, ticks=300))
    srv.run_until_idle()          # or call srv.step() from your own loop
    job.result                    # (n, ndim) positions; job.latency in seconds

Scheduling:
  * Jobs with link + many-body + centre forces (the reference benchmark's force set) run in a
    batch per dimensionality (fl_batch_*): every tick of a batch is one launch per kernel for
    all its graphs. A batch advances in blocks of `block` ticks; between blocks, finished jobs
    leave and waiting jobs join (the batch is rebuilt from the running jobs' current state), so
    a request that arrives while others are on the GPU starts at the next block boundary. A job
    whose tick count ends inside a block sits the rest of the block out (negative alpha).
  * Jobs that also have a collide force run on their own plain engine (fl_sim), each on its own
    CUDA stream, overlapping with the batches and with each other on the device.
  * Admission by device-memory footprint: a job is admitted when the footprints of the running
    jobs plus its own fit `hbm_budget`; jobs are admitted in arrival order.

A job's result does not depend on the other jobs: a graph in a batch is laid out exactly as it
would be alone (its own cube, tree, alpha schedule), up to the order of some float sums.
"""
from __future__ import annotations

import math
import time
from collections import deque
from dataclasses import dataclass, field

import numpy as np

from ._lib import Engine, desc_from_gpu
from .batch import Batch, GraphSpec
from .graphs import link_defaults

# device bytes per node and per link of a job (tree, sort and state buffers, CSR), with margin
BYTES_PER_NODE = 420
BYTES_PER_LINK = 48


@dataclass
class Job:
    """A layout request. xyz: (n, ndim) start positions; source / target: links; radii: collide
    radii (None: no collide force); ticks: how many ticks to run (d3's alpha schedule)."""
    xyz: np.ndarray
    source: np.ndarray
    target: np.ndarray
    ticks: int = 300
    radii: np.ndarray = None
    theta: float = 0.9
    velocity_decay: float = 0.4
    arrival: float = None
    # filled in by the server
    id: int = -1
    admitted: float = None
    finished: float = None
    result: np.ndarray = None
    done_ticks: int = 0
    alpha: float = 1.0
    pos: np.ndarray = field(default=None, repr=False)
    vel: np.ndarray = field(default=None, repr=False)

    @property
    def n(self):
        return len(self.xyz)

    @property
    def ndim(self):
        return self.xyz.shape[1]

    @property
    def footprint(self):
        return BYTES_PER_NODE * self.n + BYTES_PER_LINK * len(self.source) + (1 << 20)

    @property
    def latency(self):
        return None if self.finished is None else self.finished - self.arrival

    def next_alphas(self, k):
        """The next k alphas of d3's schedule (src/simulation.js:49-56); -1 once done."""
        decay = 1 - 0.001 ** (1 / 300)
        out = np.full(k, -1.0)
        a = self.alpha
        for i in range(min(k, self.ticks - self.done_ticks)):
            a += (0.0 - a) * decay
            out[i] = a
        return out


class _Lane:
    """The batch of one dimensionality: running jobs, rebuilt between blocks."""

    def __init__(self, ndim, device):
        self.ndim = ndim
        self.batch = Batch(device)
        self.jobs = []
        self.dirty = False
        self.pending = None  # alphas of the block in flight

    def spec(self, j):
        return GraphSpec(xyz=j.pos[:, :self.ndim], source=j.source, target=j.target,
                         theta=j.theta, velocity_decay=j.velocity_decay,
                         vel=j.vel[:, :self.ndim] if j.vel is not None else None)

    def launch(self, block, seed):
        if not self.jobs:
            return
        if self.dirty:
            self.batch.set_graphs([self.spec(j) for j in self.jobs], ndim=self.ndim, seed=seed)
            self.dirty = False
        al = np.stack([j.next_alphas(block) for j in self.jobs], axis=1)
        self.batch.enqueue(al)
        self.pending = al

    def land(self, now):
        """Wait for the block, update the jobs; returns the finished ones."""
        if self.pending is None:
            return []
        pos, vel = self.batch.sync()
        cuts = np.cumsum([j.n for j in self.jobs])[:-1]
        done = []
        for j, p, v, col in zip(self.jobs, np.split(pos, cuts), np.split(vel, cuts), self.pending.T):
            ran = int((col >= 0).sum())
            j.pos, j.vel = p[:, :3].astype(np.float64), v[:, :3].astype(np.float64)
            if ran:
                j.alpha = float(col[ran - 1])
            j.done_ticks += ran
            if j.done_ticks >= j.ticks:
                j.result = p[:, :self.ndim].copy()
                j.finished = now()
                done.append(j)
        self.pending = None
        if done:
            self.jobs = [j for j in self.jobs if j.done_ticks < j.ticks]
            self.dirty = True
        return done


class LayoutServer:
    def __init__(self, device=0, hbm_budget=64 << 30, block=50, seed=12345, clock=time.perf_counter,
                 batching=True):
        self.device = device
        self.batching = batching  # False: every job on its own plain engine
        self.hbm_budget = hbm_budget
        self.block = block
        self.seed = seed
        self.now = clock
        self.queue = deque()
        self.lanes = {}
        self.plain = []  # (job, engine) with a collide force
        self.used = 0
        self.finished = []
        self._ids = 0

    # --- requests ---
    def submit(self, job):
        job.id = self._ids
        self._ids += 1
        if job.arrival is None:
            job.arrival = self.now()
        self.queue.append(job)
        return job

    def busy(self):
        return bool(self.queue or self.plain or any(l.jobs for l in self.lanes.values()))

    # --- scheduling ---
    def _admit(self):
        while self.queue and self.queue[0].arrival <= self.now():
            j = self.queue[0]
            if self.used + j.footprint > self.hbm_budget and self.used > 0:
                break  # wait for memory to free up (a job larger than the budget runs alone)
            self.queue.popleft()
            self.used += j.footprint
            j.admitted = self.now()
            j.pos = np.zeros((j.n, 3))
            j.pos[:, :j.ndim] = j.xyz
            if j.radii is not None or not self.batching:
                self._start_plain(j)
            else:
                lane = self.lanes.get(j.ndim)
                if lane is None:
                    lane = self.lanes[j.ndim] = _Lane(j.ndim, self.device)
                lane.jobs.append(j)
                lane.dirty = True

    def _start_plain(self, j):
        n = j.n
        eng = Engine(self.device)
        pos4 = np.zeros((n, 4), np.float32)
        pos4[:, :j.ndim] = j.xyz
        eng.set_nodes(pos4, j.ndim)
        bias, strength = link_defaults(n, j.source, j.target)
        descs = [
            desc_from_gpu({"type": "link", "version": 1, "source": j.source, "target": j.target,
                           "iterations": 1, "strengths": strength,
                           "distances": np.full(len(j.source), 30.0), "bias": bias}, 1, n),
            desc_from_gpu({"type": "manyBody", "version": 1, "strengths": np.full(n, -30.0),
                           "distanceMin2": 1.0, "distanceMax2": math.inf,
                           "theta2": j.theta * j.theta}, 2, n),
            desc_from_gpu({"type": "center", "x": 0, "y": 0, "z": 0, "strength": 1.0}, 4, n),
        ]
        if j.radii is not None:
            descs.insert(2, desc_from_gpu({"type": "collide", "version": 1,
                                           "radii": np.asarray(j.radii, float), "strength": 1.0,
                                           "iterations": 1}, 3, n))
        eng.set_forces(descs)
        eng.set_seed(self.seed)
        self.plain.append((j, eng, descs))

    def step(self):
        """One round: admit; launch a block on every batch and queue the next block of ticks of
        every plain job (a block at a time, so that no queue of thousands of launches holds the
        host while the batches wait); land the finished plain jobs and the batches' blocks.
        Returns the jobs finished in this round."""
        self._admit()
        for lane in self.lanes.values():
            lane.launch(self.block, self.seed)
        for j, eng, _ in self.plain:
            k = min(self.block, j.ticks - j.done_ticks)
            if k > 0:
                al = j.next_alphas(k)
                eng.enqueue(al, 1 - j.velocity_decay)
                j.alpha = float(al[-1])
                j.done_ticks += k
        done = []
        still = []
        for j, eng, descs in self.plain:
            if j.done_ticks < j.ticks or eng.busy():
                still.append((j, eng, descs))
                continue
            pos, _ = eng.sync()
            eng.close()
            j.result = pos[:, :j.ndim].copy()
            j.finished = self.now()
            done.append(j)
        self.plain = still
        for lane in self.lanes.values():
            done += lane.land(self.now)
        for j in done:
            self.used -= j.footprint
        self.finished += done
        if not done and not any(l.jobs for l in self.lanes.values()) and self.plain == [] and self.queue:
            # nothing running: wait for the next arrival
            wait = self.queue[0].arrival - self.now()
            if wait > 0:
                time.sleep(min(wait, 0.05))
        elif not any(l.jobs for l in self.lanes.values()) and self.plain and \
                all(j.done_ticks >= j.ticks for j, _, _ in self.plain):
            time.sleep(0.0005)  # only queued plain work left: poll gently
        return done

    def run_until_idle(self):
        while self.busy():
            self.step()
        return self.finished

    def close(self):
        for lane in self.lanes.values():
            lane.batch.close()
        for _, eng, _ in self.plain:
            eng.close()
        self.lanes, self.plain = {}, []


def latency_summary(jobs):
    lat = np.array([j.latency for j in jobs if j.latency is not None])
    if not len(lat):
        return {}
    return {"p50_s": float(np.percentile(lat, 50)), "p99_s": float(np.percentile(lat, 99)),
            "mean_s": float(lat.mean()), "max_s": float(lat.max()), "jobs": int(len(lat))}
