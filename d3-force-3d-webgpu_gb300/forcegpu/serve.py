"""A layout server: jobs (graph + forces + tick count) arrive at any time and are laid out with
continuous batching on one GPU.

    srv = LayoutServer(hbm_budget=64 << 30)
    job = srv.submit(Job(xyz, source, target, ticks=300))
    srv.run_until_idle()          # or call srv.step() from your own loop
    job.result                    # (n, ndim) positions; job.latency in seconds

Scheduling:
  * Every job (link + many-body + centre forces, the reference benchmark's force set, and for
    some a collide force too) runs in a batch per dimensionality (fl_batch_*): every tick of a
    batch is one launch per kernel for all its graphs. A batch advances in blocks of `block`
    ticks; between blocks, finished jobs leave and waiting jobs join (the batch is rebuilt from
    the running jobs' current state), so a request that arrives while others are on the GPU
    starts at the next block boundary. A job whose tick count ends inside a block sits the rest
    of the block out (negative alpha).
  * With batching=False (the serial comparison), each job runs on its own plain engine (fl_sim).
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

from ._lib import TUNE_GRAPHS, Engine, desc_from_gpu
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
    """The batch of one dimensionality. Jobs join at block boundaries, appended to the running
    batch (fl_batch_add_graphs: the running jobs' state stays on the device). A job that
    finishes stays in the batch, sitting every tick out, until the finished jobs hold
    `dead_share` of the batch's nodes: then the batch is rebuilt from the running jobs' current
    state (read back) plus the new ones. Only a finished job's own nodes are read back when it
    ends.

    Blocks are pipelined: a job's alphas are known in advance, so the block after a block is
    queued before the first one has run (up to `depth` blocks in flight), and the host waits for
    the GPU only to read a finished job back or to change the batch."""

    def __init__(self, ndim, device, dead_share=0.5, depth=2):
        self.ndim = ndim
        self.batch = Batch(device)
        self.jobs = []       # in the batch, in its order (finished ones included until a rebuild)
        self.incoming = []   # admitted, waiting for the next block boundary
        self.dead = 0        # nodes of finished jobs still in the batch
        self.dead_share = dead_share
        self.depth = depth
        self.pending = deque()  # per block in flight: the (graph, job) pairs that end in it

    def live(self):
        return [j for j in self.jobs if j.done_ticks < j.ticks]

    def busy(self):
        return bool(self.incoming or self.pending) or any(j.done_ticks < j.ticks for j in self.jobs)

    def spec(self, j):
        return GraphSpec(xyz=j.pos[:, :self.ndim], source=j.source, target=j.target,
                         theta=j.theta, velocity_decay=j.velocity_decay,
                         vel=j.vel[:, :self.ndim] if j.vel is not None else None,
                         tick0=j.done_ticks, radii=j.radii)

    def _rebuild(self, seed):
        live = self.live()
        if live:  # the running jobs' state, from the device
            pos, vel = self.batch.sync()
            cuts = np.cumsum([j.n for j in self.jobs])[:-1]
            for j, p, v in zip(self.jobs, np.split(pos, cuts), np.split(vel, cuts)):
                if j.done_ticks < j.ticks:
                    j.pos, j.vel = p[:, :3].astype(np.float64), v[:, :3].astype(np.float64)
        self.jobs = live + self.incoming
        self.incoming = []
        self.dead = 0
        if self.jobs:
            self.batch.set_graphs([self.spec(j) for j in self.jobs], ndim=self.ndim, seed=seed)

    def launch(self, block, seed, now):
        """Queue the next block (changing the batch first if jobs join or the finished ones are
        many); returns the jobs whose results were read back on the way."""
        done = []
        total = sum(j.n for j in self.jobs)
        compact = self.jobs and self.dead > self.dead_share * total
        if compact or self.incoming:
            done = self.land(now, drain=True)  # every result out before the batch changes
            if compact or not self.live():
                self._rebuild(seed)  # compact, or start afresh
            else:  # join the running batch
                self.batch.add_graphs([self.spec(j) for j in self.incoming])
                self.jobs += self.incoming
                self.incoming = []
        if len(self.pending) >= self.depth or not any(j.done_ticks < j.ticks for j in self.jobs):
            return done
        al = np.stack([j.next_alphas(block) for j in self.jobs], axis=1)
        ended = []
        for g, (j, col) in enumerate(zip(self.jobs, al.T)):  # the jobs' schedules move on now
            ran = int((col >= 0).sum())
            if not ran:
                continue
            j.alpha = float(col[ran - 1])
            j.done_ticks += ran
            if j.done_ticks >= j.ticks:
                ended.append((g, j))
        self.batch.enqueue(al)
        self.pending.append(ended)
        return done

    def land(self, now, drain=False):
        """Read back the jobs that ended in the oldest blocks in flight (waiting for them), as
        many blocks as hold a finished job or exceed the pipeline's depth (all with drain);
        returns those jobs. A finished job sits later blocks out, so its state is still its
        result when read after them."""
        done = []
        while self.pending and (drain or self.pending[0] or len(self.pending) >= self.depth):
            ended = self.pending.popleft()
            if not ended:
                self.batch.wait()
            for g, j in ended:
                p, _ = self.batch.read(g, 1)
                j.result = p[:, :self.ndim].copy()
                j.finished = now()
                j.pos = j.vel = None
                self.dead += j.n
                done.append(j)
        return done


class LayoutServer:
    def __init__(self, device=0, hbm_budget=64 << 30, block=50, seed=12345, clock=time.perf_counter,
                 batching=True, plain_graphs=False):
        self.device = device
        self.batching = batching  # False: every job on its own plain engine
        self.hbm_budget = hbm_budget
        self.block = block
        self.seed = seed
        self.now = clock
        self.queue = deque()
        # the batches of 2D and 3D jobs exist from the start (creating one loads its kernels)
        self.lanes = {d: _Lane(d, device) for d in (2, 3)} if batching else {}
        self.plain = []  # (job, engine, descs): each job on its own plain engine (batching off)
        # finished plain engines: freeing device memory waits for the whole device, so they are
        # closed when nothing else is in flight (or at close())
        self.retired = []
        # a plain job runs a few blocks only: capturing each as a CUDA graph costs more than
        # the launches it saves
        self.plain_graphs = plain_graphs
        self.used = 0
        self.finished = []
        self._ids = 0

    def warmup(self):
        """Lay out two tiny jobs per dimensionality, with and without collide, outside any
        measurement: the first launch of each kernel in a process loads it, which a server pays
        once at start-up, not per request."""
        from .graphs import benchmark_links, phyllotaxis
        jobs = []
        for dims in (2, 3):
            for radii in (None, np.full(300, 2.0)):
                src, dst = benchmark_links(300, 150, seed=1)
                jobs.append(Job(xyz=phyllotaxis(300, dims)[:, :dims], source=src, target=dst,
                                ticks=2 * self.block, radii=radii, arrival=self.now()))
        for j in jobs:
            self.submit(j)
        self.run_until_idle()
        mine = {id(j) for j in jobs}
        self.finished = [j for j in self.finished if id(j) not in mine]
        self._ids = 0
        return self

    # --- requests ---
    def submit(self, job):
        job.id = self._ids
        self._ids += 1
        if job.arrival is None:
            job.arrival = self.now()
        self.queue.append(job)
        return job

    def busy(self):
        return bool(self.queue or self.plain or any(l.busy() for l in self.lanes.values()))

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
            if not self.batching:
                self._start_plain(j)
            else:
                lane = self.lanes.get(j.ndim)
                if lane is None:
                    lane = self.lanes[j.ndim] = _Lane(j.ndim, self.device)
                lane.incoming.append(j)

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
        if not self.plain_graphs:
            eng.set_tuning(TUNE_GRAPHS, 0)
        self.plain.append((j, eng, descs))

    def step(self):
        """One round: admit; launch a block on every batch and queue the next block of ticks of
        every plain job (a block at a time, so that no queue of thousands of launches holds the
        host while the batches wait); land the finished plain jobs and the batches' blocks.
        Returns the jobs finished in this round."""
        self._admit()
        # the plain jobs' blocks first: the GPU runs them while the host rebuilds a batch
        for j, eng, _ in self.plain:
            k = min(self.block, j.ticks - j.done_ticks)
            if k > 0:
                al = j.next_alphas(k)
                eng.enqueue(al, 1 - j.velocity_decay)
                j.alpha = float(al[-1])
                j.done_ticks += k
        landed = []
        for lane in self.lanes.values():
            landed += lane.launch(self.block, self.seed, self.now)
        done = []
        still = []
        for j, eng, descs in self.plain:
            if j.done_ticks < j.ticks or eng.busy():
                still.append((j, eng, descs))
                continue
            pos, _ = eng.sync()
            self.retired.append(eng)
            j.result = pos[:, :j.ndim].copy()
            j.finished = self.now()
            done.append(j)
        self.plain = still
        done += landed
        for lane in self.lanes.values():
            done += lane.land(self.now)
        for j in done:
            self.used -= j.footprint
        self.finished += done
        lanes_busy = any(l.busy() for l in self.lanes.values())
        if self.retired and not lanes_busy and not self.plain:
            for eng in self.retired:
                eng.close()
            self.retired = []
        if not done and not lanes_busy and self.plain == [] and self.queue:
            # nothing running: wait for the next arrival
            wait = self.queue[0].arrival - self.now()
            if wait > 0:
                time.sleep(min(wait, 0.05))
        elif not lanes_busy and self.plain and all(j.done_ticks >= j.ticks for j, _, _ in self.plain):
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
        for eng in self.retired:
            eng.close()
        self.lanes, self.plain, self.retired = {}, [], []


def latency_summary(jobs):
    lat = np.array([j.latency for j in jobs if j.latency is not None])
    if not len(lat):
        return {}
    return {"p50_s": float(np.percentile(lat, 50)), "p99_s": float(np.percentile(lat, 99)),
            "mean_s": float(lat.mean()), "max_s": float(lat.max()), "jobs": int(len(lat))}
