"""Batches: many independent force layouts advanced together on one GPU (fl_batch_*).

    from forcegpu.batch import Batch, GraphSpec
    b = Batch()
    b.set_graphs([GraphSpec(xyz, source, target), ...], ndim=3)
    b.run(300)                 # each graph's own alpha schedule (d3 defaults), 300 ticks
    positions = b.positions()  # one (n_g, ndim) array per graph

Each graph has a link force, a many-body force, optionally a collide force (after the
many-body force) and optionally a centre force, as the reference's benchmark layout and the
served jobs; its parameters follow d3's defaults unless given. The alpha
schedule of every graph is d3's (src/simulation.js:28-32, :49-56), advanced on the host; a
graph's own alphaDecay / alphaMin / alphaTarget may differ from the others'.
"""
from __future__ import annotations

import ctypes
import math
import os
from dataclasses import dataclass, field

import numpy as np

from ._lib import FL_OK, FlError, GraphDesc, Q_DEVICE_BYTES, Q_LAUNCHES, TuneResult, load


@dataclass
class GraphSpec:
    """One graph of a batch. xyz: (n, ndim) start positions; source / target: link ends (node
    indices within the graph). None means d3's default for that parameter."""
    xyz: np.ndarray
    source: np.ndarray = None
    target: np.ndarray = None
    link_distance: np.ndarray = None
    link_strength: np.ndarray = None
    link_bias: np.ndarray = None
    charge: np.ndarray = None
    theta: float = 0.9
    distance_min: float = 1.0
    distance_max: float = math.inf
    center: tuple = (0.0, 0.0, 0.0)
    center_strength: float = 1.0
    velocity_decay: float = 0.4
    alpha: float = 1.0
    alpha_min: float = 0.001
    alpha_decay: float = 1 - 0.001 ** (1 / 300)
    alpha_target: float = 0.0
    vel: np.ndarray = None
    tick0: int = 0  # ticks the layout ran before (a job moved between batches keeps its count)
    radii: np.ndarray = None  # collide radii (None: no collide force)
    collide_strength: float = 1.0
    collide_iterations: int = 1
    _keep: list = field(default_factory=list, repr=False)


class Batch:
    """An fl_batch: the device state of many graphs, concatenated."""

    def __init__(self, device=0):
        self.L = load()
        h = ctypes.c_void_p()
        rc = self.L.fl_batch_create(int(device), ctypes.byref(h))
        if rc != FL_OK:
            raise FlError(rc, "fl_batch_create failed on device %d" % device)
        self.h = h
        self.specs = []
        self.sizes = np.zeros(0, np.int64)
        self.ndim = 3

    def _check(self, rc):
        if rc != FL_OK:
            msg = self.L.fl_batch_last_error(self.h)
            raise FlError(rc, msg.decode() if msg else "")

    def close(self):
        if getattr(self, "h", None):
            self.L.fl_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _descs(self, specs):
        descs = (GraphDesc * max(1, len(specs)))()
        for i, s in enumerate(specs):
            xyz = np.asarray(s.xyz, dtype=np.float64).reshape(-1, self.ndim)
            n = len(xyz)
            pos4 = np.zeros((n, 4), np.float32)
            pos4[:, :self.ndim] = xyz
            keep = [pos4]
            d = descs[i]
            d.n, d.pos4 = n, pos4.ctypes.data
            if s.vel is not None:
                vel4 = np.zeros((n, 4), np.float32)
                vel4[:, :self.ndim] = np.asarray(s.vel).reshape(n, -1)[:, :self.ndim]
                keep.append(vel4)
                d.vel4 = vel4.ctypes.data
            src = np.ascontiguousarray(s.source if s.source is not None else [], dtype=np.int32)
            dst = np.ascontiguousarray(s.target if s.target is not None else [], dtype=np.int32)
            d.m = len(src)
            d.source, d.target = src.ctypes.data, dst.ctypes.data
            keep += [src, dst]
            for name in ("link_distance", "link_strength", "link_bias", "charge"):
                v = getattr(s, name)
                if v is not None:
                    a = np.ascontiguousarray(np.broadcast_to(v, (d.m if name != "charge" else n,)),
                                             dtype=np.float32)
                    keep.append(a)
                    setattr(d, name, a.ctypes.data)
            d.theta2 = s.theta * s.theta
            d.distance_min2 = s.distance_min * s.distance_min
            d.distance_max2 = s.distance_max * s.distance_max
            d.center_x, d.center_y, d.center_z = (list(s.center) + [0.0, 0.0, 0.0])[:3]
            d.center_strength = s.center_strength
            d.velocity_decay = s.velocity_decay
            d.tick0 = int(s.tick0) & 0xffffffff
            if s.radii is not None:
                r = np.ascontiguousarray(np.broadcast_to(s.radii, (n,)), dtype=np.float32)
                keep.append(r)
                d.radii = r.ctypes.data
                d.collide_strength = float(s.collide_strength)
                d.collide_iterations = int(s.collide_iterations)
            s._keep = keep
        return descs

    def set_graphs(self, specs, ndim=3, seed=None):
        self.specs = list(specs)
        self.ndim = int(ndim)
        descs = self._descs(self.specs)
        self._check(self.L.fl_batch_set_graphs(self.h, self.ndim, len(self.specs), descs))
        if seed is not None:
            self._check(self.L.fl_batch_set_seed(self.h, int(seed) & 0xffffffff))
        self.sizes = np.array([len(np.asarray(s.xyz).reshape(-1, self.ndim)) for s in self.specs], np.int64)
        self.alphas = np.array([s.alpha for s in self.specs], dtype=np.float64)

    def add_graphs(self, specs):
        """Append graphs to the running batch (fl_batch_add_graphs): the present graphs and their
        state stay as they are; each new graph's alpha starts from its spec."""
        specs = list(specs)
        if not specs:
            return
        descs = self._descs(specs)
        self._check(self.L.fl_batch_add_graphs(self.h, len(specs), descs))
        self.specs += specs
        self.sizes = np.concatenate([self.sizes, [len(np.asarray(s.xyz).reshape(-1, self.ndim))
                                                  for s in specs]]).astype(np.int64)
        self.alphas = np.concatenate([self.alphas, [s.alpha for s in specs]])

    def alpha_schedule(self, ticks):
        """The next `ticks` alphas of every graph, (ticks, graphs), advancing each graph's alpha
        as d3 does (src/simulation.js:49-56)."""
        out = np.empty((ticks, len(self.specs)))
        decay = np.array([s.alpha_decay for s in self.specs])
        target = np.array([s.alpha_target for s in self.specs])
        a = self.alphas
        for k in range(ticks):
            a = a + (target - a) * decay
            out[k] = a
        self.alphas = a
        return out

    def enqueue(self, alphas):
        a = np.ascontiguousarray(alphas, dtype=np.float64).reshape(-1, len(self.specs))
        self._check(self.L.fl_batch_enqueue(self.h, a.ctypes.data, len(a)))

    def run(self, ticks):
        self.enqueue(self.alpha_schedule(ticks))
        return self

    def sync(self):
        n = int(self.sizes.sum())
        pos = np.empty((max(n, 1), 4), np.float32)
        vel = np.empty((max(n, 1), 4), np.float32)
        self._check(self.L.fl_batch_sync(self.h, pos.ctypes.data, vel.ctypes.data))
        return pos[:n], vel[:n]

    def read(self, first, count=1):
        """Wait, then the positions and velocities of graphs [first, first + count), float32
        (n, 4) each (fl_batch_read: only those graphs' nodes cross to the host)."""
        n = int(self.sizes[first:first + count].sum())
        pos = np.empty((max(n, 1), 4), np.float32)
        vel = np.empty((max(n, 1), 4), np.float32)
        self._check(self.L.fl_batch_read(self.h, int(first), int(count), pos.ctypes.data,
                                         vel.ctypes.data))
        return pos[:n], vel[:n]

    def wait(self):
        """Wait for the queued ticks (and report a device-side error), reading nothing back."""
        self._check(self.L.fl_batch_sync(self.h, None, None))

    def positions(self):
        """Wait, then each graph's positions, (n_g, ndim)."""
        pos, _ = self.sync()
        cuts = np.cumsum(self.sizes)[:-1]
        return [p[:, :self.ndim] for p in np.split(pos, cuts)]

    def query(self, what):
        out = ctypes.c_int64()
        self._check(self.L.fl_batch_query(self.h, int(what), ctypes.byref(out)))
        return out.value

    def launches(self):
        return self.query(Q_LAUNCHES)

    def device_bytes(self):
        return self.query(Q_DEVICE_BYTES)

    def set_tuning(self, key, value):
        self._check(self.L.fl_batch_set_tuning(self.h, int(key), int(value)))

    def autotune(self, ticks=5, alpha=0.5, cache=None):
        """fl_batch_autotune: the fastest sort passes and walk grid for this batch, state kept."""
        out = TuneResult()
        c = None if cache is None else os.fsencode(cache)
        self._check(self.L.fl_batch_autotune(self.h, int(ticks), float(alpha), c, ctypes.byref(out)))
        return out.as_dict()

    def stream(self):
        out = ctypes.c_void_p()
        self._check(self.L.fl_batch_stream(self.h, ctypes.byref(out)))
        return out.value
