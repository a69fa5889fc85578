"""forceSimulationGPU: the reference's simulation object over the GB300 engine.

Mirrors src/gpu/simulation.js (the facade) and the host half of src/gpu/engine.js (the node
mirror: upload, edit detection, readback and landing), with libforcegpu.so in place of WebGPU.
Method names are the reference's (camelCase), so code written against it reads the same; the
Promise-returning methods (tickAsync, sync, gpuReady) are coroutines.

Differences from the reference, all deliberate:
  * No CPU path. The reference runs on the CPU when WebGPU or a force's gpu() is missing
    (src/gpu/simulation.js:110-139, :279-289); here that is an error (FlError), raised at the
    first call that needs the engine. Consequently `cpuTicks` (CPU warm-up ticks) is accepted
    and ignored: every tick runs on the GPU, as the reference does with cpuTicks 0.
  * tick() queues work and returns; the nodes are brought up to date by sync(), tickAsync() or
    the timer's own ticks (the reference lands them from an asynchronous readback).
"""
from __future__ import annotations

import math
import threading
import time

import numpy as np

from ._lib import Engine, FlError, FL_E_DEVICE, FL_E_UNSUPPORTED, desc_from_gpu

MAX_DIMENSIONS = 3
INITIAL_RADIUS = 10
INITIAL_ANGLE_ROLL = math.pi * (3 - math.sqrt(5))          # src/simulation.js:19-21
INITIAL_ANGLE_YAW = math.pi * 20 / (9 + math.sqrt(221))

_UNSET = object()

# the keys of forceSimulation (test/simulation-test.js:5-8) and the GPU additions
# (test/gpu-simulation-test.js:9)
SIMULATION_KEYS = ["alpha", "alphaDecay", "alphaMin", "alphaTarget", "find", "force", "nodes",
                   "numDimensions", "on", "randomSource", "restart", "stop", "tick", "velocityDecay"]
GPU_KEYS = ["destroy", "gpuBuffers", "gpuReady", "isGPUEnabled", "sync", "tickAsync"]


def lcg():
    """src/lcg.js: the simulation's default random source, seeded with 1."""
    state = [1]

    def random():
        state[0] = (1664525 * state[0] + 1013904223) % 4294967296
        return state[0] / 4294967296

    return random


def _num(v):
    """src/gpu/engine.js:61-63: undefined / NaN -> 0."""
    if v is None:
        return 0.0
    try:
        v = float(v)
    except (TypeError, ValueError):
        return 0.0
    return 0.0 if v != v else v


def _nan(v):
    return v is None or (isinstance(v, float) and math.isnan(v))


class _NodeMirror:
    """The host half of src/gpu/engine.js: what the GPU was last told / told us about every
    node (exact doubles), so that user edits are found and never overwritten by a readback."""

    def __init__(self, device):
        self.eng = Engine(device)
        self.nodes = []
        self.n = 0
        self.nDim = 2
        self.plan = []
        self.enqueued = 0
        self.landed = 0
        self.stale = False
        self.shadow = np.zeros((0, 3))
        self.pinned = np.zeros(0, np.uint8)
        self.pinnedAt = np.zeros((0, 3))

    # --- JS -> GPU (src/gpu/engine.js:115-194) ---
    def _read(self, a, b):
        nd = self.nDim
        pos = np.zeros((b - a, 4), np.float64)
        fix = np.zeros((b - a, 4), np.float64)
        mask = np.zeros(b - a, np.uint8)
        for k, node in enumerate(self.nodes[a:b]):
            pos[k, 0] = _num(node.get("x"))
            if nd > 1:
                pos[k, 1] = _num(node.get("y"))
            if nd > 2:
                pos[k, 2] = _num(node.get("z"))
            m = 0
            if node.get("fx") is not None:
                m |= 1
                fix[k, 0] = float(node["fx"])
            if nd > 1 and node.get("fy") is not None:
                m |= 2
                fix[k, 1] = float(node["fy"])
            if nd > 2 and node.get("fz") is not None:
                m |= 4
                fix[k, 2] = float(node["fz"])
            mask[k] = m
        return pos, fix, mask

    def _read_vel(self):
        nd = self.nDim
        vel = np.zeros((self.n, 4), np.float64)
        for k, node in enumerate(self.nodes):
            vel[k, 0] = _num(node.get("vx"))
            if nd > 1:
                vel[k, 1] = _num(node.get("vy"))
            if nd > 2:
                vel[k, 2] = _num(node.get("vz"))
        return vel

    def upload_all(self, first=False):
        n = self.n
        pos, fix, mask = self._read(0, n)
        vel = self._read_vel()
        self.shadow = pos[:, :3].copy()
        self.pinned = mask.copy()
        self.pinnedAt = fix[:, :3].copy()
        if first:
            self.eng.set_nodes(pos, self.nDim, vel, fix, mask)
        elif n:
            self.eng.update_positions_packed(0, pos[:, :self.nDim])
            self.eng.update_velocities(0, vel)
            self.eng.update_pins(0, fix, mask)
        self.stale = False
        self.landed = self.enqueued

    def sync_from_nodes(self):
        if not self.n:
            return
        pos, fix, mask = self._read(0, self.n)
        pos_dirty = np.any(pos[:, :3] != self.shadow, axis=1)
        pin_dirty = (mask != self.pinned) | np.any((fix[:, :3] != self.pinnedAt) &
                                                  (((mask[:, None] >> np.arange(3)) & 1) == 1), axis=1)
        for dirty, upload in ((pos_dirty, "pos"), (pin_dirty, "pin")):
            idx = np.flatnonzero(dirty)
            if not len(idx):
                continue
            # runs of consecutive dirty nodes, one upload each
            breaks = np.flatnonzero(np.diff(idx) != 1)
            starts = np.concatenate([[idx[0]], idx[breaks + 1]])
            ends = np.concatenate([idx[breaks], [idx[-1]]]) + 1
            for a, b in zip(starts, ends):
                if upload == "pos":
                    self.shadow[a:b] = pos[a:b, :3]
                    self.eng.update_positions_packed(int(a), pos[a:b, :self.nDim])
                else:
                    self.pinned[a:b] = mask[a:b]
                    self.pinnedAt[a:b] = fix[a:b, :3]
                    self.eng.update_pins(int(a), fix[a:b], mask[a:b])

    # --- GPU -> JS (src/gpu/engine.js:198-239) ---
    def land(self, pos, vel):
        nd = self.nDim
        for i, node in enumerate(self.nodes):
            x = _num(node.get("x"))
            y = _num(node.get("y")) if nd > 1 else 0.0
            z = _num(node.get("z")) if nd > 2 else 0.0
            s = self.shadow[i]
            if x == s[0] and y == s[1] and z == s[2]:  # untouched since the last exchange
                node["x"] = s[0] = float(pos[i, 0])
                if nd > 1:
                    node["y"] = s[1] = float(pos[i, 1])
                if nd > 2:
                    node["z"] = s[2] = float(pos[i, 2])
            node["vx"] = float(vel[i, 0])
            if nd > 1:
                node["vy"] = float(vel[i, 1])
            if nd > 2:
                node["vz"] = float(vel[i, 2])

    # --- engine calls ---
    def set_nodes(self, nodes, nDim):
        self.nodes, self.n, self.nDim = nodes, len(nodes), nDim
        self.enqueued = self.landed = 0
        self.plan = []
        self.upload_all(first=True)

    def set_forces(self, forces):
        descs = []
        for f in forces:
            if not callable(getattr(f, "gpu", None)):
                raise FlError(FL_E_UNSUPPORTED, "force %r has no gpu() description" % (f,))
            descs.append(desc_from_gpu(f.gpu() or {"type": None}, id(f), self.n))
        self.eng.set_forces(descs)
        self.plan = list(forces)

    def enqueue(self, alphas, decay):
        if not self.n:
            return
        if self.stale:
            self.upload_all()
        else:
            self.sync_from_nodes()
        self.set_forces(self.plan)  # re-reads scalars; arrays only on a version change
        self.eng.enqueue(alphas, decay)
        self.enqueued += len(alphas)

    def sync(self):
        if not self.n or self.landed == self.enqueued:
            self.eng.idle()
            return
        pos, vel = self.eng.sync_packed()  # nDim floats per node across the host link
        self.land(pos, vel)
        self.landed = self.enqueued

    def destroy(self):
        self.eng.close()
        self.nodes = []


class Simulation:
    """The object forceSimulationGPU returns (src/gpu/simulation.js:295-428)."""

    def __init__(self, nodes=None, numDimensions=None, options=None):
        options = dict(options or {})
        self._options = options
        self._readback = options.get("readback", True) is not False
        self._device = int(options.get("device") or 0)
        self._nDim = min(MAX_DIMENSIONS, max(1, int(round(numDimensions or 2))))
        self._alpha = 1.0
        self._alphaMin = 0.001
        self._alphaDecay = 1 - math.pow(self._alphaMin, 1 / 300)
        self._alphaTarget = 0.0
        self._velocityDecay = 0.6
        self._forces = {}
        self._random = lcg()
        self._events = {"tick": {}, "end": {}}
        self._nodes = nodes if nodes is not None else []
        self._engine = None
        self._error = None
        self._usable = False
        self._seeded = False
        self._destroyed = False
        self._lock = threading.RLock()
        self._running = True
        self._timer = None
        self._initialize_nodes()
        self._init()
        self._start_timer()

    # --- setup ---
    def _init(self):
        try:
            self._engine = _NodeMirror(self._device)
            self._reset()
        except FlError as e:
            self._engine, self._error, self._usable = None, e, False

    def _reset(self):
        if not self._engine:
            return
        if not self._engine.eng.fits(len(self._nodes)):
            raise FlError(FL_E_DEVICE, "%d nodes exceed this GPU's memory" % len(self._nodes))
        self._engine.set_nodes(self._nodes, self._nDim)
        self._refresh()

    def _refresh(self):
        if not self._engine:
            return
        self._engine.set_forces(list(self._forces.values()))
        self._usable = True

    def _initialize_nodes(self):
        """src/simulation.js:79-107 (phyllotaxis start for nodes without a position)."""
        nd = self._nDim
        for i, node in enumerate(self._nodes):
            node["index"] = i
            if node.get("fx") is not None:
                node["x"] = node["fx"]
            if node.get("fy") is not None:
                node["y"] = node["fy"]
            if node.get("fz") is not None:
                node["z"] = node["fz"]
            if _nan(node.get("x")) or (nd > 1 and _nan(node.get("y"))) or (nd > 2 and _nan(node.get("z"))):
                radius = INITIAL_RADIUS * (math.cbrt(0.5 + i) if nd > 2 else (math.sqrt(0.5 + i) if nd > 1 else i))
                roll, yaw = i * INITIAL_ANGLE_ROLL, i * INITIAL_ANGLE_YAW
                if nd == 1:
                    node["x"] = radius
                elif nd == 2:
                    node["x"] = radius * math.cos(roll)
                    node["y"] = radius * math.sin(roll)
                else:
                    node["x"] = radius * math.sin(roll) * math.cos(yaw)
                    node["y"] = radius * math.cos(roll)
                    node["z"] = radius * math.sin(roll) * math.sin(yaw)
            if _nan(node.get("vx")) or (nd > 1 and _nan(node.get("vy"))) or (nd > 2 and _nan(node.get("vz"))):
                node["vx"] = 0.0
                if nd > 1:
                    node["vy"] = 0.0
                if nd > 2:
                    node["vz"] = 0.0

    def _initialize_force(self, force):
        init = getattr(force, "initialize", None)
        if init:
            init(self._nodes, self._random, self._nDim)
        return force

    def _need_engine(self):
        if self._destroyed:
            raise FlError(FL_E_DEVICE, "the simulation was destroyed")
        if not self._usable:
            raise self._error or FlError(FL_E_DEVICE, "the GPU engine is not available")

    # --- stepping ---
    def _advance(self, iterations):
        """src/gpu/simulation.js:141-151: the alpha schedule on the host, in FP64."""
        if not self._seeded:
            self._seeded = True
            self._engine.eng.set_seed(math.floor(self._random() * 4294967296))
        alphas = np.empty(iterations)
        for k in range(iterations):
            self._alpha += (self._alphaTarget - self._alpha) * self._alphaDecay
            alphas[k] = self._alpha
        self._engine.enqueue(alphas, self._velocityDecay)

    def tick(self, iterations=1):
        """Queue `iterations` ticks; the nodes follow at the next sync(). A destroyed simulation
        ignores it (src/gpu/simulation.js: destroy() leaves tick() callable)."""
        with self._lock:
            if self._destroyed:
                return self
            self._need_engine()
            self._advance(int(iterations))
        return self

    async def tickAsync(self, iterations=1):
        with self._lock:
            self._need_engine()
            self._advance(int(iterations))
            self._engine.sync()
        return self

    async def sync(self):
        with self._lock:
            if self._usable and not self._destroyed:
                self._engine.sync()
        return self

    async def gpuReady(self):
        return self._usable

    def isGPUEnabled(self):
        return self._usable and not self._destroyed

    def gpuBuffers(self):
        if not (self._usable and self._engine) or self._destroyed:
            return None
        return self._engine.eng.buffers()

    def destroy(self):
        with self._lock:
            self._destroyed, self._running, self._usable = True, False, False
            self._stop_timer()
            if self._engine:
                self._engine.destroy()
                self._engine = None
        return self

    # --- the timer (d3-timer's role: one step per frame while running) ---
    def _start_timer(self):
        self._stop_timer()
        if self._destroyed:
            return
        stop = threading.Event()

        def loop():
            time.sleep(0.016)
            while not stop.is_set():
                self._step()
                time.sleep(0.016)

        t = threading.Thread(target=loop, daemon=True)
        self._timer = (t, stop)
        t.start()

    def _stop_timer(self):
        if self._timer:
            self._timer[1].set()
            if self._timer[0] is not threading.current_thread():
                self._timer[0].join(timeout=1.0)
            self._timer = None

    def _step(self):
        with self._lock:
            if not self._running or not self._usable or self._destroyed:
                return
            try:
                self._advance(1)
                if self._readback:
                    self._engine.sync()
                else:
                    self._engine.eng.idle()
            except FlError as e:
                self._error, self._usable = e, False
                return
            self._emit("tick")
            if self._alpha < self._alphaMin:
                self._running = False
                if self._timer:
                    self._timer[1].set()
                self._emit("end")

    def _emit(self, name):
        for fn in list(self._events[name].values()):
            fn(self)

    def restart(self):
        self._running = True
        self._start_timer()
        return self

    def stop(self):
        self._running = False
        self._stop_timer()
        return self

    # --- accessors (src/gpu/simulation.js:306-380) ---
    def numDimensions(self, _=_UNSET):
        if _ is _UNSET:
            return self._nDim
        with self._lock:
            self._nDim = min(MAX_DIMENSIONS, max(1, int(round(_))))
            for f in self._forces.values():
                self._initialize_force(f)
            self._reset()
        return self

    def nodes(self, _=_UNSET):
        if _ is _UNSET:
            return self._nodes
        with self._lock:
            self._nodes = _
            self._initialize_nodes()
            for f in self._forces.values():
                self._initialize_force(f)
            self._reset()
        return self

    def alpha(self, _=_UNSET):
        if _ is _UNSET:
            return self._alpha
        self._alpha = float(_)
        return self

    def alphaMin(self, _=_UNSET):
        if _ is _UNSET:
            return self._alphaMin
        self._alphaMin = float(_)
        return self

    def alphaDecay(self, _=_UNSET):
        if _ is _UNSET:
            return self._alphaDecay
        self._alphaDecay = float(_)
        return self

    def alphaTarget(self, _=_UNSET):
        if _ is _UNSET:
            return self._alphaTarget
        self._alphaTarget = float(_)
        return self

    def velocityDecay(self, _=_UNSET):
        if _ is _UNSET:
            return 1 - self._velocityDecay
        self._velocityDecay = 1 - float(_)
        return self

    def randomSource(self, _=_UNSET):
        if _ is _UNSET:
            return self._random
        with self._lock:
            self._random = _
            for f in self._forces.values():
                self._initialize_force(f)
            if self._engine:
                self._seeded = True
                self._engine.eng.set_seed(math.floor(self._random() * 4294967296))
        return self

    def force(self, name, *args):
        if not args:
            return self._forces.get(name)
        f = args[0]
        if f is not None and not callable(getattr(f, "gpu", None)):
            # the reference runs such a simulation on the CPU (src/gpu/simulation.js:110-139);
            # this engine has no CPU path, so the force is refused and the simulation unchanged
            raise FlError(FL_E_UNSUPPORTED, "force %r has no gpu() description" % (name,))
        with self._lock:
            if f is None:
                self._forces.pop(name, None)
            else:
                self._forces[name] = self._initialize_force(f)
            self._refresh()
        return self

    def find(self, *args):
        args = list(args)
        nd = self._nDim
        x = (args.pop(0) if args else 0) or 0
        y = ((args.pop(0) if args else None) if nd > 1 else None) or 0
        z = ((args.pop(0) if args else None) if nd > 2 else None) or 0
        radius = (args.pop(0) if args else None) or math.inf
        radius *= radius
        closest = None
        for node in self._nodes:
            dx = x - node["x"]
            dy = y - (node.get("y") or 0)
            dz = z - (node.get("z") or 0)
            d2 = dx * dx + dy * dy + dz * dz
            if d2 < radius:
                closest, radius = node, d2
        return closest

    def on(self, name, *args):
        base, _, key = name.partition(".")
        if not args:
            return self._events[base].get(key)
        if args[0] is None:
            self._events[base].pop(key, None)
        else:
            self._events[base][key] = args[0]
        return self


def forceSimulationGPU(nodes=None, numDimensions=None, options=None):
    """forceSimulation(nodes, numDimensions) with the physics on the GPU.

    options: device (CUDA ordinal, default 0), readback (False: the timer does not copy
    positions back on every tick; call sync()), cpuTicks (accepted; the GPU runs every tick)."""
    return Simulation(nodes, numDimensions, options)
