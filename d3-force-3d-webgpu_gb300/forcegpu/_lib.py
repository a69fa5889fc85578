"""ctypes bindings of libforcegpu.so (include/forcegpu.h).

The engine is CUDA-only: if the library is missing or no GPU is present, every entry point
raises. There is no CPU fallback.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libforcegpu.so")

FL_OK, FL_E_ARG, FL_E_OOM, FL_E_DEVICE, FL_E_TIMEOUT, FL_E_OVERFLOW, FL_E_STATE, FL_E_UNSUPPORTED = range(8)
STATUS_NAMES = ["FL_OK", "FL_E_ARG", "FL_E_OOM", "FL_E_DEVICE", "FL_E_TIMEOUT", "FL_E_OVERFLOW",
                "FL_E_STATE", "FL_E_UNSUPPORTED"]
FORCE_TYPES = {"manyBody": 1, "link": 2, "collide": 3, "center": 4, "radial": 5, "position": 6}
Q_LAUNCHES, Q_TICKS, Q_NODES, Q_ERRWORD, Q_DEVICE_BYTES, Q_WALK_TESTS, Q_WALK_USEFUL = 1, 2, 3, 4, 5, 6, 7
Q_WALK_MAX_STACK, Q_WALK_OPENS, Q_WALK_APPLIES, Q_WALK_RARE = 8, 9, 10, 11

# every symbol include/forcegpu.h declares
EXPORTS = ["fl_create", "fl_destroy", "fl_last_error", "fl_fits", "fl_set_nodes",
           "fl_update_positions", "fl_update_pins", "fl_update_velocities", "fl_set_forces",
           "fl_set_seed", "fl_enqueue", "fl_sync", "fl_idle", "fl_busy", "fl_buffers",
           "fl_stream", "fl_query", "fl_profile", "fl_profile_read", "fl_radix_sort",
           "fl_debug_tree", "fl_set_tuning", "fl_radix_sort_noalloc", "fl_batch_create",
           "fl_batch_destroy", "fl_batch_last_error", "fl_batch_set_graphs", "fl_batch_set_seed",
           "fl_batch_enqueue", "fl_batch_sync", "fl_batch_query", "fl_batch_stream",
           "fl_autotune", "fl_batch_set_tuning", "fl_batch_autotune", "fl_batch_read",
           "fl_update_positions_packed", "fl_update_positions_packed_async", "fl_sync_packed",
           "fl_upload_all", "fl_debug_links",
           "fl_batch_add_graphs"]
SORT_NOALLOC_MAX_PAIRS = 262144  # FL_SORT_NOALLOC_MAX_PAIRS
TUNE_WALK_GROUP, TUNE_CELL_SUMS, TUNE_GRAPHS = 1, 2, 3
TUNE_SORT_PASSES, TUNE_WALK_BLOCKS, TUNE_COLLIDE_CELL, TUNE_TEST_LOOKBACK = 4, 5, 6, 7
CELLS_AUTO, CELLS_FP64_TOP, CELLS_FP32 = 0, 1, 2


class FlError(RuntimeError):
    """A failed engine call: .code is the FL_* status."""

    def __init__(self, code, message):
        self.code = code
        super().__init__("%s: %s" % (STATUS_NAMES[code] if 0 <= code < len(STATUS_NAMES) else code,
                                     message))


class ForceDesc(ctypes.Structure):
    _fields_ = [
        ("type", ctypes.c_int32), ("version", ctypes.c_uint32), ("key", ctypes.c_uint64),
        ("node_a", ctypes.c_void_p), ("node_b", ctypes.c_void_p),
        ("m", ctypes.c_int32), ("source", ctypes.c_void_p), ("target", ctypes.c_void_p),
        ("link_distance", ctypes.c_void_p), ("link_strength", ctypes.c_void_p),
        ("link_bias", ctypes.c_void_p),
        ("iterations", ctypes.c_int32), ("axis", ctypes.c_int32),
        ("distance_min2", ctypes.c_double), ("distance_max2", ctypes.c_double),
        ("theta2", ctypes.c_double), ("strength", ctypes.c_double),
        ("x", ctypes.c_double), ("y", ctypes.c_double), ("z", ctypes.c_double),
    ]


class GraphDesc(ctypes.Structure):
    """fl_graph_desc: one graph of a batch."""
    _fields_ = [
        ("n", ctypes.c_int32), ("m", ctypes.c_int32),
        ("pos4", ctypes.c_void_p), ("vel4", ctypes.c_void_p),
        ("source", ctypes.c_void_p), ("target", ctypes.c_void_p),
        ("link_distance", ctypes.c_void_p), ("link_strength", ctypes.c_void_p),
        ("link_bias", ctypes.c_void_p), ("charge", ctypes.c_void_p),
        ("theta2", ctypes.c_double), ("distance_min2", ctypes.c_double),
        ("distance_max2", ctypes.c_double),
        ("center_x", ctypes.c_double), ("center_y", ctypes.c_double), ("center_z", ctypes.c_double),
        ("center_strength", ctypes.c_double), ("velocity_decay", ctypes.c_double),
        ("tick0", ctypes.c_uint32),
        ("radii", ctypes.c_void_p), ("collide_strength", ctypes.c_double),
        ("collide_iterations", ctypes.c_int32),
    ]


class TuneResult(ctypes.Structure):
    _fields_ = [("walk_group", ctypes.c_int32), ("sort_passes", ctypes.c_int32),
                ("walk_blocks", ctypes.c_int32), ("collide_cell", ctypes.c_int32),
                ("ms_per_tick", ctypes.c_double), ("ms_default", ctypes.c_double),
                ("candidates", ctypes.c_int32), ("from_cache", ctypes.c_int32)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class BufferInfo(ctypes.Structure):
    _fields_ = [("positions", ctypes.c_void_p), ("velocities", ctypes.c_void_p),
                ("count", ctypes.c_int32), ("stride", ctypes.c_int32)]


_lib = None


def load():
    """Load libforcegpu.so (built by d3-force-3d-webgpu_gb300/build.py)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise FlError(FL_E_DEVICE, "libforcegpu.so is not built (run d3-force-3d-webgpu_gb300/build.py)")
    L = ctypes.CDLL(LIB_PATH)
    P, I32, I64, U32, D = ctypes.c_void_p, ctypes.c_int32, ctypes.c_int64, ctypes.c_uint32, ctypes.c_double
    sig = {
        "fl_create": (I32, [I32, ctypes.POINTER(P)]),
        "fl_destroy": (I32, [P]),
        "fl_last_error": (ctypes.c_char_p, [P]),
        "fl_fits": (I32, [P, I64, ctypes.POINTER(I32)]),
        "fl_set_nodes": (I32, [P, I32, I32, P, P, P, P]),
        "fl_update_positions": (I32, [P, I32, I32, P]),
        "fl_upload_all": (I32, [P, P, P, P, P]),
        "fl_debug_links": (I32, [P, I32, P, P, P]),
        "fl_update_pins": (I32, [P, I32, I32, P, P]),
        "fl_update_velocities": (I32, [P, I32, I32, P]),
        "fl_set_forces": (I32, [P, I32, ctypes.POINTER(ForceDesc)]),
        "fl_set_seed": (I32, [P, U32]),
        "fl_enqueue": (I32, [P, P, I32, D]),
        "fl_sync": (I32, [P, P, P]),
        "fl_sync_packed": (I32, [P, P, P]),
        "fl_update_positions_packed": (I32, [P, I32, I32, P]),
        "fl_update_positions_packed_async": (I32, [P, I32, I32, P]),
        "fl_idle": (I32, [P]),
        "fl_busy": (I32, [P, ctypes.POINTER(I32)]),
        "fl_buffers": (I32, [P, ctypes.POINTER(BufferInfo)]),
        "fl_stream": (I32, [P, ctypes.POINTER(P)]),
        "fl_query": (I32, [P, I32, ctypes.POINTER(I64)]),
        "fl_profile": (I32, [P, I32]),
        "fl_profile_read": (I32, [P, I32, P, P, P, ctypes.POINTER(I32)]),
        "fl_radix_sort": (I32, [P, P, I64, I32, P, P]),
        "fl_debug_tree": (I32, [P, I32, P, P, P, P, P, P]),
        "fl_set_tuning": (I32, [P, I32, I32]),
        "fl_radix_sort_noalloc": (I32, [P, P, I64, I32, P, P, P]),
        "fl_batch_create": (I32, [I32, ctypes.POINTER(P)]),
        "fl_batch_destroy": (I32, [P]),
        "fl_batch_last_error": (ctypes.c_char_p, [P]),
        "fl_batch_set_graphs": (I32, [P, I32, I32, ctypes.POINTER(GraphDesc)]),
        "fl_batch_add_graphs": (I32, [P, I32, ctypes.POINTER(GraphDesc)]),
        "fl_batch_set_seed": (I32, [P, U32]),
        "fl_batch_enqueue": (I32, [P, P, I32]),
        "fl_batch_sync": (I32, [P, P, P]),
        "fl_batch_query": (I32, [P, I32, ctypes.POINTER(I64)]),
        "fl_batch_stream": (I32, [P, ctypes.POINTER(P)]),
        "fl_autotune": (I32, [P, I32, D, D, ctypes.c_char_p, ctypes.POINTER(TuneResult)]),
        "fl_batch_set_tuning": (I32, [P, I32, I32]),
        "fl_batch_autotune": (I32, [P, I32, D, ctypes.c_char_p, ctypes.POINTER(TuneResult)]),
        "fl_batch_read": (I32, [P, I32, I32, P, P]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L


def _ptr(a):
    return None if a is None else a.ctypes.data


class Engine:
    """One simulation's device state (an fl_sim). Thin: every method is one C-ABI call."""

    def __init__(self, device=0):
        self.L = load()
        h = ctypes.c_void_p()
        self._check(self.L.fl_create(int(device), ctypes.byref(h)), None)
        self.h = h
        self.n = 0
        self.ndim = 2
        self._keep = []
        self._in_flight = None  # the host array an async upload still reads

    def _check(self, rc, h=...):
        if rc != FL_OK:
            handle = self.h if h is ... else h
            msg = self.L.fl_last_error(handle)
            raise FlError(rc, msg.decode() if msg else "")

    def close(self):
        if getattr(self, "h", None):
            self.L.fl_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def fits(self, count):
        out = ctypes.c_int32()
        self._check(self.L.fl_fits(self.h, int(count), ctypes.byref(out)))
        return bool(out.value)

    def set_nodes(self, pos4, ndim, vel4=None, fix4=None, mask=None):
        pos4 = np.ascontiguousarray(pos4, dtype=np.float32).reshape(-1, 4)
        n = len(pos4)
        vel4 = None if vel4 is None else np.ascontiguousarray(vel4, dtype=np.float32).reshape(n, 4)
        fix4 = None if fix4 is None else np.ascontiguousarray(fix4, dtype=np.float32).reshape(n, 4)
        mask = None if mask is None else np.ascontiguousarray(mask, dtype=np.uint32).reshape(n)
        self._check(self.L.fl_set_nodes(self.h, n, int(ndim), _ptr(pos4), _ptr(vel4), _ptr(fix4), _ptr(mask)))
        self.n, self.ndim = n, min(3, max(1, int(ndim)))

    def upload_all(self, pos4, vel4=None, fix4=None, mask=None):
        """fl_upload_all: replace the state of the current n nodes, keeping the forces."""
        n = self.n
        pos4 = np.ascontiguousarray(pos4, dtype=np.float32).reshape(n, 4)
        vel4 = None if vel4 is None else np.ascontiguousarray(vel4, dtype=np.float32).reshape(n, 4)
        fix4 = None if fix4 is None else np.ascontiguousarray(fix4, dtype=np.float32).reshape(n, 4)
        mask = None if mask is None else np.ascontiguousarray(mask, dtype=np.uint32).reshape(n)
        self._check(self.L.fl_upload_all(self.h, _ptr(pos4), _ptr(vel4), _ptr(fix4), _ptr(mask)))

    def update_positions(self, first, pos4):
        pos4 = np.ascontiguousarray(pos4, dtype=np.float32).reshape(-1, 4)
        self._check(self.L.fl_update_positions(self.h, int(first), len(pos4), _ptr(pos4)))

    def update_positions_packed(self, first, pos):
        """fl_update_positions with ndim floats per node: a (count, ndim) array."""
        pos = np.ascontiguousarray(pos, dtype=np.float32).reshape(-1, self.ndim)
        self._check(self.L.fl_update_positions_packed(self.h, int(first), len(pos), _ptr(pos)))

    def update_positions_packed_async(self, first, pos):
        """fl_update_positions_packed_async: queued, not waited for. `pos` must be a C-contiguous
        float32 (count, ndim) array (best in pinned memory); it is used in place, kept alive here
        and must stay unchanged until the next sync or idle."""
        if pos.dtype != np.float32 or not pos.flags.c_contiguous or pos.size % self.ndim:
            raise ValueError("update_positions_packed_async wants a C-contiguous float32 array "
                             "of count * ndim floats")
        self._check(self.L.fl_update_positions_packed_async(self.h, int(first),
                                                            pos.size // self.ndim, _ptr(pos)))
        self._in_flight = pos

    def update_velocities(self, first, vel4):
        vel4 = np.ascontiguousarray(vel4, dtype=np.float32).reshape(-1, 4)
        self._check(self.L.fl_update_velocities(self.h, int(first), len(vel4), _ptr(vel4)))

    def update_pins(self, first, fix4, mask):
        fix4 = np.ascontiguousarray(fix4, dtype=np.float32).reshape(-1, 4)
        mask = np.ascontiguousarray(mask, dtype=np.uint32).reshape(-1)
        self._check(self.L.fl_update_pins(self.h, int(first), len(fix4), _ptr(fix4), _ptr(mask)))

    def set_forces(self, descs):
        """descs: list of (ForceDesc, [arrays to keep alive during the call])."""
        arr = (ForceDesc * max(1, len(descs)))()
        for i, (d, _) in enumerate(descs):
            arr[i] = d
        self._check(self.L.fl_set_forces(self.h, len(descs), arr))

    def set_seed(self, seed):
        self._check(self.L.fl_set_seed(self.h, int(seed) & 0xffffffff))

    def enqueue(self, alphas, decay):
        a = np.ascontiguousarray(alphas, dtype=np.float64).reshape(-1)
        self._check(self.L.fl_enqueue(self.h, _ptr(a), len(a), float(decay)))

    def sync(self, pos_out=None, vel_out=None):
        """Wait, then read back into float32 (n, 4) arrays (allocated when None and n > 0)."""
        if pos_out is None:
            pos_out = np.empty((self.n, 4), np.float32)
        if vel_out is None:
            vel_out = np.empty((self.n, 4), np.float32)
        self._check(self.L.fl_sync(self.h, _ptr(pos_out), _ptr(vel_out)))
        self._in_flight = None
        return pos_out, vel_out

    def sync_into(self, pos_ptr, vel_ptr):
        """Wait, then read back into caller-owned host memory given by address (e.g. pinned)."""
        self._check(self.L.fl_sync(self.h, pos_ptr, vel_ptr))
        self._in_flight = None

    def sync_packed(self, pos_out=None, vel_out=None):
        """fl_sync into float32 (n, ndim) arrays: ndim floats per node cross the host link."""
        if pos_out is None:
            pos_out = np.empty((self.n, self.ndim), np.float32)
        if vel_out is None:
            vel_out = np.empty((self.n, self.ndim), np.float32)
        for a in (pos_out, vel_out):
            if a.dtype != np.float32 or not a.flags.c_contiguous or a.size != self.n * self.ndim:
                raise ValueError("sync_packed wants C-contiguous float32 arrays of n * ndim floats")
        self._check(self.L.fl_sync_packed(self.h, _ptr(pos_out), _ptr(vel_out)))
        self._in_flight = None
        return pos_out, vel_out

    def sync_packed_into(self, pos_ptr, vel_ptr):
        """fl_sync_packed into caller-owned host memory given by address (e.g. pinned)."""
        self._check(self.L.fl_sync_packed(self.h, pos_ptr, vel_ptr))
        self._in_flight = None

    def idle(self):
        self._check(self.L.fl_idle(self.h))
        self._in_flight = None

    def busy(self):
        out = ctypes.c_int32()
        self._check(self.L.fl_busy(self.h, ctypes.byref(out)))
        return bool(out.value)

    def buffers(self):
        b = BufferInfo()
        self._check(self.L.fl_buffers(self.h, ctypes.byref(b)))
        return {"positions": b.positions, "velocities": b.velocities, "count": b.count,
                "stride": b.stride}

    def set_tuning(self, key, value):
        self._check(self.L.fl_set_tuning(self.h, int(key), int(value)))

    def autotune(self, ticks=10, alpha=0.5, decay=0.6, cache=None):
        """Time candidate tunings on the current nodes and forces, keep the fastest (fl_autotune);
        the state is left as it was. Returns the choice and its timing as a dict."""
        out = TuneResult()
        c = None if cache is None else os.fsencode(cache)
        self._check(self.L.fl_autotune(self.h, int(ticks), float(alpha), float(decay), c,
                                       ctypes.byref(out)))
        return out.as_dict()

    def stream(self):
        out = ctypes.c_void_p()
        self._check(self.L.fl_stream(self.h, ctypes.byref(out)))
        return out.value

    def query(self, what):
        out = ctypes.c_int64()
        self._check(self.L.fl_query(self.h, int(what), ctypes.byref(out)))
        return out.value

    def profile(self, enable):
        self._check(self.L.fl_profile(self.h, int(enable)))

    def debug_tree(self, index):
        """The last tick's tree of force `index`: (keys, perm, left, right, depth, cube5)."""
        n = self.n
        m = max(n - 1, 1)
        keys = np.zeros(n, np.uint64)
        perm = np.zeros(n, np.uint32)
        left = np.zeros(m, np.uint32)
        right = np.zeros(m, np.uint32)
        depth = np.zeros(m, np.uint8)
        cube = np.zeros(5, np.float32)
        self._check(self.L.fl_debug_tree(self.h, int(index), _ptr(keys), _ptr(perm), _ptr(left),
                                         _ptr(right), _ptr(depth), _ptr(cube)))
        return keys, perm, left[:n - 1], right[:n - 1], depth[:n - 1], cube

    def debug_links(self, index, m):
        """The link CSR of force `index` (m links): (row[n + 1], other[2m], code[2m])."""
        row = np.zeros(self.n + 1, np.int32)
        other = np.zeros(max(2 * m, 1), np.int32)
        code = np.zeros(max(2 * m, 1), np.uint32)
        self._check(self.L.fl_debug_links(self.h, int(index), _ptr(row), _ptr(other), _ptr(code)))
        return row, other[:2 * m], code[:2 * m]

    def profile_read(self):
        cap = 32
        names = (ctypes.c_char_p * cap)()
        ms = np.zeros(cap)
        cnt = np.zeros(cap, np.int64)
        count = ctypes.c_int32()
        self._check(self.L.fl_profile_read(self.h, cap, ctypes.addressof(names), _ptr(ms), _ptr(cnt),
                                           ctypes.byref(count)))
        k = min(cap, count.value)
        return {names[i].decode(): (float(ms[i]), int(cnt[i])) for i in range(k)}


def radix_sort(keys, vals, lo_bit=0):
    """The engine's onesweep sort alone: stable, on key bits [lo_bit, 64)."""
    L = load()
    keys = np.ascontiguousarray(keys, dtype=np.uint64)
    vals = np.ascontiguousarray(vals, dtype=np.uint32)
    ko = np.zeros_like(keys)
    vo = np.zeros_like(vals)
    rc = L.fl_radix_sort(_ptr(keys), _ptr(vals), len(keys), int(lo_bit), _ptr(ko), _ptr(vo))
    if rc != FL_OK:
        raise FlError(rc, (L.fl_last_error(None) or b"").decode())
    return ko, vo


def radix_sort_noalloc(keys_ptr, vals_ptr, n, lo_bit, keys_out_ptr, vals_out_ptr, stream=0):
    """fl_radix_sort_noalloc on device buffers (addresses as integers): the sort without any
    device allocation, for callers whose device memory all comes from their own pool."""
    L = load()
    rc = L.fl_radix_sort_noalloc(keys_ptr, vals_ptr, int(n), int(lo_bit), keys_out_ptr,
                                 vals_out_ptr, stream)
    if rc != FL_OK:
        raise FlError(rc, (L.fl_last_error(None) or b"").decode())


def desc_from_gpu(g, key, n):
    """fl_force_desc from a force.gpu() dict (the reference's descriptor, src/*.js gpu()).

    Returns (ForceDesc, keepalive arrays). Per-node arrays become float32 with non-numbers as 0,
    as the reference's floats() does (src/gpu/passes/util.js:17-22)."""
    t = g["type"]
    if t not in FORCE_TYPES:
        raise FlError(FL_E_UNSUPPORTED, "force type %r has no GPU pass" % (t,))
    d = ForceDesc()
    d.type = FORCE_TYPES[t]
    d.version = int(g.get("version", 0)) & 0xffffffff
    d.key = int(key) & 0xffffffffffffffff
    keep = []

    def f32(values, count):
        a = np.zeros(count, np.float32)
        if values is not None and count:
            v = np.asarray(values, dtype=np.float64)[:count]
            v = np.where(np.isfinite(v), v, np.where(np.isnan(v), 0.0, np.sign(v) * 3e38))
            a[:len(v)] = v
        keep.append(a)
        return a.ctypes.data

    if t == "manyBody":
        d.node_a = f32(g["strengths"], n)
        d.distance_min2 = float(g["distanceMin2"])
        d.distance_max2 = float(g["distanceMax2"])
        d.theta2 = float(g["theta2"])
    elif t == "link":
        if "source" in g:  # arrays of endpoint indices instead of link objects
            src = np.ascontiguousarray(g["source"], dtype=np.int32)
            dst = np.ascontiguousarray(g["target"], dtype=np.int32)
            m = len(src)
        else:
            links = g["links"]
            m = len(links)
            src = np.fromiter((l["source"]["index"] for l in links), np.int32, count=m)
            dst = np.fromiter((l["target"]["index"] for l in links), np.int32, count=m)
        if not m:
            src = dst = np.zeros(1, np.int32)
        keep += [src, dst]
        d.m = m
        d.source, d.target = src.ctypes.data, dst.ctypes.data
        d.link_distance = f32(g["distances"], m)
        d.link_strength = f32(g["strengths"], m)
        d.link_bias = f32(g["bias"], m)
        d.iterations = int(g["iterations"]) if m else 0
    elif t == "collide":
        d.node_a = f32(g["radii"], n)
        d.strength = float(g["strength"])
        d.iterations = int(g["iterations"])
    elif t == "center":
        d.x, d.y, d.z, d.strength = (float(g[k]) for k in ("x", "y", "z", "strength"))
    elif t == "radial":
        d.node_a = f32(g["radiuses"], n)
        d.node_b = f32(g["strengths"], n)
        d.x, d.y, d.z = (float(g[k]) for k in ("x", "y", "z"))
    elif t == "position":
        d.axis = int(g["axis"])
        d.node_a = f32(g["targets"], n)
        d.node_b = f32(g["strengths"], n)
    return d, keep
