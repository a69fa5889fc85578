"""CPU oracle: an FP64 C restatement of d3-force-3d's CPU simulation (src/*.js).

Test infrastructure only. The GB300 engine is checked against it; it is never the thing
measured or shipped. Only tests/, ``__graft_entry__.smoke()`` and bench.py's ``cpu_baseline``
and ``--impl reference`` legs import this package.

The C source (d3force_oracle.c) cites, function by function, the reference files it follows.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libd3oracle.so")
SRC = os.path.join(HERE, "d3force_oracle.c")

MODE_D3, MODE_JACOBI, MODE_EXACT = 0, 1, 2


def build(force: bool = False) -> str:
    """Compile the oracle with gcc. -ffp-contract=off keeps every a*b+c rounded twice, as in
    JavaScript, on both x86 and Arm (gcc contracts to FMA by default on aarch64)."""
    os.makedirs(BUILD, exist_ok=True)
    stale = force or not os.path.exists(LIB) or os.path.getmtime(LIB) < max(
        os.path.getmtime(SRC), os.path.getmtime(os.path.join(HERE, "d3force_oracle.h")))
    if stale:
        tmp = LIB + ".tmp%d" % os.getpid()
        subprocess.check_call(["gcc", "-O2", "-std=gnu11", "-fPIC", "-shared",
                               "-ffp-contract=off", "-fno-fast-math", "-pthread", "-o", tmp, SRC, "-lm"])
        os.replace(tmp, LIB)
    return LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB)
        P = ctypes.c_void_p
        D = ctypes.POINTER(ctypes.c_double)
        I32 = ctypes.c_int32
        L.ofl_create.restype = P
        L.ofl_create.argtypes = [I32, I32, D, D, D, ctypes.c_void_p]
        L.ofl_destroy.argtypes = [P]
        L.ofl_set_params.argtypes = [P] + [ctypes.c_double] * 5
        L.ofl_get_params.argtypes = [P, D]
        L.ofl_set_pins.argtypes = [P, D, ctypes.c_void_p]
        L.ofl_get_state.argtypes = [P, D, D]
        L.ofl_set_state.argtypes = [P, D, D]
        L.ofl_get_lcg.restype = ctypes.c_uint32
        L.ofl_get_lcg.argtypes = [P]
        L.ofl_set_lcg.argtypes = [P, ctypes.c_uint32]
        L.ofl_random.restype = ctypes.c_double
        L.ofl_random.argtypes = [P]
        L.ofl_add_manybody.restype = I32
        L.ofl_add_manybody.argtypes = [P, D, ctypes.c_double, ctypes.c_double, ctypes.c_double, I32]
        L.ofl_add_link.restype = I32
        L.ofl_add_link.argtypes = [P, I32, ctypes.c_void_p, ctypes.c_void_p, D, D, I32, I32]
        L.ofl_add_collide.restype = I32
        L.ofl_add_collide.argtypes = [P, D, ctypes.c_double, I32, I32]
        L.ofl_add_center.restype = I32
        L.ofl_add_center.argtypes = [P] + [ctypes.c_double] * 4
        L.ofl_add_radial.restype = I32
        L.ofl_add_radial.argtypes = [P, D, D, ctypes.c_double, ctypes.c_double, ctypes.c_double]
        L.ofl_add_position.restype = I32
        L.ofl_add_position.argtypes = [P, I32, D, D]
        L.ofl_clear_forces.argtypes = [P]
        L.ofl_link_params.argtypes = [P, I32, D, D]
        L.ofl_tick.argtypes = [P, I32]
        L.ofl_apply_force.argtypes = [P, I32, ctypes.c_double]
        L.ofl_walk_stats.argtypes = [P, ctypes.c_void_p]
        L.ofl_collide_probe.restype = I32
        L.ofl_collide_probe.argtypes = [P, I32, I32, ctypes.c_void_p, I32, ctypes.c_void_p]
        L.ofl_manybody_probe.restype = I32
        L.ofl_manybody_probe.argtypes = [P, I32, ctypes.c_double, I32, I32, ctypes.c_void_p, I32,
                                         ctypes.c_void_p]
        L.ofl_levels.restype = I32
        L.ofl_levels.argtypes = [I32]
        L.ofl_cube.restype = I32
        L.ofl_cube.argtypes = [I32, I32, ctypes.c_void_p, D]
        L.ofl_morton.argtypes = [I32, I32, ctypes.c_void_p, ctypes.c_void_p]
        L.ofl_sort_perm.argtypes = [I32, ctypes.c_void_p, ctypes.c_void_p]
        L.ofl_karras.argtypes = [I32, I32, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                 ctypes.c_void_p]
        L.ofl_csr.argtypes = [I32, I32, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                              ctypes.c_void_p, ctypes.c_void_p]
        _lib = L
    return _lib


def _dptr(a):
    if a is None:
        return None
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _f64(a, n, cols=None):
    if a is None:
        return None
    a = np.ascontiguousarray(a, dtype=np.float64)
    if cols is not None:
        a = a.reshape(n, cols)
    return a


class OracleSim:
    """forceSimulation(nodes, numDimensions) in FP64, with forces added in application order.

    xyz / vxyz / fxyz are (n, 3) arrays (NaN = unset, as a missing x in the reference's node
    objects); fmask holds the pinned axes (bits 1, 2, 4 for fx, fy, fz)."""

    def __init__(self, n, ndim=2, xyz=None, vxyz=None, fxyz=None, fmask=None):
        self.n, self.ndim = int(n), int(ndim)
        L = lib()
        self._keep = [_f64(xyz, n, 3), _f64(vxyz, n, 3), _f64(fxyz, n, 3)]
        m = None if fmask is None else np.ascontiguousarray(fmask, dtype=np.uint8)
        self._keep.append(m)
        self._h = L.ofl_create(self.n, self.ndim, _dptr(self._keep[0]), _dptr(self._keep[1]),
                               _dptr(self._keep[2]), None if m is None else m.ctypes.data)
        self.ndim = min(3, max(1, self.ndim))

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            lib().ofl_destroy(h)
            self._h = None

    # --- parameters (names as in the reference's simulation object) ---
    def params(self):
        out = np.zeros(5)
        lib().ofl_get_params(self._h, _dptr(out))
        return out

    def set_params(self, alpha=None, alphaMin=None, alphaDecay=None, alphaTarget=None,
                   velocityDecay=None):
        p = self.params()
        if alpha is not None: p[0] = alpha
        if alphaMin is not None: p[1] = alphaMin
        if alphaDecay is not None: p[2] = alphaDecay
        if alphaTarget is not None: p[3] = alphaTarget
        if velocityDecay is not None: p[4] = 1 - velocityDecay
        lib().ofl_set_params(self._h, *[float(v) for v in p])
        return self

    @property
    def alpha(self):
        return float(self.params()[0])

    def set_pins(self, fxyz, fmask):
        fxyz = _f64(fxyz, self.n, 3)
        m = np.ascontiguousarray(fmask, dtype=np.uint8)
        lib().ofl_set_pins(self._h, _dptr(fxyz), m.ctypes.data)

    def state(self):
        x = np.zeros((self.n, 3))
        v = np.zeros((self.n, 3))
        lib().ofl_get_state(self._h, _dptr(x), _dptr(v))
        return x, v

    def set_state(self, xyz=None, vxyz=None):
        xyz, vxyz = _f64(xyz, self.n, 3), _f64(vxyz, self.n, 3)
        lib().ofl_set_state(self._h, _dptr(xyz), _dptr(vxyz))

    @property
    def lcg(self):
        return lib().ofl_get_lcg(self._h)

    @lcg.setter
    def lcg(self, v):
        lib().ofl_set_lcg(self._h, int(v) & 0xffffffff)

    def random(self):
        return lib().ofl_random(self._h)

    # --- forces ---
    def manybody(self, strengths=None, distanceMin=1.0, distanceMax=float("inf"), theta=0.9,
                 mode=MODE_D3):
        s = _f64(np.full(self.n, -30.0) if strengths is None else strengths, self.n)
        self._keep.append(s)
        return lib().ofl_add_manybody(self._h, _dptr(s), float(distanceMin) ** 2,
                                      float(distanceMax) ** 2, float(theta) ** 2, mode)

    def link(self, src, dst, distance=None, strength=None, iterations=1, mode=MODE_D3):
        src = np.ascontiguousarray(src, dtype=np.int32)
        dst = np.ascontiguousarray(dst, dtype=np.int32)
        m = len(src)
        d = None if distance is None else _f64(np.broadcast_to(distance, (m,)), m)
        s = None if strength is None else _f64(np.broadcast_to(strength, (m,)), m)
        self._keep += [src, dst, d, s]
        return lib().ofl_add_link(self._h, m, src.ctypes.data, dst.ctypes.data, _dptr(d),
                                  _dptr(s), int(iterations), mode)

    def link_params(self, k, m):
        bias = np.zeros(m)
        st = np.zeros(m)
        lib().ofl_link_params(self._h, k, _dptr(bias), _dptr(st))
        return bias, st

    def collide(self, radii=1.0, strength=1.0, iterations=1, mode=MODE_D3):
        r = _f64(np.broadcast_to(radii, (self.n,)), self.n)
        self._keep.append(r)
        return lib().ofl_add_collide(self._h, _dptr(r), float(strength), int(iterations), mode)

    def center(self, x=0.0, y=0.0, z=0.0, strength=1.0):
        return lib().ofl_add_center(self._h, float(x), float(y), float(z), float(strength))

    def radial(self, radius, strength=0.1, x=0.0, y=0.0, z=0.0):
        r = _f64(np.broadcast_to(radius, (self.n,)), self.n)
        s = _f64(np.broadcast_to(strength, (self.n,)), self.n).copy()
        s[np.isnan(r)] = 0
        self._keep += [r, s]
        return lib().ofl_add_radial(self._h, _dptr(r), _dptr(s), float(x), float(y), float(z))

    def position(self, axis, target=0.0, strength=0.1):
        t = _f64(np.broadcast_to(target, (self.n,)), self.n)
        s = _f64(np.broadcast_to(strength, (self.n,)), self.n).copy()
        s[np.isnan(t)] = 0
        self._keep += [t, s]
        return lib().ofl_add_position(self._h, int(axis), _dptr(t), _dptr(s))

    def clear_forces(self):
        lib().ofl_clear_forces(self._h)

    def tick(self, iterations=1):
        lib().ofl_tick(self._h, int(iterations))
        return self

    def apply_force(self, k, alpha):
        lib().ofl_apply_force(self._h, int(k), float(alpha))

    def manybody_probe(self, k, alpha, targets, mode=MODE_D3, threads=1):
        """Velocity change many-body force k would give the target nodes (count x 3), state
        unchanged: MODE_D3 by d3's tree walk, MODE_EXACT by the FP64 sum over all pairs."""
        t = np.ascontiguousarray(targets, dtype=np.int32)
        out = np.zeros((len(t), 3), dtype=np.float64)
        rc = lib().ofl_manybody_probe(self._h, int(k), float(alpha), int(mode), len(t), t.ctypes.data,
                                      int(threads), out.ctypes.data)
        if rc != 0:
            raise ValueError("manybody_probe: bad force index or target")
        return out

    def collide_probe(self, k, targets, threads=1):
        """Velocity change one Jacobi iteration of collide force k gives the target nodes (count
        x 3), state unchanged: the values of the JACOBI mode's full pass, at O(count n)."""
        t = np.ascontiguousarray(targets, dtype=np.int32)
        out = np.zeros((len(t), 3), dtype=np.float64)
        rc = lib().ofl_collide_probe(self._h, int(k), len(t), t.ctypes.data, int(threads),
                                     out.ctypes.data)
        if rc != 0:
            raise ValueError("collide_probe: bad force index or target")
        return out

    def walk_stats(self):
        out = np.zeros(3, dtype=np.int64)
        lib().ofl_walk_stats(self._h, out.ctypes.data)
        return out


# --- integer rebuilds -----------------------------------------------------------------------

def levels(ndim):
    return lib().ofl_levels(int(ndim))


def cube(pos4, ndim):
    pos4 = np.ascontiguousarray(pos4, dtype=np.float32)
    out = np.zeros(4)
    lg = lib().ofl_cube(len(pos4), int(ndim), pos4.ctypes.data, _dptr(out))
    return out, lg


def morton(pos4, ndim):
    pos4 = np.ascontiguousarray(pos4, dtype=np.float32)
    codes = np.zeros(len(pos4), dtype=np.uint64)
    lib().ofl_morton(len(pos4), int(ndim), pos4.ctypes.data, codes.ctypes.data)
    return codes


def sort_perm(codes):
    codes = np.ascontiguousarray(codes, dtype=np.uint64)
    perm = np.zeros(len(codes), dtype=np.uint32)
    lib().ofl_sort_perm(len(codes), codes.ctypes.data, perm.ctypes.data)
    return perm


def karras(sorted_codes, ndim):
    sc = np.ascontiguousarray(sorted_codes, dtype=np.uint64)
    n = len(sc)
    m = max(n - 1, 0)
    left = np.zeros(max(m, 1), dtype=np.uint32)
    right = np.zeros(max(m, 1), dtype=np.uint32)
    depth = np.zeros(max(m, 1), dtype=np.int32)
    lib().ofl_karras(n, int(ndim), sc.ctypes.data, left.ctypes.data, right.ctypes.data,
                     depth.ctypes.data)
    return left[:m], right[:m], depth[:m]


def csr(n, src, dst):
    src = np.ascontiguousarray(src, dtype=np.int32)
    dst = np.ascontiguousarray(dst, dtype=np.int32)
    m = len(src)
    row = np.zeros(n + 1, dtype=np.int32)
    other = np.zeros(max(2 * m, 1), dtype=np.int32)
    code = np.zeros(max(2 * m, 1), dtype=np.int32)
    lib().ofl_csr(int(n), m, src.ctypes.data, dst.ctypes.data, row.ctypes.data,
                  other.ctypes.data, code.ctypes.data)
    return row, other[:2 * m], code[:2 * m]
