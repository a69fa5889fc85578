"""Helpers of the GPU parity tests: the same run on the oracle (FP64 d3 CPU simulation) and on
the GB300 engine, and the reference's tolerance scheme (test/gpu-helpers.js:41-104)."""
import asyncio
import math

import numpy as np

import oracle
from forcegpu import forceSimulationGPU
from forcegpu.graphs import make_nodes as _make_xyz


def make_nodes(n, dims, size=200.0, seed=12345):
    """test/gpu-helpers.js:42-53: f32-exact coordinates, as dict nodes."""
    xyz = _make_xyz(n, dims, size, seed)
    keys = ["x", "y", "z"][:dims]
    return [{k: float(xyz[i, a]) for a, k in enumerate(keys)} for i in range(n)]


def fields(dims):
    return ["x", "y", "z"][:dims] + ["vx", "vy", "vz"][:dims]


def assert_nodes_close(actual, expected, dims, rtol=1e-4, atol=1e-4, outliers=0):
    """test/gpu-helpers.js:63-79: |a - e| <= atol + rtol * max(1, |a|, |e|) for every field of
    every node, except at most `outliers` nodes (which must still be finite)."""
    assert len(actual) == len(expected)
    missed, worst = [], 0.0
    for i, (a, e) in enumerate(zip(actual, expected)):
        miss = None
        for f in fields(dims):
            av, ev = a[f], e[f]
            assert math.isfinite(av), "node %d.%s is %r" % (i, f, av)
            tol = atol + rtol * max(1.0, abs(av), abs(ev))
            d = abs(av - ev)
            worst = max(worst, d / tol)
            if not d <= tol and miss is None:
                miss = "node %d.%s: %r vs %r (|diff| %g > %g)" % (i, f, av, ev, d, tol)
        if miss:
            missed.append(miss)
    assert len(missed) <= outliers, "%d node(s) off (%d allowed): %s" % (
        len(missed), outliers, "; ".join(missed[:3]))
    return worst


def tree_outliers(n):
    """test/gpu-helpers.js:82-84: one per 1000 nodes, at least 1."""
    return max(1, math.ceil(n / 1000))


def oracle_from(nodes, dims, forces, sim_params=None):
    """An OracleSim with the nodes' state and the forces' evaluated descriptors (force.gpu())."""
    n = len(nodes)
    xyz = np.full((n, 3), np.nan)
    vxyz = np.full((n, 3), np.nan)
    fxyz = np.zeros((n, 3))
    fmask = np.zeros(n, np.uint8)
    for i, d in enumerate(nodes):
        for a, k in enumerate("xyz"):
            if d.get(k) is not None:
                xyz[i, a] = d[k]
            if d.get("v" + k) is not None:
                vxyz[i, a] = d["v" + k]
            if d.get("f" + k) is not None:
                fxyz[i, a] = d["f" + k]
                fmask[i] |= 1 << a
    # pins are set after creation: a node pinned after its simulation was made keeps its x until
    # the first integration, in the reference as here
    o = oracle.OracleSim(n, dims, xyz=xyz, vxyz=vxyz)
    o.set_pins(fxyz, fmask)
    if sim_params:
        o.set_params(**sim_params)
    for f in forces:
        add_oracle_force(o, f.gpu(), n)
    return o


def add_oracle_force(o, g, n, mode=None):
    t = g["type"]
    if t == "manyBody":
        return o.manybody(np.asarray(g["strengths"], float), math.sqrt(g["distanceMin2"]),
                          math.sqrt(g["distanceMax2"]), math.sqrt(g["theta2"]),
                          oracle.MODE_D3 if mode is None else mode)
    if t == "link":
        links = g["links"]
        src = [l["source"]["index"] for l in links]
        dst = [l["target"]["index"] for l in links]
        k = o.link(src, dst, np.asarray(g["distances"], float), np.asarray(g["strengths"], float),
                   g["iterations"], oracle.MODE_D3 if mode is None else mode)
        return k
    if t == "collide":
        return o.collide(np.asarray(g["radii"], float), g["strength"], g["iterations"],
                         oracle.MODE_D3 if mode is None else mode)
    if t == "center":
        return o.center(g["x"], g["y"], g["z"], g["strength"])
    if t == "radial":
        return o.radial(np.asarray(g["radiuses"], float), np.asarray(g["strengths"], float),
                        g["x"], g["y"], g["z"])
    if t == "position":
        return o.position(g["axis"], np.asarray(g["targets"], float), np.asarray(g["strengths"], float))
    raise ValueError(t)


def oracle_nodes(o, template):
    """The oracle's state as dict nodes (same keys as the template nodes)."""
    x, v = o.state()
    out = []
    for i in range(len(template)):
        out.append({"x": x[i, 0], "y": x[i, 1], "z": x[i, 2],
                    "vx": v[i, 0], "vy": v[i, 1], "vz": v[i, 2]})
    return out


def run_both(dims, n, ticks, make_forces, nodes_fn=None, setup=None, options=None):
    """test/gpu-helpers.js:86-104: the same forces from the same start, k ticks on the oracle
    (the reference's CPU simulation) and on the GPU engine through the C ABI."""
    nodes_fn = nodes_fn or (lambda n_, d_: make_nodes(n_, d_))
    gpu_nodes = nodes_fn(n, dims)
    sim = forceSimulationGPU(gpu_nodes, dims, options).stop()
    forces = make_forces()
    for name, f in forces:
        sim.force(name, f)
    if setup:
        setup(sim, gpu_nodes)
    assert asyncio.run(sim.gpuReady()) is True, "the simulation should run on the GPU"
    # the oracle starts from the state the GPU simulation starts from (after its own init)
    o = oracle_from(gpu_nodes, dims, [f for _, f in forces])
    asyncio.run(sim.tickAsync(ticks))
    o.tick(ticks)
    sim.destroy()
    return {"gpu": gpu_nodes, "cpu": oracle_nodes(o, gpu_nodes), "sim": sim, "oracle": o}
