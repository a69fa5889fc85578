"""The integer stages of the GPU tree, bit-exact against the oracle's CPU rebuild: the radix
sort alone (test/gpu-sort-test.js), Morton codes of the d3 cube, the sort permutation and the
Karras topology with its d3 depths."""
import asyncio

import numpy as np
import pytest

import oracle
from forcegpu import forceManyBody, forceSimulationGPU
from forcegpu._lib import TUNE_SORT_PASSES, radix_sort
from gpu_helpers import make_nodes

pytestmark = pytest.mark.gpu

SMALL_TILE, TILE = 2048, 5120  # pairs per onesweep tile: up to 131,072 pairs, and the fewest above


def lcg_keys(n, spread, seed=7):
    s, out = seed, np.empty(n, np.uint64)
    for i in range(n):
        s = (s * 1664525 + 1013904223) & 0xffffffff
        out[i] = s % spread
    return out


def stable_order(keys):
    return np.argsort(keys, kind="stable")


# above 131,072 pairs the tiles hold 1024 threads x 5 to 8 pairs, as few as give every SM one
# (5 up to 152 x 5,120 pairs, then 6, 7 and 8)
@pytest.mark.parametrize("n", [1, 2, 3, 255, 256, 257, SMALL_TILE - 1, SMALL_TILE, SMALL_TILE + 1,
                               3 * SMALL_TILE + 17, 100000, 131072, 131073, 131072 + 3 * TILE + 5,
                               700001, 900000, 1_100_003, 1_300_000])
def test_sort_random_32bit_keys(n):
    keys32 = lcg_keys(n, 1 << 32)
    keys = keys32 << np.uint64(32)
    ko, vo = radix_sort(keys, np.arange(n, dtype=np.uint32), lo_bit=32)
    order = stable_order(keys32)
    assert np.array_equal(vo, order.astype(np.uint32))
    assert np.array_equal(ko, keys[order])


def test_sort_is_stable():
    keys = lcg_keys(20000, 37) << np.uint64(32)
    _, vo = radix_sort(keys, np.arange(20000, dtype=np.uint32), lo_bit=32)
    assert np.array_equal(vo, stable_order(keys).astype(np.uint32))


def test_sort_on_requested_digits_only():
    """2 passes from bit 8 of 32-bit keys: the sort sees only bits 8..23."""
    keys32 = lcg_keys(5000, 1 << 32)
    digits = (keys32 >> np.uint64(8)) & np.uint64(0xffff)
    _, vo = radix_sort(digits << np.uint64(48), np.arange(5000, dtype=np.uint32), lo_bit=48)
    assert np.array_equal(vo, stable_order(digits).astype(np.uint32))


def test_sort_full_64bit_keys():
    rng = np.random.default_rng(5)
    keys = rng.integers(0, 2**63, size=300000, dtype=np.uint64) | (rng.integers(0, 2, 300000, dtype=np.uint64) << np.uint64(63))
    keys[::7] = keys[3]  # ties
    ko, vo = radix_sort(keys, np.arange(len(keys), dtype=np.uint32), lo_bit=0)
    order = stable_order(keys)
    assert np.array_equal(vo, order.astype(np.uint32))


def _tree_of(nodes, dims, sort_passes=0):
    sim = forceSimulationGPU(nodes, dims).stop()
    if sort_passes:  # digit passes and the run fix-up even for a small layout
        sim._engine.eng.set_tuning(TUNE_SORT_PASSES, sort_passes)
    sim.force("charge", forceManyBody())
    asyncio.run(sim.tickAsync(1))
    # positions the tree was built from: the state before the tick
    return sim


def clustered_nodes(dims, clusters, per, spread, tight, seed, loose=0):
    """`clusters` clusters of `per` points each, their centres spread over `spread` and their
    points within `tight` of the centre (some exactly coincident), plus `loose` spread points:
    many points share the top 32 bits of their Morton codes but differ below."""
    rng = np.random.default_rng(seed)
    xyz = []
    for c in range(clusters):
        centre = rng.uniform(-spread / 2, spread / 2, dims)
        off = rng.uniform(0, tight, (per, dims))
        off[per // 3] = off[0]  # a coincident pair
        xyz.append(centre + off)
    xyz.append(rng.uniform(-spread / 2, spread / 2, (loose, dims)))
    xyz = np.float32(np.concatenate(xyz)).astype(np.float64)
    rng.shuffle(xyz)
    return [{k: float(v) for k, v in zip("xyz", row)} for row in xyz]


# the tree's sort orders the top 32 key bits by digit passes and then the runs of equal top
# bits by a fix-up: runs of a few points, of up to 1024 (ranked in place) and longer ones (sorted
# by the last block of the fix-up); up to 6144 points it ranks every pair in one launch instead,
# unless digit passes are asked for (sort_passes 4: both paths are checked at every size)
CLUSTERED = {
    "short runs 3d": (3, 200, 30, 200.0, 1e-3, 1, 0),
    "long run 3d": (3, 1, 3000, 200.0, 1e-3, 2, 2000),
    "several long runs 3d": (3, 3, 1500, 200.0, 1e-3, 3, 500),
    "short and long runs 2d": (2, 50, 40, 200.0, 1e-5, 4, 0),
    "long run 2d": (2, 1, 2500, 200.0, 1e-5, 5, 300),
}


@pytest.mark.parametrize("dims,n,size", [(1, 500, 200), (2, 2000, 200), (3, 5000, 200),
                                         (3, 3000, 2), (3, 1000, 2e5), (2, 257, 1),
                                         (3, 6144, 300), (3, 6145, 300), (2, 4, 1)]
                         + [pytest.param(v[0], None, k, id=k) for k, v in CLUSTERED.items()])
@pytest.mark.parametrize("sort_passes", [0, 4])
def test_tree_matches_cpu_rebuild(dims, n, size, sort_passes):
    if n is None:
        nodes = clustered_nodes(*CLUSTERED[size])
        n = len(nodes)
    else:
        nodes = make_nodes(n, dims, size)
    nodes[0]["x"] = nodes[1]["x"]  # shared coordinates
    if dims > 1:
        nodes[2]["x"], nodes[2]["y"] = nodes[3]["x"], nodes[3]["y"]
    start = np.zeros((n, 4), np.float32)
    for i, d in enumerate(nodes):
        for a, k in enumerate("xyz"[:dims]):
            start[i, a] = d[k]
    sim = _tree_of(nodes, dims, sort_passes)
    keys, perm, left, right, depth, cube = sim._engine.eng.debug_tree(0)
    sim.destroy()
    codes = oracle.morton(start, dims)
    L = oracle.levels(dims)
    bits = L * dims
    ref_cube, lg = oracle.cube(start, dims)
    assert list(cube[:4]) == [np.float32(v) for v in ref_cube] and int(cube[4]) == lg
    ref_perm = oracle.sort_perm(codes)
    assert np.array_equal(perm, ref_perm), "sort permutation"
    assert np.array_equal(keys, codes[ref_perm] << np.uint64(64 - bits)), "Morton codes"
    rl, rr, rd = oracle.karras(codes[ref_perm], dims)
    assert np.array_equal(left, rl) and np.array_equal(right, rr), "Karras topology"
    assert np.array_equal(depth.astype(np.int32), rd), "d3 depths"
