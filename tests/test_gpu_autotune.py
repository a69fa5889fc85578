"""The autotuner (fl_autotune, fl_batch_autotune): it leaves the simulation's state as it found
it, keeps values every knob accepts, caches its choice per configuration, and the tuned engine
lays out the same as the untuned one (the knobs change launch shapes and the order of some float
sums, not the forces)."""
import numpy as np
import pytest

from forcegpu._lib import (Q_TICKS, TUNE_COLLIDE_CELL, TUNE_SORT_PASSES, TUNE_WALK_BLOCKS,
                           TUNE_WALK_GROUP, Engine, desc_from_gpu)
from forcegpu.batch import Batch, GraphSpec
from forcegpu.graphs import benchmark_links, make_nodes
from gpu_helpers import tree_outliers

pytestmark = pytest.mark.gpu


def engine(n, dims, collide=False):
    xyz = make_nodes(n, dims, 8.0 * n ** (1 / dims), seed=6)
    pos4 = np.zeros((n, 4), np.float32)
    pos4[:, :dims] = xyz[:, :dims]
    src, dst = benchmark_links(n, n // 2, seed=6)
    deg = np.bincount(np.concatenate([src, dst]), minlength=n).astype(float)
    forces = [
        {"type": "link", "version": 1, "source": src, "target": dst, "iterations": 1,
         "strengths": 1.0 / np.minimum(deg[src], deg[dst]), "distances": np.full(len(src), 30.0),
         "bias": deg[src] / (deg[src] + deg[dst])},
        {"type": "manyBody", "version": 1, "strengths": np.full(n, -30.0), "distanceMin2": 1.0,
         "distanceMax2": np.inf, "theta2": 0.81},
        {"type": "center", "x": 0, "y": 0, "z": 0, "strength": 1.0},
    ]
    if collide:
        forces.insert(2, {"type": "collide", "version": 1, "radii": 1.0 + np.arange(n) % 5,
                          "strength": 0.7, "iterations": 1})
    e = Engine(0)
    e.set_nodes(pos4, dims)
    e.set_forces([desc_from_gpu(f, k + 1, n) for k, f in enumerate(forces)])
    e.set_seed(3)
    return e


def close(a, b, rtol, outliers):
    tol = 1e-3 + rtol * np.maximum(1.0, np.maximum(np.abs(a), np.abs(b)))
    bad = np.any(np.abs(a - b) > tol, axis=1)
    return np.isfinite(a).all() and bad.sum() <= outliers


@pytest.mark.parametrize("dims,collide", [(3, False), (2, True)])
def test_autotune_keeps_the_state_and_the_layout(dims, collide, tmp_path):
    n = 20000
    e = engine(n, dims, collide)
    e.enqueue(np.full(3, 0.9), 0.6)
    before_p, before_v = (a.copy() for a in e.sync())
    ticks = e.query(Q_TICKS)
    got = e.autotune(ticks=3, alpha=0.5, cache=str(tmp_path / "tune.txt"))
    after_p, after_v = e.sync()
    assert np.array_equal(after_p, before_p) and np.array_equal(after_v, before_v)
    assert e.query(Q_TICKS) == ticks
    assert got["walk_group"] in (0, 1, 16, 32) and 0 <= got["sort_passes"] <= 8
    assert got["walk_blocks"] in (0, 8, 6, 4) and got["collide_cell"] in (100, 150, 200)
    assert got["candidates"] >= 2 and got["from_cache"] == 0
    assert 0 < got["ms_per_tick"] <= got["ms_default"] * 1.0001
    # the tuned engine against one with the defaults, from the same state
    ref = engine(n, dims, collide)
    ref.enqueue(np.full(3, 0.9), 0.6)
    al = np.linspace(0.8, 0.5, 6)
    e.enqueue(al, 0.6)
    ref.enqueue(al, 0.6)
    assert close(e.sync()[0][:, :dims], ref.sync()[0][:, :dims], 1e-3, tree_outliers(n))
    e.close(), ref.close()


def test_autotune_reads_its_cache(tmp_path):
    cache = str(tmp_path / "tune.txt")
    e = engine(10000, 3)
    first = e.autotune(ticks=2, cache=cache)
    e.close()
    e = engine(10000, 3)
    second = e.autotune(ticks=2, cache=cache)
    assert second["from_cache"] == 1 and second["candidates"] == 0
    for k in ("walk_group", "sort_passes", "walk_blocks"):
        assert second[k] == first[k]
    e.close()
    assert open(cache).read().count("\n") == 1


@pytest.mark.parametrize("key,value", [(TUNE_SORT_PASSES, 3), (TUNE_SORT_PASSES, 8),
                                       (TUNE_WALK_BLOCKS, 4), (TUNE_WALK_GROUP, 16),
                                       (TUNE_WALK_GROUP, 32), (TUNE_WALK_GROUP, 1),
                                       (TUNE_COLLIDE_CELL, 200)])
def test_each_knob_value_lays_out_the_same(key, value):
    n = 12000
    al = np.linspace(0.9, 0.6, 5)
    tuned, ref = engine(n, 3, collide=True), engine(n, 3, collide=True)
    tuned.set_tuning(key, value)
    tuned.enqueue(al, 0.6)
    ref.enqueue(al, 0.6)
    a, b = tuned.sync()[0][:, :3], ref.sync()[0][:, :3]
    if key in (TUNE_SORT_PASSES, TUNE_WALK_BLOCKS):
        assert np.array_equal(a, b), "the same sort and the same per-point walk: bit for bit"
    else:
        assert close(a, b, 1e-3, tree_outliers(n))
    tuned.close(), ref.close()


def test_batch_autotune_keeps_the_state(tmp_path):
    specs = []
    for i, n in enumerate([300, 5000, 40, 1200]):
        xyz = make_nodes(n, 3, 200.0 + n, 60 + i)[:, :3]
        src, dst = benchmark_links(n, n // 3, seed=60 + i)
        specs.append(GraphSpec(xyz=xyz, source=src, target=dst))
    b = Batch()
    b.set_graphs(specs, ndim=3, seed=1)
    b.run(2)
    p0, v0 = (a.copy() for a in b.sync())
    got = b.autotune(ticks=2, cache=str(tmp_path / "t.txt"))
    p1, v1 = b.sync()
    assert np.array_equal(p0, p1) and np.array_equal(v0, v1)
    assert got["candidates"] >= 2 and got["walk_blocks"] in (0, 8, 6, 4)
    again = b.autotune(ticks=2, cache=str(tmp_path / "t.txt"))
    assert again["from_cache"] == 1
    b.run(2)
    assert all(np.isfinite(p).all() for p in b.positions())
    b.close()
