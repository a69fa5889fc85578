"""The link's snapshot of p + v, which the integrate writes for the next tick when the tick's first
pass is a link (a link end then gathers one record instead of p and v).

Host edits between ticks must reach it: velocities overwritten with fl_update_velocities, and
positions with fl_update_positions, are what the next tick's link sees. Each test runs an engine
that is edited mid-run against a fresh engine handed the same state, and compares them bit for
bit: the fresh engine builds its snapshot (and its box and centre sums) from scratch, so any stale
record in the edited one shows up as a difference."""
import numpy as np
import pytest

from forcegpu._lib import Engine, desc_from_gpu
from forcegpu.graphs import benchmark_links, make_nodes

pytestmark = pytest.mark.gpu


def forces(n, src, dst):
    deg = np.bincount(np.concatenate([src, dst]), minlength=n).astype(float)
    return [
        {"type": "link", "version": 1, "source": src, "target": dst, "iterations": 1,
         "strengths": 1.0 / np.minimum(deg[src], deg[dst]), "distances": np.full(len(src), 30.0),
         "bias": deg[src] / (deg[src] + deg[dst])},
        {"type": "manyBody", "version": 1, "strengths": np.full(n, -30.0), "distanceMin2": 1.0,
         "distanceMax2": np.inf, "theta2": 0.81},
        {"type": "center", "x": 0, "y": 0, "z": 0, "strength": 1.0},
    ]


def engine(pos4, vel4, fs, n):
    e = Engine(0)
    e.set_nodes(pos4, 3, vel4)
    e.set_forces([desc_from_gpu(f, k + 1, n) for k, f in enumerate(fs)])
    e.set_seed(5)
    return e


@pytest.mark.parametrize("n", [3000, 60000])  # the one-point-per-warp walk, then 32-point groups
@pytest.mark.parametrize("edit", ["velocities", "positions"])
def test_an_edit_between_ticks_reaches_the_next_link(n, edit):
    xyz = make_nodes(n, 3, 10.0 * n ** (1 / 3), seed=9)
    pos4 = np.zeros((n, 4), np.float32)
    pos4[:, :3] = xyz[:, :3]
    src, dst = benchmark_links(n, n // 2, seed=9)
    fs = forces(n, src, dst)
    al = np.linspace(0.9, 0.8, 6)
    a = engine(pos4, None, fs, n)
    a.enqueue(al[:5], 0.6)  # blocks of one length, so that the next block replays a graph
    p, v = (x.copy() for x in a.sync())
    rng = np.random.default_rng(1)
    if edit == "velocities":
        v[:, :3] = rng.normal(0.0, 2.0, (n, 3)).astype(np.float32)
        a.update_velocities(0, v)
    else:
        p[:, :3] += rng.normal(0.0, 2.0, (n, 3)).astype(np.float32)
        a.update_positions(0, p)
    a.enqueue(al[5:6], 0.6)
    pa, va = a.sync()
    b = engine(p, v, fs, n)
    b.enqueue(al[5:6], 0.6)
    pb, vb = b.sync()
    # the jiggle's step differs between the two (b starts at 0), but nothing here coincides
    np.testing.assert_array_equal(pa, pb)
    np.testing.assert_array_equal(va, vb)
    a.close(), b.close()
