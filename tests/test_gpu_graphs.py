"""Blocks of ticks replayed as CUDA graphs give the same layout as the same ticks launched one
kernel at a time.

fl_enqueue captures a block of ticks the second time it sees one of that length (starting from
the same velocity buffer) and replays the graph from then on; a force change forgets the
graphs. The kernels read each tick's alpha, step and seed from device memory, so a replay sees
the new values; these tests hold the replayed run to the directly launched one."""
import numpy as np
import pytest

from forcegpu._lib import TUNE_GRAPHS, Engine, desc_from_gpu
from forcegpu.batch import Batch, GraphSpec
from forcegpu.graphs import benchmark_links, make_nodes

pytestmark = pytest.mark.gpu


def engine(n, dims, graphs, collide=False, charge=-30.0):
    xyz = make_nodes(n, dims, 10.0 * n ** (1 / 3), seed=4)
    pos4 = np.zeros((n, 4), np.float32)
    pos4[:, :dims] = xyz[:, :dims]
    src, dst = benchmark_links(n, n // 2, seed=4)
    deg = np.bincount(np.concatenate([src, dst]), minlength=n).astype(float)
    forces = [
        {"type": "link", "version": 1, "source": src, "target": dst, "iterations": 1,
         "strengths": 1.0 / np.minimum(deg[src], deg[dst]), "distances": np.full(len(src), 30.0),
         "bias": deg[src] / (deg[src] + deg[dst])},
        {"type": "manyBody", "version": 1, "strengths": np.full(n, charge), "distanceMin2": 1.0,
         "distanceMax2": np.inf, "theta2": 0.81},
        {"type": "center", "x": 0, "y": 0, "z": 0, "strength": 1.0},
    ]
    if collide:
        forces.append({"type": "collide", "version": 1, "radii": 1.0 + np.arange(n) % 4,
                       "strength": 0.7, "iterations": 1})
    e = Engine(0)
    e.set_nodes(pos4, dims)
    e.set_forces([desc_from_gpu(f, k + 1, n) for k, f in enumerate(forces)])
    e.set_seed(99)
    e.set_tuning(TUNE_GRAPHS, 1 if graphs else 0)
    return e


def alphas(count, a=1.0):
    out = []
    for _ in range(count):
        a += (0.0 - a) * 0.0228
        out.append(a)
    return np.array(out)


def blocks(e, al, sizes):
    k = 0
    for c in sizes:
        e.enqueue(al[k:k + c], 0.6)
        k += c
    return k


@pytest.mark.parametrize("dims,collide", [(3, False), (2, True)])
def test_replayed_blocks_match_direct_launches(dims, collide):
    # blocks of 3 ticks start from alternating velocity buffers, so two graphs are captured;
    # the 5-tick and 1-tick blocks are captured and replayed in between
    sizes = [3, 3, 3, 3, 5, 3, 5, 5, 1, 1, 1, 3]
    al = alphas(sum(sizes))
    out = []
    for graphs in (True, False):
        e = engine(3000, dims, graphs, collide)
        blocks(e, al, sizes)
        pos, vel = e.sync()
        out.append((pos.copy(), vel.copy(), e.query(1)))
        e.close()
    (p1, v1, l1), (p0, v0, l0) = out
    assert np.isfinite(p1).all()
    assert l1 == l0, "a replay counts the launches its graph holds"
    np.testing.assert_array_equal(p1, p0)
    np.testing.assert_array_equal(v1, v0)


def test_a_force_change_between_blocks_is_seen_by_the_next_block():
    al = alphas(24)
    out = []
    for graphs in (True, False):
        e = engine(2000, 3, graphs)
        k = blocks(e, al, [4, 4, 4])
        n = 2000
        e.set_forces([desc_from_gpu({"type": "manyBody", "version": 2, "strengths": np.full(n, -5.0),
                                     "distanceMin2": 1.0, "distanceMax2": np.inf, "theta2": 0.81}, 2, n)])
        blocks(e, al[k:], [4, 4, 4])
        out.append(e.sync()[0].copy())
        e.close()
    np.testing.assert_array_equal(out[0], out[1])


def test_batch_replayed_blocks_match_direct_launches():
    def specs():
        out = []
        for i, n in enumerate([40, 700, 2, 1500]):
            xyz = make_nodes(n, 3, 200.0 + n, 30 + i)[:, :3]
            src, dst = benchmark_links(n, n // 3, seed=30 + i)
            out.append(GraphSpec(xyz=xyz, source=src, target=dst))
        return out
    got = []
    # 4-tick blocks are captured on the second and replayed from the third; 5 + 7 never repeat
    for sizes in ([4, 4, 4], [5, 7]):
        b = Batch()
        b.set_graphs(specs(), ndim=3, seed=5)
        for c in sizes:
            b.enqueue(b.alpha_schedule(c))
        got.append(b.sync())
        b.close()
    np.testing.assert_array_equal(got[0][0], got[1][0])
    np.testing.assert_array_equal(got[0][1], got[1][1])
