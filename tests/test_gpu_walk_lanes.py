"""The walk of one point per warp (FL_TUNE_WALK_GROUP 1, the default up to 32,768 nodes) against
the union walk of 32-point groups.

Both make each point's own d3 traversal (src/manyBody.js:73-115): the same cells opened and the
same cells or points applied, the uncommon cases (chains, jiggles, distanceMin) decided the
same way. The walk counters count those (point, child) pairs, so they must agree exactly; the
velocities agree up to the order in which each point's FP32 sum is added."""
import numpy as np
import pytest

from forcegpu._lib import (Q_WALK_APPLIES, Q_WALK_OPENS, Q_WALK_USEFUL, TUNE_WALK_GROUP, Engine,
                           desc_from_gpu)
from forcegpu.graphs import make_nodes

pytestmark = pytest.mark.gpu


def run(n, dims, group, dmax2=np.inf, mixed=False, theta2=0.81):
    xyz = make_nodes(n, dims, 8.0 * n ** (1 / dims), seed=7)
    pos4 = np.zeros((n, 4), np.float32)
    pos4[:, :dims] = xyz[:, :dims]
    pos4[10:14] = pos4[9]   # coincident points: d3's jiggle
    pos4[20, 0] = pos4[21, 0]  # a zero component only
    s = np.where(np.arange(n) % 4 == 0, 12.0, -20.0) if mixed else np.full(n, -30.0)
    e = Engine(0)
    e.set_nodes(pos4, dims)
    e.set_forces([desc_from_gpu({"type": "manyBody", "version": 1, "strengths": s,
                                 "distanceMin2": 4.0, "distanceMax2": dmax2, "theta2": theta2},
                                1, n)])
    e.set_seed(3)
    e.set_tuning(TUNE_WALK_GROUP, group)
    e.profile(2)
    e.enqueue(np.array([0.7]), 0.6)
    _, vel = e.sync()
    counts = [e.query(q) for q in (Q_WALK_USEFUL, Q_WALK_OPENS, Q_WALK_APPLIES)]
    e.close()
    return vel[:, :dims].astype(np.float64), counts


@pytest.mark.parametrize("n,dims,dmax2,mixed", [(1000, 3, np.inf, False), (5000, 3, 900.0, False),
                                                (3000, 2, np.inf, True), (700, 1, np.inf, False),
                                                (20000, 3, np.inf, True)])
def test_lanes_walk_makes_the_union_walks_traversal(n, dims, dmax2, mixed):
    v32, c32 = run(n, dims, 32, dmax2, mixed)
    v1, c1 = run(n, dims, 1, dmax2, mixed)
    assert c1 == c32, "the same (point, child) tests, opens and applies"
    assert c1[0] > n and c1[2] > 0
    scale = np.abs(v32).max()
    assert np.isfinite(v1).all() and scale > 0
    np.testing.assert_allclose(v1, v32, rtol=0, atol=2e-5 * scale)


def test_default_group_by_size_is_the_lanes_walk_up_to_32768_nodes():
    for n, group in ((32768, 1), (32769, 32)):
        v_default, c_default = run(n, 3, 0)
        v_group, c_group = run(n, 3, group)
        assert c_default == c_group
        np.testing.assert_array_equal(v_default, v_group)
