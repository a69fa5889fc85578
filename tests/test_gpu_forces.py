"""Every force on the GPU against the oracle (the reference's CPU forces) on identical input:
the cases of test/gpu-forces-test.js, through the C ABI. The GPU works in f32, so agreement is
to ~1e-4 relative, with the reference's tolerances and outlier allowance."""
import math

import numpy as np
import pytest

from forcegpu import (forceCenter, forceCollide, forceLink, forceManyBody, forceRadial, forceX,
                      forceY, forceZ)
from forcegpu._lib import CELLS_FP32, CELLS_FP64_TOP, TUNE_CELL_SUMS, TUNE_WALK_GROUP
from gpu_helpers import assert_nodes_close, make_nodes, run_both, tree_outliers

pytestmark = pytest.mark.gpu

DIMS = [1, 2, 3]


@pytest.mark.parametrize("dims", DIMS)
def test_manybody_all_pairs(dims):
    r = run_both(dims, 300, 1, lambda: [("charge", forceManyBody().theta(1e-6))])
    assert_nodes_close(r["gpu"], r["cpu"], dims)


@pytest.mark.parametrize("dims", DIMS)
def test_manybody_strength_distance_min_max(dims):
    r = run_both(dims, 200, 3, lambda: [("charge", forceManyBody().theta(1e-6)
                                         .strength(lambda d, i, *a: -20 - i % 7 if i % 3 else 15)
                                         .distanceMin(5).distanceMax(150))])
    assert_nodes_close(r["gpu"], r["cpu"], dims, rtol=1e-3)


@pytest.mark.parametrize("dims", DIMS)
def test_center(dims):
    def nodes(n, d):
        out = make_nodes(n, d, 100)
        for node in out:
            node["x"] = float(np.float32(node["x"] + 40))
            if d > 1:
                node["y"] = float(np.float32(node["y"] - 25))
            if d > 2:
                node["z"] = float(np.float32(node["z"] + 10))
        return out
    r = run_both(dims, 1000, 2, lambda: [("center", forceCenter(3, 4 if dims > 1 else 0,
                                                                5 if dims > 2 else 0).strength(0.7))],
                 nodes_fn=nodes)
    assert_nodes_close(r["gpu"], r["cpu"], dims, rtol=1e-3)


@pytest.mark.parametrize("dims", DIMS)
def test_radial(dims):
    r = run_both(dims, 200, 3, lambda: [("radial", forceRadial(lambda d, i, *a: 30 + i % 5 * 10, 5,
                                                               -5 if dims > 1 else 0,
                                                               2 if dims > 2 else 0).strength(0.3))])
    assert_nodes_close(r["gpu"], r["cpu"], dims, rtol=1e-3)


@pytest.mark.parametrize("dims", DIMS)
def test_position(dims):
    def forces():
        f = [("x", forceX(lambda d, i, *a: i % 10).strength(lambda d, i, *a: 0.2 if i % 4 else 0.05))]
        if dims > 1:
            f.append(("y", forceY(-20).strength(0.3)))
        if dims > 2:
            f.append(("z", forceZ(15).strength(0.1)))
        return f
    r = run_both(dims, 200, 3, forces)
    assert_nodes_close(r["gpu"], r["cpu"], dims, rtol=1e-3)


@pytest.mark.parametrize("dims", DIMS)
def test_link_disjoint(dims):
    def forces():
        links = [{"source": i, "target": i + 1} for i in range(0, 200, 2)]
        return [("link", forceLink(links).distance(lambda l, i, *a: 10 + i % 5).strength(0.8))]
    r = run_both(dims, 200, 5, forces)
    assert_nodes_close(r["gpu"], r["cpu"], dims, rtol=1e-3)


@pytest.mark.parametrize("dims", DIMS)
def test_link_iterations_disjoint(dims):
    def forces():
        links = [{"source": i, "target": i + 1} for i in range(0, 100, 2)]
        return [("link", forceLink(links).distance(25).strength(1).iterations(3))]
    r = run_both(dims, 100, 3, forces)
    assert_nodes_close(r["gpu"], r["cpu"], dims, rtol=1e-3)


def _pairs(n, d):
    nodes = []
    for i in range(0, n, 2):
        a, b = {"x": float(i * 20)}, {"x": float(i * 20 + 3 + i % 5)}
        if d > 1:
            a["y"] = b["y"] = float((i % 7) * 3)
        if d > 2:
            a["z"] = b["z"] = 0.0
        nodes += [a, b]
    return nodes


@pytest.mark.parametrize("iterations", [1, 3])
@pytest.mark.parametrize("dims", DIMS)
def test_collide_separated_pairs(dims, iterations):
    """Each node overlaps one partner only, so d3's sequential pushes equal the GPU's Jacobi
    ones; with iterations(3), each iteration sees the velocities the one before left
    (src/gpu/passes/collide.js:127-133)."""
    r = run_both(dims, 100, 4, lambda: [("collide", forceCollide(lambda d, i, *a: 6 + i % 3)
                                         .strength(0.9).iterations(iterations))],
                 nodes_fn=_pairs)
    assert_nodes_close(r["gpu"], r["cpu"], dims, rtol=1e-3)


@pytest.mark.parametrize("n", [1, 2, 3, 7, 8, 9, 127, 128, 129, 255, 257])
def test_manybody_sizes_around_block_width(n):
    r = run_both(3, n, 2, lambda: [("charge", forceManyBody().theta(1e-6))])
    assert_nodes_close(r["gpu"], r["cpu"], 3, rtol=1e-3, atol=1e-3)


# --- the Barnes-Hut tree (theta > 0): the same tree as the CPU ---

@pytest.mark.parametrize("dims,rtol", [(1, 2e-2), (2, 1e-3), (3, 1e-3)])
def test_tree_500(dims, rtol):
    r = run_both(dims, 500, 1, lambda: [("charge", forceManyBody())])
    assert_nodes_close(r["gpu"], r["cpu"], dims, rtol=rtol, outliers=tree_outliers(500))


@pytest.mark.parametrize("theta", [0.5, 1.5])
def test_tree_theta(theta):
    r = run_both(3, 2000, 1, lambda: [("charge", forceManyBody().theta(theta))])
    assert_nodes_close(r["gpu"], r["cpu"], 3, rtol=1e-3, outliers=tree_outliers(2000))


def test_tree_strength_distance_min_max():
    r = run_both(3, 2000, 1, lambda: [("charge", forceManyBody().strength(lambda d, i, *a: -10 - i % 7)
                                       .distanceMin(3).distanceMax(60))])
    assert_nodes_close(r["gpu"], r["cpu"], 3, rtol=1e-3, outliers=tree_outliers(2000))


def _walk_group(group):
    return lambda sim, _: sim._engine.eng.set_tuning(TUNE_WALK_GROUP, group)


@pytest.mark.parametrize("group", [32, 16, 1])
def test_tree_walk_groups_distances_theta(group):
    r = run_both(3, 2000, 2, lambda: [("charge", forceManyBody().theta(0.7)
                                       .strength(lambda d, i, *a: -10 - i % 7)
                                       .distanceMin(2).distanceMax(80))],
                 setup=_walk_group(group))
    assert_nodes_close(r["gpu"], r["cpu"], 3, rtol=1e-3, outliers=tree_outliers(2000))


@pytest.mark.parametrize("group", [32, 16, 1])
def test_tree_walk_groups_mixed_signs(group):
    r = run_both(3, 2000, 2, lambda: [("charge", forceManyBody().theta(0.7)
                                       .strength(lambda d, i, *a: -20 if i % 4 else 12))],
                 setup=_walk_group(group))
    assert_nodes_close(r["gpu"], r["cpu"], 3, rtol=1e-3, outliers=tree_outliers(2000))


@pytest.mark.parametrize("cells", [CELLS_FP64_TOP, CELLS_FP32])
def test_tree_cell_sum_variants(cells):
    """The recursion's cell sums (FP64 near the root, or all FP32) in place of the exact
    fixed-point closed form: the same tree, the same forces within the tolerance."""
    r = run_both(3, 2000, 1, lambda: [("charge", forceManyBody())],
                 setup=lambda sim, _: sim._engine.eng.set_tuning(TUNE_CELL_SUMS, cells))
    assert_nodes_close(r["gpu"], r["cpu"], 3, rtol=1e-3, outliers=tree_outliers(2000))


@pytest.mark.parametrize("dims,group", [(3, 0), (3, 32), (2, 0)])
def test_tree_mixed_signs_cancelling_cells(dims, group):
    """Cells whose children's strengths cancel: in 3D (c = sqrt(1/2)) the sum can leave d3 a
    tiny FP64 residual, a value that d3 does not skip (`!quad.value`, src/manyBody.js:74) and
    that it opens when the cell is near. Here one such cell sits inside distanceMax of 30 nodes
    at the second tick; skipping it moved each by ~800x the tolerance, so the recursion keeps
    d3's FP64 values bit for bit and no node may be off. In 2D (c = 1) the values are sums of
    the integer strengths, so cells that cancel are exactly 0 and skipped at both ends."""
    r = run_both(dims, 2000, 2, lambda: [("charge", forceManyBody().theta(0.7)
                                          .strength(lambda d, i, *a: -20 if i % 4 else 12)
                                          .distanceMin(2).distanceMax(80 if dims == 3 else 60))],
                 setup=_walk_group(group))
    assert_nodes_close(r["gpu"], r["cpu"], dims, rtol=1e-3, outliers=0)


@pytest.mark.parametrize("dims,rtol", [(1, 2e-2), (2, 1e-3), (3, 1e-3)])
def test_tree_mixed_signs(dims, rtol):
    r = run_both(dims, 1000, 1, lambda: [("charge", forceManyBody().strength(lambda d, i, *a: -30 if i % 3 else 20))])
    assert_nodes_close(r["gpu"], r["cpu"], dims, rtol=rtol, outliers=tree_outliers(1000))


def test_tree_huge_cube():
    def nodes(n, d):
        out = make_nodes(n, d)
        out[0]["x"], out[1]["y"] = 1e5, -2e5
        return out
    r = run_both(3, 1000, 1, lambda: [("charge", forceManyBody())], nodes_fn=nodes)
    assert_nodes_close(r["gpu"], r["cpu"], 3, rtol=1e-3, outliers=tree_outliers(1000))


def test_tree_far_from_origin():
    def nodes(n, d):
        out = make_nodes(n, d)
        for node in out:
            node["x"] = float(np.float32(node["x"] + 5e4))
            node["y"] = float(np.float32(node["y"] - 3e4))
            node["z"] = float(np.float32(node["z"] + 1e4))
        return out
    r = run_both(3, 1000, 1, lambda: [("charge", forceManyBody())], nodes_fn=nodes)
    assert_nodes_close(r["gpu"], r["cpu"], 3, rtol=1e-2, outliers=tree_outliers(1000))


@pytest.mark.parametrize("n", [2, 3, 1025])
def test_tree_small_sizes(n):
    r = run_both(3, n, 2, lambda: [("charge", forceManyBody())])
    assert_nodes_close(r["gpu"], r["cpu"], 3, rtol=1e-3, outliers=tree_outliers(n))


@pytest.mark.parametrize("n", [8192, 8193, 32769])
def test_tree_method_switch_sizes(n):
    r = run_both(3, n, 1, lambda: [("charge", forceManyBody())],
                 nodes_fn=lambda n_, d: make_nodes(n_, d, 20 * n_ ** (1 / 3)))
    assert_nodes_close(r["gpu"], r["cpu"], 3, rtol=1e-3, outliers=tree_outliers(n))


@pytest.mark.parametrize("dims,far", [(2, 120), (3, 120), (2, 2000), (3, 2000)])
def test_tree_shared_top_levels(dims, far):
    """A clump of side 2 and one outlier: long runs of points sharing the top levels."""
    def nodes(n, d):
        out = make_nodes(n, d, 2)
        out[0]["x"] = float(far)
        return out
    r = run_both(dims, 9000, 1, lambda: [("charge", forceManyBody())], nodes_fn=nodes)
    assert_nodes_close(r["gpu"], r["cpu"], dims, rtol=1e-3, outliers=tree_outliers(9000))


def test_tree_20_ticks():
    r = run_both(3, 1000, 20, lambda: [("charge", forceManyBody()), ("center", forceCenter())])
    assert_nodes_close(r["gpu"], r["cpu"], 3, rtol=1e-3, outliers=tree_outliers(1000))


# --- collide on large graphs: the grid finds the pairs ---

# iterations(3) in 2D and 3D only: the 1D layout spans 200,000 units, where FP32 positions are
# 1/64 apart and three iterations' velocities no longer agree with the FP64 CPU to 1e-3
@pytest.mark.parametrize("dims,iterations", [(1, 1), (2, 1), (3, 1), (2, 3), (3, 3)])
def test_collide_grid_separated_pairs(dims, iterations):
    def pairs(n, d):
        nodes, side = [], math.ceil((n / 2) ** (1 / d))
        for i in range(0, n, 2):
            k = i // 2
            a, b = {"x": float((k % side) * 40)}, {"x": float((k % side) * 40 + 3 + i % 5)}
            if d > 1:
                a["y"] = b["y"] = float((k // side) % side * 40 + i % 7)
            if d > 2:
                a["z"] = b["z"] = float((k // side // side) * 40)
            nodes += [a, b]
        return nodes
    r = run_both(dims, 10000, 3, lambda: [("collide", forceCollide(lambda d, i, *a: 6 + i % 3)
                                           .strength(0.9).iterations(iterations))],
                 nodes_fn=pairs)
    assert_nodes_close(r["gpu"], r["cpu"], dims, rtol=1e-3)


def test_collide_grid_coincident():
    def clump(n, d):
        nodes = make_nodes(n, 3, 60)
        for i in range(50):
            nodes[i]["x"] = nodes[i]["y"] = nodes[i]["z"] = 0.0
        return nodes
    r = run_both(3, 10000, 1, lambda: [("collide", forceCollide(2))], nodes_fn=clump)
    g = r["gpu"]
    closest = min(math.dist([g[i]["x"], g[i]["y"], g[i]["z"]], [g[j]["x"], g[j]["y"], g[j]["z"]])
                  for i in range(50) for j in range(i + 1, 50))
    assert closest > 0, "coincident nodes separated"
    assert all(math.isfinite(d["x"] + d["y"] + d["z"]) for d in g)


def test_force_order():
    """center moves positions, x and charge move velocities: the order is observable."""
    def nodes(n, d):
        out = make_nodes(n, d, 120)
        for node in out:
            node["x"] = float(np.float32(node["x"] + 30))
        return out
    r = run_both(3, 250, 5, lambda: [("charge", forceManyBody().theta(1e-6).strength(-15)),
                                     ("x", forceX(10).strength(0.05)), ("center", forceCenter()),
                                     ("radial", forceRadial(60).strength(0.02))], nodes_fn=nodes)
    assert_nodes_close(r["gpu"], r["cpu"], 3, rtol=2e-3, atol=1e-3)


def test_fixed_positions():
    def setup(sim, nodes):
        nodes[0].update(fx=5.0, fy=-6.0, fz=7.0)
        nodes[1]["fx"] = 100.0
    r = run_both(3, 120, 5, lambda: [("charge", forceManyBody().theta(1e-6)), ("center", forceCenter())],
                 setup=setup)
    g = r["gpu"]
    assert (g[0]["x"], g[0]["y"], g[0]["z"], g[0]["vx"]) == (5, -6, 7, 0)
    assert g[1]["x"] == 100
    assert_nodes_close(r["gpu"], r["cpu"], 3, rtol=2e-3, atol=1e-3)


def test_coincident_nodes_separate():
    r = run_both(3, 10, 30, lambda: [("charge", forceManyBody()), ("collide", forceCollide(2))],
                 nodes_fn=lambda n, d: [{"x": 1.0, "y": 2.0, "z": 3.0} for _ in range(n)])
    g = r["gpu"]
    for i in range(10):
        assert math.isfinite(g[i]["x"]) and math.isfinite(g[i]["y"]) and math.isfinite(g[i]["z"])
        for j in range(i + 1, 10):
            assert math.dist([g[i][k] for k in "xyz"], [g[j][k] for k in "xyz"]) > 0.5
