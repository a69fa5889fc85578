"""Batches of graphs (fl_batch_*): every graph of a batch against the oracle run on that graph
alone, and a graph alone against the same graph in a mix.

The batch's forces are link (applied as the reference's GPU does: all links against one
snapshot, the oracle's Jacobi mode), many-body by d3's tree and centre, with d3's defaults."""
import math

import numpy as np
import pytest

import oracle
from forcegpu import FlError
from forcegpu.batch import Batch, GraphSpec
from forcegpu.graphs import benchmark_links, make_nodes
from gpu_helpers import tree_outliers

pytestmark = pytest.mark.gpu


def spec(n, dims, seed, **kw):
    xyz = make_nodes(n, dims, 200.0 + n, seed)[:, :dims]
    src, dst = benchmark_links(n, n // 3, seed=seed)
    return GraphSpec(xyz=xyz, source=src, target=dst, **kw)


def oracle_run(s, dims, ticks):
    """The reference's CPU simulation of one graph (Jacobi links and collide, as the GPU), the
    forces in the batch's order: link, many-body, collide, centre."""
    n = len(s.xyz)
    xyz = np.zeros((n, 3))
    xyz[:, :dims] = s.xyz
    o = oracle.OracleSim(n, dims, xyz=xyz)
    o.set_params(alphaDecay=s.alpha_decay, velocityDecay=s.velocity_decay)
    if len(s.source):
        o.link(s.source, s.target, mode=oracle.MODE_JACOBI)
    o.manybody(None if s.charge is None else np.asarray(s.charge, float), theta=s.theta,
               distanceMin=s.distance_min, distanceMax=s.distance_max)
    if s.radii is not None:
        o.collide(np.asarray(s.radii, float), s.collide_strength, s.collide_iterations,
                  oracle.MODE_JACOBI)
    if s.center_strength:
        o.center(*s.center, strength=s.center_strength)
    o.tick(ticks)
    return o.state()[0][:, :dims]


def assert_close(got, want, rtol, outliers):
    tol = 1e-3 + rtol * np.maximum(1.0, np.maximum(np.abs(got), np.abs(want)))
    bad = np.any(np.abs(got - want) > tol, axis=1)
    assert np.isfinite(got).all()
    assert bad.sum() <= outliers, "%d nodes off (%d allowed), worst %g" % (
        bad.sum(), outliers, (np.abs(got - want) / tol).max())


@pytest.mark.parametrize("dims", [2, 3])
def test_every_graph_of_a_batch_matches_the_oracle(dims):
    sizes = [1, 2, 3, 40, 257, 1500, 31, 700]
    specs = [spec(n, dims, 100 + i) for i, n in enumerate(sizes)]
    specs[3].alpha_decay = 0.05                     # a graph with its own schedule
    specs[4].theta, specs[4].distance_max = 0.6, 150.0
    specs[5].center, specs[5].center_strength = (10.0, -5.0, 3.0), 0.5
    specs[6].velocity_decay = 0.2
    b = Batch()
    b.set_graphs(specs, ndim=dims, seed=7)
    ticks = 3
    b.run(ticks)
    got = b.positions()
    for s, p in zip(specs, got):
        want = oracle_run(s, dims, ticks)
        assert_close(p, want, 1e-3, tree_outliers(len(p)))


@pytest.mark.parametrize("dims", [2, 3])
def test_graphs_with_collide_in_a_batch_match_the_oracle(dims):
    """Collide in a batch: one grid over every graph, each with its own cell side (twice its
    largest radius), strength and iterations; graphs without a collide force beside them."""
    sizes = [300, 2, 1200, 40, 900, 5000]
    specs = [spec(n, dims, 300 + i) for i, n in enumerate(sizes)]
    rng = np.random.default_rng(8)
    for i, s_ in enumerate(specs):
        if i % 3 != 1:  # graphs 1 and 4 have no collide force
            s_.radii = rng.uniform(1.0, 5.0, len(s_.xyz)).astype(np.float32).astype(float)
            # dense enough for overlaps: spacing ~ a few radii
            s_.xyz = np.float32(s_.xyz * (0.15 if dims == 3 else 0.05)).astype(float)
    specs[2].collide_strength, specs[2].collide_iterations = 0.7, 2
    b = Batch()
    b.set_graphs(specs, ndim=dims, seed=7)
    ticks = 3
    b.run(ticks)
    got = b.positions()
    for s_, p in zip(specs, got):
        want = oracle_run(s_, dims, ticks)
        assert_close(p, want, 1e-3, tree_outliers(len(p)) + len(p) // 200)


def mixed_charges(n):
    return np.where(np.arange(n) % 4 == 0, 12.0, -20.0)


@pytest.mark.parametrize("dims", [2, 3])
def test_graphs_with_mixed_sign_charges_in_a_batch_match_the_oracle(dims):
    """A graph whose charges have both signs puts the whole batch on d3's cell recursion (the
    others' cells too): every graph against the oracle, the mixed ones with distanceMax, where
    a cell whose children cancel decides whether a near node sees its children."""
    sizes = [2, 600, 2000, 40, 1500]
    specs = [spec(n, dims, 400 + i) for i, n in enumerate(sizes)]
    for i in (1, 2, 4):
        specs[i].charge = mixed_charges(sizes[i])
    specs[2].theta, specs[2].distance_min, specs[2].distance_max = 0.7, 2.0, 80.0
    b = Batch()
    b.set_graphs(specs, ndim=dims, seed=7)
    ticks = 2
    b.run(ticks)
    got = b.positions()
    for s_, p in zip(specs, got):
        want = oracle_run(s_, dims, ticks)
        assert_close(p, want, 1e-3, tree_outliers(len(p)))


def test_a_mixed_charge_graph_alone_and_in_a_mix_agree_bit_for_bit():
    """The cell recursion keeps each graph's cells its own: a mixed-charge graph alone and among
    other graphs, 100 ticks, the same bit for bit."""
    me = spec(1500, 3, 9)
    me.charge = mixed_charges(1500)
    others = [spec(n, 3, 50 + i) for i, n in enumerate([700, 2, 2500, 31])]
    others[0].charge = mixed_charges(700)
    alone = Batch()
    alone.set_graphs([me], ndim=3, seed=3)
    alone.run(100)
    a = alone.positions()[0]
    mix = Batch()
    mix.set_graphs(others[:2] + [me] + others[2:], ndim=3, seed=3)
    mix.run(100)
    m = mix.positions()[2]
    assert np.isfinite(a).all()
    assert np.array_equal(m, a)


@pytest.mark.parametrize("dims", [2, 3])
def test_a_graph_alone_and_in_a_mix_agree_bit_for_bit(dims):
    """The same graph laid out alone and among others, 300 ticks: its result does not depend on
    the rest of the batch (the continuous-batching property a server relies on). Every sum of a
    graph is the graph's own: exact integer centre sums and cell sums at the graph's own scale,
    walk groups that start at the graph's first point, jiggles drawn from graph-local ids. So
    the layouts agree bit for bit (a force layout is chaotic: any difference in the last bit
    would grow by orders of magnitude over 300 ticks)."""
    me = spec(900, dims, 5)
    me.xyz = me.xyz.copy() * 0.2
    me.xyz[7] = me.xyz[3]  # a coincident pair: jiggles in the walk and the collide
    me.radii = 1.0 + np.arange(900) % 4
    others = [spec(n, dims, 20 + i) for i, n in enumerate([300, 2, 1200, 77, 33])]
    others[2].radii = np.full(1200, 3.0)
    alone = Batch()
    alone.set_graphs([me], ndim=dims, seed=3)
    alone.run(300)
    a = alone.positions()[0]
    mix = Batch()
    mix.set_graphs(others[:2] + [me] + others[2:], ndim=dims, seed=3)
    mix.run(300)
    m = mix.positions()[2]
    assert np.isfinite(a).all()
    assert np.array_equal(m, a)


def test_graphs_with_finished_schedules_and_many_ticks_stay_finite():
    specs = [spec(n, 3, 50 + n) for n in (5, 60, 600)]
    b = Batch()
    b.set_graphs(specs, ndim=3)
    b.run(300)
    for p in b.positions():
        assert np.isfinite(p).all()
        assert np.abs(p).max() < 1e5


def test_a_bad_link_is_refused():
    s = spec(10, 3, 1)
    s.target = s.target.copy()
    s.target[0] = 10
    b = Batch()
    with pytest.raises(FlError):
        b.set_graphs([s], ndim=3)


def test_the_batch_counts_its_launches_per_tick_independent_of_graphs():
    one, many = Batch(), Batch()
    one.set_graphs([spec(500, 3, 9)], ndim=3)
    many.set_graphs([spec(500, 3, 9 + i) for i in range(64)], ndim=3)
    one.run(2)
    many.run(2)
    one.sync(), many.sync()
    assert one.launches() == many.launches(), "one launch per kernel per tick, whatever the batch"


def test_graphs_added_to_a_running_batch_match_them_alone():
    """fl_batch_add_graphs: a graph appended to a batch that has run for a while (without a
    readback of the others) lays out as it would alone, and the graphs already there go on as
    if nothing joined, bit for bit."""
    a, b_, c = spec(700, 3, 61), spec(90, 3, 62), spec(500, 3, 63)
    c.xyz = c.xyz * 0.3
    c.xyz[5] = c.xyz[9]  # coincident: jiggles in the walk and the collide
    c.radii = 1.0 + np.arange(500) % 3
    mix = Batch()
    mix.set_graphs([a, b_], ndim=3, seed=4)
    mix.run(7)
    mix.add_graphs([c])
    mix.run(9)
    got = mix.positions()
    alone_a = Batch()
    alone_a.set_graphs([a], ndim=3, seed=4)
    alone_a.run(16)
    alone_c = Batch()
    alone_c.set_graphs([c], ndim=3, seed=4)
    alone_c.run(9)
    assert np.isfinite(got[2]).all()
    assert np.array_equal(got[0], alone_a.positions()[0])
    assert np.array_equal(got[2], alone_c.positions()[0])
