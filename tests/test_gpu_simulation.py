"""forceSimulationGPU, the facade, on the GPU: the behaviours test/gpu-simulation-test.js checks
(the timer, tick / tickAsync / sync, alpha, edits to the nodes while it runs, forces added,
changed and removed, nodes replaced, dimensionality, buffers, readback off, determinism,
destroy). CPU results come from the oracle, the reference's CPU simulation in FP64.

Where the reference falls back to the CPU (a force without gpu(), nodes beyond the device's
limits), this engine has no CPU path: those cases check that the refusal is an error and that
the simulation stays usable."""
import asyncio
import gc
import math
import time
import weakref

import numpy as np
import pytest

from forcegpu import (FlError, forceCenter, forceCollide, forceLink, forceManyBody,
                      forceSimulationGPU, forceX, forceZ)
from forcegpu._lib import FL_E_UNSUPPORTED
from gpu_helpers import assert_nodes_close, make_nodes, oracle_from, oracle_nodes

pytestmark = pytest.mark.gpu


def run(coro):
    return asyncio.run(coro)


def make(nodes, dims, options=None):
    sim = forceSimulationGPU(nodes, dims, options)
    assert run(sim.gpuReady()) is True, "the simulation should run on the GPU"
    return sim


def cpu_twin(sim, nodes, dims, forces, **params):
    """The oracle from the state the GPU simulation starts from, with the same forces."""
    return oracle_from(nodes, dims, forces, params or None)


def test_runs_on_the_gpu_when_a_device_is_available():
    sim = make(make_nodes(10, 3), 3).stop()
    assert sim.isGPUEnabled() is True
    sim.destroy()


def test_advances_alpha_exactly_like_force_simulation():
    nodes = make_nodes(20, 2)
    sim = make(nodes, 2).stop().alphaTarget(0.1).alphaDecay(0.05)
    charge = forceManyBody()
    sim.force("charge", charge)
    o = cpu_twin(sim, nodes, 2, [charge], alphaTarget=0.1, alphaDecay=0.05)
    run(sim.tickAsync(17))
    o.tick(17)
    assert sim.alpha() == o.alpha
    sim.destroy()


def test_tick_async_resolves_with_the_simulation_once_the_nodes_are_up_to_date():
    nodes = make_nodes(50, 3)
    before = [n["x"] for n in nodes]
    sim = make(nodes, 3).stop().force("charge", forceManyBody())
    assert run(sim.tickAsync(3)) is sim
    assert any(n["x"] != b for n, b in zip(nodes, before)), "nodes moved"
    sim.destroy()


def test_tick_is_asynchronous_nodes_are_current_after_sync():
    nodes = make_nodes(50, 3)
    charge = forceManyBody().theta(1e-6)
    sim = make(nodes, 3).stop().force("charge", charge)
    o = cpu_twin(sim, nodes, 3, [charge])
    assert sim.tick(4) is sim
    o.tick(4)
    run(sim.sync())
    assert_nodes_close(nodes, oracle_nodes(o, nodes), 3, rtol=1e-3)
    sim.destroy()


def test_emits_tick_events_with_up_to_date_nodes_then_end():
    nodes = make_nodes(30, 2)
    seen = {"ticks": 0, "ends": 0, "x": []}
    sim = forceSimulationGPU(nodes, 2, {"cpuTicks": 0}).alphaDecay(0.3).force("charge", forceManyBody())

    def on_tick(_):
        seen["ticks"] += 1
        seen["x"].append(nodes[0]["x"])

    sim.on("tick", on_tick)
    sim.on("end", lambda _: seen.__setitem__("ends", seen["ends"] + 1))
    time.sleep(1.5)
    assert seen["ends"] == 1, "end fires once"
    assert sim.alpha() < sim.alphaMin()
    assert 3 < seen["ticks"] <= 40, seen["ticks"]
    assert seen["x"][-1] != seen["x"][0], "positions change from tick to tick"
    sim.destroy()


def test_stop_and_restart_control_the_timer():
    nodes = make_nodes(30, 2)
    ticks = [0]
    sim = forceSimulationGPU(nodes, 2, {"cpuTicks": 0}).force("charge", forceManyBody())
    sim.on("tick", lambda _: ticks.__setitem__(0, ticks[0] + 1))
    time.sleep(0.1)
    sim.stop()
    time.sleep(0.1)
    stopped = ticks[0]
    time.sleep(0.2)
    assert ticks[0] == stopped, "no ticks while stopped"
    sim.alpha(1).restart()
    time.sleep(0.2)
    assert ticks[0] > stopped, "ticks resume"
    sim.destroy()


def test_picks_up_force_parameter_changes_made_after_the_simulation_started():
    nodes = make_nodes(30, 3)
    charge = forceManyBody().theta(1e-6)
    sim = make(nodes, 3).stop().force("charge", charge)
    o = cpu_twin(sim, nodes, 3, [charge])
    run(sim.tickAsync(2))
    o.tick(2)
    charge.strength(lambda d, i, *a: -10 - i).distanceMin(3)
    o.clear_forces()
    o.manybody(np.array([-10.0 - i for i in range(30)]), 3.0, math.inf, 1e-6)
    run(sim.tickAsync(2))
    o.tick(2)
    assert_nodes_close(nodes, oracle_nodes(o, nodes), 3, rtol=1e-3)
    sim.destroy()


def test_supports_adding_and_removing_forces():
    nodes = make_nodes(40, 3)
    charge = forceManyBody().theta(1e-6)
    sim = make(nodes, 3).stop().force("charge", charge)
    o = cpu_twin(sim, nodes, 3, [charge])
    run(sim.tickAsync(2))
    o.tick(2)
    fx, fz = forceX(20).strength(0.2), forceZ(-10)
    sim.force("x", fx).force("z", fz)
    o.position(0, 20.0, 0.2)
    o.position(2, -10.0, 0.1)
    run(sim.tickAsync(2))
    o.tick(2)
    sim.force("charge", None)
    o.clear_forces()
    o.position(0, 20.0, 0.2)
    o.position(2, -10.0, 0.1)
    run(sim.tickAsync(2))
    o.tick(2)
    assert_nodes_close(nodes, oracle_nodes(o, nodes), 3, rtol=1e-3, atol=1e-3)
    assert sim.force("charge") is None
    assert sim.isGPUEnabled() is True
    sim.destroy()


def test_replaces_the_nodes_with_nodes():
    first, second = make_nodes(30, 2), make_nodes(70, 2, 100, 999)
    sim = make(first, 2).stop().force("charge", forceManyBody())
    run(sim.tickAsync(2))
    frozen = [n["x"] for n in first]
    sim.nodes(second)
    run(sim.tickAsync(2))
    assert [n["x"] for n in first] == frozen, "old nodes are left alone"
    assert second[69]["index"] == 69
    assert all(math.isfinite(n["x"]) and math.isfinite(n["y"]) for n in second)
    sim.destroy()


def test_changes_dimensionality_with_num_dimensions():
    nodes = make_nodes(30, 3)
    sim = make(nodes, 3).stop().force("charge", forceManyBody())
    run(sim.tickAsync(2))
    assert all(math.isfinite(n["z"]) for n in nodes)
    sim.numDimensions(2)
    z = [n["z"] for n in nodes]
    run(sim.tickAsync(2))
    assert [n["z"] for n in nodes] == z, "z is left alone in 2D"
    assert sim.isGPUEnabled() is True
    sim.destroy()


def test_respects_a_node_pinned_with_fx_fy_fz_and_releases_it():
    nodes = make_nodes(30, 3)
    sim = make(nodes, 3).stop().force("charge", forceManyBody())
    run(sim.tickAsync(2))
    nodes[3]["fx"], nodes[3]["fy"], nodes[3]["fz"] = 11, 12, 13
    run(sim.tickAsync(2))
    assert [nodes[3]["x"], nodes[3]["y"], nodes[3]["z"], nodes[3]["vx"]] == [11, 12, 13, 0]
    nodes[3]["fx"] = 20  # dragged
    run(sim.tickAsync(1))
    assert nodes[3]["x"] == 20
    nodes[3]["fx"] = nodes[3]["fy"] = nodes[3]["fz"] = None  # released
    run(sim.tickAsync(5))
    assert nodes[3]["x"] != 20, "moves again once released"
    sim.destroy()


def test_moves_a_node_whose_xyz_the_user_has_set():
    nodes = make_nodes(30, 3)
    sim = make(nodes, 3).stop().force("x", forceX(0).strength(0))
    run(sim.tickAsync(2))
    nodes[5]["x"], nodes[5]["y"], nodes[5]["z"] = 1000, -1000, 500
    run(sim.tickAsync(1))
    assert [nodes[5]["x"], nodes[5]["y"], nodes[5]["z"]] == [1000, -1000, 500], "no forces: it stays"
    sim.destroy()


def test_keeps_a_users_edit_made_between_a_tick_and_its_readback():
    nodes = make_nodes(30, 3)
    sim = make(nodes, 3).stop().force("x", forceX(0).strength(0))
    run(sim.tickAsync(1))
    sim.tick()  # queued, not yet read back
    nodes[7]["x"] = -777
    run(sim.sync())
    assert nodes[7]["x"] == -777, "not overwritten by the older GPU state"
    run(sim.tickAsync(1))
    assert nodes[7]["x"] == -777
    sim.destroy()


def test_a_force_without_gpu_is_refused_and_the_simulation_keeps_running():
    def gravity():
        state = {}

        def force(alpha):
            for n in state["nodes"]:
                n["vy"] -= 0.5 * alpha

        force.initialize = lambda nodes, *a: state.__setitem__("nodes", nodes)
        return force

    nodes = make_nodes(20, 2)
    sim = make(nodes, 2).stop().force("charge", forceManyBody())
    with pytest.raises(FlError) as e:
        sim.force("gravity", gravity())
    assert e.value.code == FL_E_UNSUPPORTED and "gravity" in str(e.value)
    assert sim.force("gravity") is None
    run(sim.tickAsync(3))
    assert sim.isGPUEnabled() is True
    sim.destroy()


def test_resolves_links_by_id_like_force_link_on_the_cpu():
    def with_links(sim):
        return sim.force("link", forceLink([{"source": "a", "target": "b"}, {"source": "b", "target": "c"}])
                         .id(lambda d, *a: d["name"]).distance(20))

    nodes = [{"name": "a"}, {"name": "b"}, {"name": "c"}]
    sim = with_links(make(nodes, 3).stop())
    run(sim.tickAsync(200))

    def dist(a, b):
        return math.hypot(a["x"] - b["x"], a["y"] - b["y"], a["z"] - b["z"])

    assert abs(dist(nodes[0], nodes[1]) - 20) < 1, dist(nodes[0], nodes[1])
    assert abs(dist(nodes[1], nodes[2]) - 20) < 1
    sim.destroy()


def test_runs_a_link_force_with_no_links():
    nodes = make_nodes(10, 2)
    sim = make(nodes, 2).stop().force("link", forceLink([])).force("charge", forceManyBody())
    run(sim.tickAsync(3))
    assert sim.isGPUEnabled() is True
    assert all(math.isfinite(n["x"]) and math.isfinite(n["y"]) for n in nodes)
    sim.destroy()


def test_runs_with_no_nodes_and_with_nodes_added_afterwards():
    sim = make([], 3).stop().force("charge", forceManyBody()).force("center", forceCenter())
    run(sim.tickAsync(3))
    nodes = make_nodes(20, 3)
    sim.nodes(nodes)
    run(sim.tickAsync(3))
    assert all(math.isfinite(n["x"]) and math.isfinite(n["z"]) for n in nodes)
    sim.nodes([])
    run(sim.tickAsync(1))
    sim.destroy()


def test_reports_when_the_nodes_would_exceed_the_device():
    sim = make(make_nodes(30, 2), 2).stop()
    assert sim._engine.eng.fits(30) is True
    assert sim._engine.eng.fits(1 << 40) is False
    sim.destroy()


def test_keeps_the_passes_of_the_forces_that_stay_when_another_is_added():
    nodes = make_nodes(30, 3)
    links = lambda: [{"source": 2 * i, "target": 2 * i + 1} for i in range(15)]  # disjoint: exact
    link, charge = forceLink(links()), forceManyBody().theta(1e-6)
    sim = make(nodes, 3).stop().force("link", link).force("charge", charge)
    o = cpu_twin(sim, nodes, 3, [link, charge])
    run(sim.tickAsync(2))
    o.tick(2)
    center = forceCenter()
    sim.force("center", center)
    o.center()
    run(sim.tickAsync(2))
    o.tick(2)
    assert_nodes_close(nodes, oracle_nodes(o, nodes), 3, rtol=2e-3, atol=1e-3)
    sim.destroy()


def test_exposes_its_gpu_buffers_for_rendering():
    nodes = make_nodes(25, 3)
    sim = make(nodes, 3).stop().force("charge", forceManyBody())
    run(sim.tickAsync(2))
    b = sim.gpuBuffers()
    assert b["count"] == 25 and b["stride"] == 16
    assert b["positions"] and b["velocities"] and b["positions"] != b["velocities"]
    run(sim.tickAsync(1))
    assert sim.gpuBuffers() == b, "the buffers stay put while the node count does"
    sim.destroy()
    assert sim.gpuBuffers() is None


def test_with_readback_false_keeps_the_nodes_untouched_until_sync():
    nodes = make_nodes(40, 3)
    start = [n["x"] for n in nodes]
    ticks = [0]
    sim = forceSimulationGPU(nodes, 3, {"readback": False}).force("charge", forceManyBody())
    sim.on("tick", lambda _: ticks.__setitem__(0, ticks[0] + 1))
    time.sleep(0.3)
    assert ticks[0] > 2, "tick events still fire (%d)" % ticks[0]
    assert [n["x"] for n in nodes] == start, "nodes are not updated"
    sim.stop()
    run(sim.sync())
    assert any(n["x"] != s for n, s in zip(nodes, start)), "sync() brings them up to date"
    sim.destroy()


@pytest.mark.parametrize("n,ticks", [(2000, 300), (60000, 40)])
def test_is_deterministic_with_the_centre_force(n, ticks):
    """link + charge + center, twice from the same start: bit for bit the same layout. The
    centre's mean is an exact integer sum (independent of the order its blocks add in), the
    tree and its cell sums are exact, and every walk sums in a fixed order."""
    from forcegpu.graphs import benchmark_links

    def once():
        nodes = make_nodes(n, 3, 200)
        src, dst = benchmark_links(n, n // 2, seed=9)
        links = [{"source": int(a), "target": int(b)} for a, b in zip(src, dst)]
        sim = make(nodes, 3).stop().force("link", forceLink(links)).force("charge", forceManyBody()) \
            .force("center", forceCenter(3, -2, 1))
        run(sim.tickAsync(ticks))
        sim.destroy()
        return np.array([(d["x"], d["y"], d["z"], d["vx"], d["vy"], d["vz"]) for d in nodes])

    a, b = once(), once()
    assert np.isfinite(a).all()
    assert np.array_equal(a, b)


def test_is_deterministic_for_a_given_random_source_coincident_nodes():
    def once():
        nodes = [{"x": 0.0, "y": 0.0, "z": 0.0} for _ in range(20)]
        sim = make(nodes, 3).stop().force("charge", forceManyBody()).force("collide", forceCollide(3))
        run(sim.tickAsync(10))
        sim.destroy()
        return [(n["x"], n["y"], n["z"]) for n in nodes]

    a, b = once(), once()
    assert a == b
    assert len(set(a)) == 20, "coincident nodes were separated"


def test_runs_every_tick_of_a_synchronous_batch():
    nodes = make_nodes(40, 3)
    charge = forceManyBody().theta(1e-6)
    sim = make(nodes, 3).stop().force("charge", charge)
    o = cpu_twin(sim, nodes, 3, [charge])
    for _ in range(100):
        sim.tick()
        o.tick(1)
    assert sim.alpha() == o.alpha, "all 100 ticks were taken"
    run(sim.sync())
    assert_nodes_close(nodes, oracle_nodes(o, nodes), 3, rtol=5e-3, atol=5e-3)
    sim.destroy()


def test_takes_a_tick_per_call_even_when_calls_are_spread_out():
    nodes = make_nodes(40, 3)
    sim = make(nodes, 3).stop().force("charge", forceManyBody())
    for _ in range(20):
        sim.tick()
        time.sleep(0.025)
    assert abs(sim.alpha() - (1 - sim.alphaDecay()) ** 20) < 1e-12, sim.alpha()
    sim.destroy()


def test_destroy_stops_everything_and_is_safe_to_call_more_than_once():
    nodes = make_nodes(20, 2)
    sim = make(nodes, 2).force("charge", forceManyBody())
    sim.destroy()
    assert sim.isGPUEnabled() is False
    sim.destroy()
    time.sleep(0.06)
    sim.tick()  # does not raise


class NodeList(list):
    """A list that can be referenced weakly."""


def test_a_destroyed_simulations_nodes_can_be_collected():
    def scope():
        nodes = NodeList(make_nodes(100, 3))
        sim = make(nodes, 3).stop().force("charge", forceManyBody())
        run(sim.tickAsync(2))
        sim.destroy()
        return weakref.ref(nodes)

    ref = scope()
    for _ in range(20):
        if ref() is None:
            break
        gc.collect()
        time.sleep(0.01)
    assert ref() is None, "still reachable"


# --- simulation.find (test/find-test.js) ---

def test_find_finds_the_closest_node_within_a_radius():
    a, b, c = {"x": 5, "y": 0}, {"x": 10, "y": 16}, {"x": -10, "y": -4}
    sim = make([a, b, c], 2).stop()
    assert sim.find(0, 0) is a
    assert sim.find(0, 0, 1) is None
    assert sim.find(0, 20) is b
    sim.destroy()


def test_find_uses_every_dimension_of_a_3d_layout():
    a, b = {"x": 0, "y": 0, "z": 10}, {"x": 0, "y": 0, "z": -3}
    sim = make([a, b], 3).stop()
    assert sim.find(0, 0, 8) is a
    assert sim.find(0, 0, -1) is b
    assert sim.find(0, 0, 4, 2) is None
    sim.destroy()
