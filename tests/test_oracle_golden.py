"""The oracle against the reference's CPU known answers (tests/golden/known_answers.json).

Mirrors test/simulation-test.js, test/center-test.js, test/collide-test.js and test/x-test.js of
the reference, plus the published layout sizes of docs/differences.md:35-40 (which pin the
many-body force's d3 tree semantics: the reference has no CPU known answer for it)."""
import json
import os

import numpy as np
import pytest

import oracle

GOLD = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "known_answers.json")))
TOL = GOLD["tolerance_abs"]
NAN = float("nan")


def check(x, v, i, expect):
    for k, a in (("x", x[i, 0]), ("y", x[i, 1]), ("vx", v[i, 0]), ("vy", v[i, 1])):
        if k in expect:
            assert abs(a - expect[k]) < TOL, (i, k, a, expect[k])


def test_phyllotaxis_2d():
    x, v = oracle.OracleSim(3, 2).state()
    for i, e in enumerate(GOLD["phyllotaxis_2d"]):
        check(x, v, i, e["expect"])


def test_center_repositions_nodes():
    xyz = np.array([[100, 0, 0], [200, 0, 0], [300, 0, 0]], float)
    s = oracle.OracleSim(3, 2, xyz=xyz)
    s.center(0, 0)
    x, v = s.tick().state()
    for i, e in enumerate(GOLD["center"][:3]):
        check(x, v, i, e["expect"])


def test_center_respects_fixed_positions():
    f = np.zeros((3, 3))
    s = oracle.OracleSim(3, 2, fxyz=f, fmask=np.array([7, 0, 0], np.uint8))
    s.center()
    x, v = s.tick().state()
    check(x, v, 0, GOLD["center"][3]["expect"])


def test_collide_collides_nodes():
    s = oracle.OracleSim(3, 2)
    s.collide(1.0)
    x, v = s.tick(10).state()
    for i, e in enumerate(GOLD["collide"][:3]):
        check(x, v, i, e["expect"])
    s.clear_forces()
    s.collide(100.0)
    x, v = s.tick(10).state()
    for i, e in enumerate(GOLD["collide"][3:6]):
        check(x, v, i, e["expect"])


def test_collide_respects_fixed_positions():
    s = oracle.OracleSim(3, 2, fxyz=np.zeros((3, 3)), fmask=np.array([3, 0, 0], np.uint8))
    s.collide(1.0)
    x, v = s.tick(10).state()
    check(x, v, 0, GOLD["collide"][6]["expect"])
    s.clear_forces()
    s.collide(100.0)
    x, v = s.tick(10).state()
    check(x, v, 0, GOLD["collide"][7]["expect"])


def test_collide_jiggles_equal_positions():
    s = oracle.OracleSim(2, 2, xyz=np.zeros((2, 3)))
    s.collide()
    x, v = s.tick().state()
    assert x[0, 0] != x[1, 0] and x[0, 1] != x[1, 1]
    assert v[0, 0] == -v[1, 0] and v[0, 1] == -v[1, 1]


def test_collide_jiggles_reproducibly():
    """The LCG stream and the quadtree visit order, pinned by one number pair."""
    s = oracle.OracleSim(10, 2, xyz=np.zeros((10, 3)))
    s.collide()
    x, v = s.tick(50).state()
    check(x, v, 0, GOLD["collide"][8]["expect"])


def test_force_x_centers_nodes():
    xyz = np.array([[100, 0, 0], [200, 0, 0], [300, 0, 0]], float)
    s = oracle.OracleSim(3, 2, xyz=xyz)
    s.position(0, 200.0)
    x, v = s.tick(30).state()
    assert x[0, 0] > 190 and v[0, 0] > 0
    assert x[1, 0] == 200 and v[1, 0] == 0
    assert x[2, 0] < 210 and v[2, 0] < 0


def test_force_y_centers_nodes():
    xyz = np.array([[0, 100, 0], [0, 200, 0], [0, 300, 0]], float)
    s = oracle.OracleSim(3, 2, xyz=xyz)
    s.position(1, 200.0)
    x, v = s.tick(30).state()
    assert x[0, 1] > 190 and v[0, 1] > 0
    assert x[1, 1] == 200 and v[1, 1] == 0
    assert x[2, 1] < 210 and v[2, 1] < 0


def test_alpha_schedule():
    """alpha after k ticks with alphaTarget 0 is (1 - alphaDecay)^k (gpu-simulation-test.js:481-488)."""
    s = oracle.OracleSim(5, 2)
    s.tick(20)
    decay = 1 - 0.001 ** (1 / 300)
    assert abs(s.alpha - (1 - decay) ** 20) < 1e-12


def benchmark_graph(n):
    """examples/benchmark.html:86-93: a random tree, then n/2 random pairs, LCG seed 42."""
    s = 42
    links = []

    def rnd():
        nonlocal s
        s = (s * 1664525 + 1013904223) % 4294967296
        return s / 4294967296

    for i in range(1, n):
        links.append((i, int(rnd() * i)))
    for _ in range(n // 2):
        links.append((int(rnd() * n), int(rnd() * n)))
    return np.array(links, dtype=np.int32)


@pytest.mark.parametrize("dims,theta_index", [(d, t) for d in (2, 3) for t in range(4)])
def test_published_layout_sizes(dims, theta_index):
    """RMS radius after 300 ticks of link(30) + charge + center on the 1,000-node graph: the
    CPU row of docs/differences.md:35-40, to the published integer."""
    lay = GOLD["layout_rms_radius"]
    links = benchmark_graph(lay["nodes"])
    s = oracle.OracleSim(lay["nodes"], dims)
    s.link(links[:, 0], links[:, 1], distance=lay["link_distance"])
    s.manybody(theta=lay["thetas"][theta_index])
    s.center()
    x, _ = s.tick(lay["ticks"]).state()
    rms = float(np.sqrt((x ** 2).sum(1).mean()))
    assert round(rms) == lay["values"]["%dD_CPU" % dims][theta_index], rms


def test_manybody_tree_converges_to_exact():
    """theta -> 0 opens every cell: the tree force equals the FP64 all-pairs sum."""
    rng = np.random.default_rng(3)
    xyz = rng.uniform(-100, 100, (200, 3))
    strengths = np.where(np.arange(200) % 3 == 0, 15.0, -25.0)
    out = []
    for mode in (oracle.MODE_D3, oracle.MODE_EXACT):
        s = oracle.OracleSim(200, 3, xyz=xyz)
        s.manybody(strengths, distanceMin=5, distanceMax=150, theta=1e-3, mode=mode)
        s.apply_force(0, 0.7)
        out.append(s.state()[1])
    np.testing.assert_allclose(out[0], out[1], rtol=1e-9, atol=1e-12)


def test_link_defaults():
    """count, bias and the default strength 1 / min(count) of src/link.js:30-32, :65-75."""
    s = oracle.OracleSim(4, 2)
    k = s.link([0, 0, 1], [1, 2, 3])
    bias, st = s.link_params(k, 3)
    # counts: 0 -> 2, 1 -> 2, 2 -> 1, 3 -> 1
    np.testing.assert_allclose(bias, [2 / 4, 2 / 3, 2 / 3])
    np.testing.assert_allclose(st, [1 / 2, 1 / 1, 1 / 1])
