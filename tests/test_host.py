"""Host-side logic without a GPU: the synthetic workloads, the force descriptors (accessors,
defaults, versions) against the oracle's restatement of the reference's forces."""
import math

import numpy as np
import pytest

import oracle
from forcegpu import forceCollide, forceLink, forceManyBody, forceRadial, forceX, forceZ
from forcegpu._lib import FORCE_TYPES, desc_from_gpu
from forcegpu.graphs import LCG, benchmark_links, link_defaults, make_nodes, phyllotaxis


def reference_lcg(seed, k):
    s, out = seed, []
    for _ in range(k):
        s = (s * 1664525 + 1013904223) % 4294967296
        out.append(s / 4294967296)
    return out


def test_lcg_matches_the_reference_stream():
    assert np.array_equal(LCG(42).draw(10000), reference_lcg(42, 10000))
    g = LCG(1)
    a = g.draw(3)
    b = g.draw(5000)
    assert np.array_equal(np.concatenate([a, b]), reference_lcg(1, 5003))


def test_make_nodes_is_f32_exact_and_matches_reference_formula():
    xyz = make_nodes(50, 3, 200, 12345)
    u = reference_lcg(12345, 150)
    exp = [float(np.float32((float(np.float32(v)) - 0.5) * 200)) for v in u]
    assert np.array_equal(xyz.reshape(-1), exp)


@pytest.mark.parametrize("n", [2, 10, 1000, 20000])
def test_benchmark_links_shape(n):
    src, dst = benchmark_links(n)
    m = len(src)
    assert m == (n - 1) + min(n // 2, n * (n - 1) // 2 - (n - 1))
    assert (src != dst).all()
    keys = np.minimum(src, dst).astype(np.int64) * n + np.maximum(src, dst)
    assert len(np.unique(keys)) == m, "no duplicate links"
    assert (src[:n - 1] == np.arange(1, n)).all() and (dst[:n - 1] < src[:n - 1]).all(), "a random tree"
    u = reference_lcg(42, n - 1)
    assert (dst[:n - 1] == [math.floor(u[i - 1] * i) for i in range(1, n)]).all()


def test_link_defaults_match_oracle():
    n = 500
    src, dst = benchmark_links(n)
    o = oracle.OracleSim(n, 3)
    k = o.link(src, dst)
    bias, st = o.link_params(k, len(src))
    b2, s2 = link_defaults(n, src, dst)
    np.testing.assert_allclose(bias, b2, rtol=0, atol=0)
    np.testing.assert_allclose(st, s2, rtol=0, atol=0)


def test_force_link_descriptor_matches_oracle():
    n = 300
    src, dst = benchmark_links(n)
    nodes = [{"index": i} for i in range(n)]
    f = forceLink([{"source": int(a), "target": int(b)} for a, b in zip(src, dst)])
    f.initialize(nodes, None, 3)
    g = f.gpu()
    bias, st = link_defaults(n, src, dst)
    assert np.array_equal(g["bias"], bias) and np.array_equal(g["strengths"], st)
    assert g["distances"] == [30.0] * len(src) and g["iterations"] == 1
    v = g["version"]
    f.distance(10)
    assert f.gpu()["version"] == v + 1


def test_force_link_resolves_ids():
    nodes = [{"name": "a", "index": 0}, {"name": "b", "index": 1}, {"name": "c", "index": 2}]
    f = forceLink([{"source": "a", "target": "b"}, {"source": "b", "target": "c"}]).id(lambda d, *a: d["name"])
    f.initialize(nodes, None, 3)
    assert [l["source"]["index"] for l in f.links()] == [0, 1]
    with pytest.raises(KeyError):
        forceLink([{"source": "a", "target": "zz"}]).id(lambda d, *a: d["name"]).initialize(nodes, None, 3)


def test_descriptors_convert():
    nodes = [{"index": i} for i in range(4)]
    for f in (forceManyBody().strength(lambda d, i, *a: -i), forceCollide(3), forceRadial(5),
              forceX(2), forceZ(1)):
        f.initialize(nodes, None, 3)
        d, keep = desc_from_gpu(f.gpu(), id(f), 4)
        assert d.type == FORCE_TYPES[f.gpu()["type"]]
    m = forceManyBody().theta(0.5).distanceMax(100)
    m.initialize(nodes, None, 3)
    d, _ = desc_from_gpu(m.gpu(), 1, 4)
    assert d.theta2 == 0.25 and d.distance_max2 == 10000 and d.distance_min2 == 1


def test_radial_and_x_zero_strength_where_target_is_nan():
    nodes = [{"index": i} for i in range(3)]
    r = forceRadial(lambda d, i, *a: float("nan") if i == 1 else 10).strength(0.5)
    r.initialize(nodes, None, 2)
    assert r.gpu()["strengths"] == [0.5, 0.0, 0.5]
    x = forceX(lambda d, i, *a: None if i == 2 else 1)
    x.initialize(nodes, None, 2)
    assert x.gpu()["strengths"] == [0.1, 0.1, 0.0]


def test_phyllotaxis_matches_oracle():
    for dims in (1, 2, 3):
        x, _ = oracle.OracleSim(100, dims).state()
        np.testing.assert_allclose(phyllotaxis(100, dims), x, rtol=1e-14, atol=1e-12)


def test_oracle_integer_rebuild_self_consistent():
    """Morton codes: the d3 child order (bit k of a level = coordinate k in the upper half)."""
    pos = np.zeros((4, 4), np.float32)
    pos[:, :3] = [[0.1, 0.1, 0.1], [0.9, 0.1, 0.1], [0.1, 0.9, 0.1], [0.1, 0.1, 0.9]]
    codes = oracle.morton(pos, 3)
    top = codes >> np.uint64(60)  # the first level's 3 bits
    assert list(top) == [0, 1, 2, 4]
    perm = oracle.sort_perm(codes)
    left, right, depth = oracle.karras(codes[perm], 3)
    assert len(left) == 3 and depth[0] == 0
    row, other, code = oracle.csr(3, [0, 1], [1, 2])
    assert list(row) == [0, 1, 3, 4] and list(other) == [1, 0, 2, 1] and list(code) == [0, 1, 2, 3]
