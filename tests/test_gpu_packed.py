"""The packed transfers (fl_sync_packed, fl_update_positions_packed): ndim floats per node
across the host link instead of four. They carry exactly the first ndim components of what
fl_sync and fl_update_positions carry, and a layout stepped after a packed upload is the one
stepped after the float4 upload of the same positions, bit for bit."""
import numpy as np
import pytest

from forcegpu._lib import Engine, FlError, desc_from_gpu
from forcegpu.graphs import benchmark_links, make_nodes

pytestmark = pytest.mark.gpu


def engine(n, dims, seed=5):
    xyz = make_nodes(n, dims, 8.0 * n ** (1 / dims), seed=seed)
    pos4 = np.zeros((n, 4), np.float32)
    pos4[:, :dims] = xyz[:, :dims]
    src, dst = benchmark_links(n, n // 2, seed=seed)
    deg = np.bincount(np.concatenate([src, dst]), minlength=n).astype(float)
    forces = [
        {"type": "link", "version": 1, "source": src, "target": dst, "iterations": 1,
         "strengths": 1.0 / np.minimum(deg[src], deg[dst]), "distances": np.full(len(src), 30.0),
         "bias": deg[src] / (deg[src] + deg[dst])},
        {"type": "manyBody", "version": 1, "strengths": np.full(n, -30.0), "distanceMin2": 1.0,
         "distanceMax2": np.inf, "theta2": 0.81},
        {"type": "center", "x": 0, "y": 0, "z": 0, "strength": 1.0},
    ]
    e = Engine(0)
    e.set_nodes(pos4, dims)
    e.set_forces([desc_from_gpu(f, k + 1, n) for k, f in enumerate(forces)])
    e.set_seed(9)
    return e


@pytest.mark.parametrize("dims", [1, 2, 3])
def test_packed_readback_is_the_first_ndim_components(dims):
    n = 7001
    e = engine(n, dims)
    e.enqueue(np.linspace(0.9, 0.7, 4), 0.6)
    p4, v4 = e.sync()
    p, v = e.sync_packed()
    assert p.shape == (n, dims) and v.shape == (n, dims)
    assert np.array_equal(p, p4[:, :dims]) and np.array_equal(v, v4[:, :dims])
    # one side only
    p_only = np.empty((n, dims), np.float32)
    assert e.L.fl_sync_packed(e.h, p_only.ctypes.data, None) == 0
    assert np.array_equal(p_only, p)
    e.close()


@pytest.mark.parametrize("dims", [2, 3])
def test_packed_upload_steps_like_the_float4_upload(dims):
    n = 6000
    a, b = engine(n, dims), engine(n, dims)
    al = np.linspace(0.9, 0.6, 3)
    a.enqueue(al, 0.6)
    b.enqueue(al, 0.6)
    p4, _ = a.sync()
    assert np.array_equal(p4, b.sync()[0])
    rng = np.random.default_rng(3)
    first, count = 1234, 2500
    moved = (p4[first:first + count, :dims] + rng.normal(0, 5, (count, dims))).astype(np.float32)
    full = np.zeros((count, 4), np.float32)
    full[:, :dims] = moved
    a.update_positions(first, full)
    b.update_positions_packed(first, moved)
    pa, pb = a.sync()[0], b.sync()[0]
    assert np.array_equal(pa, pb)
    assert np.array_equal(pb[first:first + count, :dims], moved)
    assert not pb[:, dims:].any()
    a.enqueue(al, 0.6)
    b.enqueue(al, 0.6)
    assert np.array_equal(a.sync()[0], b.sync()[0])
    a.close(), b.close()


def test_packed_calls_check_their_arguments():
    e = engine(1000, 3)
    with pytest.raises(FlError):
        e.update_positions_packed(990, np.zeros((20, 3), np.float32))
    with pytest.raises(ValueError):
        e.sync_packed(np.empty((1000, 4), np.float32), None)
    e.update_positions_packed(0, np.zeros((0, 3), np.float32))  # an empty range is fine
    e.close()


@pytest.mark.parametrize("dims", [2, 3])
def test_a_queued_upload_steps_as_the_waited_one(dims):
    """fl_update_positions_packed_async: the same layout as the waited upload, tick after tick,
    with the host array read in place (it stays unchanged until the next sync)."""
    n = 40000
    rng = np.random.default_rng(3)
    out = []
    for queued in (False, True):
        e = engine(n, dims)
        e.enqueue(np.array([0.9]), 0.6)
        p, _ = (x.copy() for x in e.sync_packed())
        for k in range(4):
            up = np.ascontiguousarray(p + rng.normal(0.0, 0.5, p.shape).astype(np.float32)) \
                if k == 0 else p.copy()
            if queued:
                e.update_positions_packed_async(0, up)
            else:
                e.update_positions_packed(0, up)
            e.enqueue(np.array([0.8 - 0.05 * k]), 0.6)
            p, v = (x.copy() for x in e.sync_packed())
        out.append((p, v))
        e.close()
        rng = np.random.default_rng(3)
    np.testing.assert_array_equal(out[0][0], out[1][0])
    np.testing.assert_array_equal(out[0][1], out[1][1])


def test_a_queued_upload_wants_an_array_it_can_read_in_place():
    e = engine(1000, 3)
    with pytest.raises(ValueError):
        e.update_positions_packed_async(0, np.zeros((1000, 3), np.float64))
    with pytest.raises(ValueError):
        e.update_positions_packed_async(0, np.zeros((3, 1000), np.float32).T)
    e.close()
