"""The layout server: continuous batching of jobs that arrive while others run.

A job's result must not depend on which other jobs share the GPU with it: the same job laid
out alone and in a mix (joining a running batch, with jobs leaving around it) gives the same
layout within the tolerance of the other GPU tests."""
import numpy as np
import pytest

from forcegpu.graphs import benchmark_links, make_nodes
from forcegpu.serve import Job, LayoutServer, latency_summary
from gpu_helpers import tree_outliers

pytestmark = pytest.mark.gpu


def job(n, dims, seed, ticks, radii=False, arrival=0.0):
    xyz = make_nodes(n, dims, 150.0 + n, seed)[:, :dims]
    src, dst = benchmark_links(n, n // 2, seed=seed)
    r = (1.0 + (np.arange(n) % 5)).astype(float) if radii else None
    return Job(xyz=xyz, source=src, target=dst, ticks=ticks, radii=r, arrival=arrival)


def close(a, b, outliers, rtol=1e-3):
    tol = 1e-3 + rtol * np.maximum(1.0, np.maximum(np.abs(a), np.abs(b)))
    bad = np.any(np.abs(a - b) > tol, axis=1)
    return np.isfinite(a).all() and bad.sum() <= outliers


class FakeClock:
    """Time that advances by one step per server round, so arrivals land mid-run."""

    def __init__(self):
        self.t = 0.0

    def __call__(self):
        self.t += 1.0
        return self.t


@pytest.mark.parametrize("dims", [2, 3])
def test_a_job_alone_and_in_the_mix_gives_the_same_layout(dims):
    """300 ticks, in blocks of 10, with the mix changing around the job: others join the running
    batch and leave it while it runs. Every sum of a layout is its own (exact integer centre
    sums, cell sums at the layout's own scale, walk groups from its own first point, jiggles
    from its own ids and tick count), so the layout comes out bit for bit the same; a force
    layout is chaotic, and any difference in a last bit would have grown by orders of
    magnitude over 300 ticks."""
    ticks = 300
    alone = LayoutServer(block=10, clock=FakeClock())
    me = alone.submit(job(600, dims, 11, ticks))
    alone.run_until_idle()
    alone.close()
    # the same job in a mix: it joins a running batch, others join and leave while it runs
    srv = LayoutServer(block=10, clock=FakeClock())
    srv.submit(job(300, dims, 12, 60, arrival=0.0))
    srv.submit(job(1500, dims, 13, 200, radii=True, arrival=0.0))
    mine = srv.submit(job(600, dims, 11, ticks, arrival=3.0))
    srv.submit(job(50, dims, 14, 50, arrival=6.0))
    srv.submit(job(900, dims, 15, 120, arrival=9.0))
    srv.submit(job(2000, dims, 16, 100, arrival=17.0))
    srv.run_until_idle()
    srv.close()
    assert all(j.result is not None for j in srv.finished)
    assert len(srv.finished) == 6
    assert mine.done_ticks == ticks
    assert np.isfinite(me.result).all()
    assert np.array_equal(mine.result, me.result)


def test_admission_waits_for_memory_to_free_up():
    a, b = job(2000, 3, 21, 30), job(2000, 3, 22, 30)
    srv = LayoutServer(block=10, hbm_budget=a.footprint + b.footprint // 2, clock=FakeClock())
    srv.submit(a)
    srv.submit(b)
    srv.run_until_idle()
    srv.close()
    assert a.finished is not None and b.finished is not None
    assert b.admitted >= a.finished, "the second job waits for the first one's memory"


def test_jobs_with_collide_join_the_batch():
    """Jobs with a collide force run in the same batch as the others (the batch's grid keys each
    graph's cells apart), no plain engine of their own."""
    srv = LayoutServer(block=10, clock=FakeClock())
    with_collide = srv.submit(job(400, 3, 31, 20, radii=True))
    without = srv.submit(job(400, 3, 32, 20))
    srv.step()
    assert not srv.plain, "no job runs on a plain engine of its own"
    srv.run_until_idle()
    srv.close()
    for j in (with_collide, without):
        assert j.result is not None and np.isfinite(j.result).all()
        assert j.result.shape == (400, 3)
    s = latency_summary(srv.finished)
    assert s["jobs"] == 2 and s["p99_s"] >= s["p50_s"] > 0


@pytest.mark.parametrize("dims,radii", [(2, False), (3, False), (3, True)])
def test_a_served_job_matches_the_oracle(dims, radii):
    """A job served among others (it joins a running batch, others join and leave around it)
    against the reference's CPU simulation of the same job alone: link and collide in their
    Jacobi form, as the GPU applies them, the forces in the job's order (link, many-body,
    collide, centre), d3's alpha schedule; 4 ticks in blocks of 2 (a force layout is chaotic,
    so a comparison with the FP64 CPU holds for a few ticks)."""
    import oracle
    from gpu_helpers import tree_outliers
    ticks = 4
    srv = LayoutServer(block=2, clock=FakeClock())
    srv.submit(job(300, dims, 41, 2, arrival=0.0))
    srv.submit(job(1500, dims, 42, 8, radii=radii, arrival=0.0))
    mine = job(700, dims, 43, ticks, radii=radii, arrival=2.0)
    if radii:
        mine.xyz = np.float32(mine.xyz * 0.2).astype(float)  # dense: overlaps to push apart
    srv.submit(mine)
    srv.submit(job(80, dims, 44, 3, arrival=4.0))
    srv.run_until_idle()
    srv.close()
    assert mine.done_ticks == ticks
    n = mine.n
    xyz = np.zeros((n, 3))
    xyz[:, :dims] = mine.xyz
    o = oracle.OracleSim(n, dims, xyz=xyz)
    o.link(mine.source, mine.target, mode=oracle.MODE_JACOBI)
    o.manybody(theta=mine.theta)
    if radii:
        o.collide(np.asarray(mine.radii, float), 1.0, 1, oracle.MODE_JACOBI)
    o.center()
    o.tick(ticks)
    want = o.state()[0][:, :dims]
    tol = 1e-3 + 1e-3 * np.maximum(1.0, np.maximum(np.abs(mine.result), np.abs(want)))
    bad = np.any(np.abs(mine.result - want) > tol, axis=1)
    assert np.isfinite(mine.result).all()
    assert bad.sum() <= tree_outliers(n) + (n // 200 if radii else 0), (
        bad.sum(), np.abs(mine.result - want).max())
