"""Execution graph on the GPU: step / adapt nodes scheduled by hazards give the
populations of the same operations called directly, with and without CUDA-graph
capture and replay; independent pools run as parallel branches; kernel and host
nodes run in dependency order."""
import ctypes

import numpy as np
import pytest

from fluidloom_gb300 import DeviceArray
from fluidloom_gb300 import graph as G

pytestmark = pytest.mark.gpu


def _cases():
    from fluidloom_gb300 import lbm
    cav = lbm.cavity(16, 1, u_lid=0.06, tau=0.6)
    sph = lbm.sphere_channel(32, 16, 16, 2, radius=2.0, centre=(8.0, 8.0, 8.0), u_in=0.04, band=2.0)
    return cav, sph


def _same(p, q):
    a, b = p.bricks(), q.bricks()
    for k in ("x", "y", "z", "level", "case_id"):
        np.testing.assert_array_equal(a[k], b[k])
    np.testing.assert_array_equal(p.populations(), q.populations())


@pytest.mark.parametrize("cuda_graphs", [False, True])
def test_step_adapt_step_matches_direct_calls(ctx, cuda_graphs):
    from fluidloom_gb300.lbm import Pool
    _, sph = _cases()
    p, ref = Pool(ctx, [sph]), Pool(ctx, [sph])
    g = G.Graph(ctx)
    g.add(G.LBM_STEP, "lbm_a", reads=["f"], writes=["f"], pool=p, nsteps=3)
    g.add(G.ADAPT_MESH, "adapt", reads=["f", "mesh"], writes=["f", "mesh"], pool=p)
    g.add(G.LBM_STEP, "lbm_b", reads=["f", "mesh"], writes=["f"], pool=p, nsteps=2)
    hz = g.analyze()
    assert {(h[0], h[1]) for h in hz} >= {(0, 1), (1, 2)}
    g.build()
    assert g.order() == [0, 1, 2]
    for _ in range(2):
        g.execute(cuda_graphs=cuda_graphs)
        ref.step(3)
        ref.regrid()
        ref.step(2)
        _same(p, ref)


def test_replayed_segments_match_direct_steps(ctx):
    from fluidloom_gb300.lbm import Pool
    cav, _ = _cases()
    p, ref = Pool(ctx, [cav]), Pool(ctx, [cav])
    g = G.Graph(ctx)
    g.add(G.LBM_STEP, "two", reads=["f"], writes=["f"], pool=p, nsteps=2)
    g.add(G.LBM_STEP, "one", reads=["f"], writes=["f"], pool=p, nsteps=1)
    g.analyze()
    g.build()
    counts = []
    for _ in range(4):  # capture, then replays (the level-0 parity alternates: two cached keys)
        c0 = ctx.launch_count()
        g.execute(cuda_graphs=True)
        counts.append(ctx.launch_count() - c0)
        ref.step(3)
    _same(p, ref)
    assert len(set(counts)) == 1 and counts[0] > 0


def test_independent_pools_run_as_branches(ctx):
    from fluidloom_gb300.lbm import Pool
    cav, sph = _cases()
    pa, pb = Pool(ctx, [cav]), Pool(ctx, [sph])
    ra, rb = Pool(ctx, [cav]), Pool(ctx, [sph])
    seen = []
    g = G.Graph(ctx)
    a = g.add(G.LBM_STEP, "cavity", reads=["fa"], writes=["fa"], pool=pa, nsteps=4)
    b = g.add(G.LBM_STEP, "sphere", reads=["fb"], writes=["fb"], pool=pb, nsteps=4)
    j = g.add(G.BARRIER, "join", reads=["fa", "fb"])
    h = g.add(G.HOST, "record", reads=["fa", "fb"], host_fn=lambda: seen.append(1))
    hz = g.analyze()
    assert not any(x[:2] == (a, b) for x in hz)  # no edge between the two pools
    g.build()
    order = g.order()
    assert order.index(j) > max(order.index(a), order.index(b))
    for rnd in range(2):
        g.execute(cuda_graphs=bool(rnd))
        ctx.sync()
        ra.step(4)
        rb.step(4)
    _same(pa, ra)
    _same(pb, rb)
    assert seen == [1, 1]
    assert h in order


def test_kernel_node_enqueues_on_its_stream(ctx):
    n = 100000
    x = np.random.default_rng(3).integers(0, 1000, n).astype(np.uint32)
    src = DeviceArray.from_host(ctx, x)
    dst = DeviceArray(ctx, (n,), np.uint32)
    tot = DeviceArray(ctx, (1,), np.uint32)
    L = ctx.lib

    def scan(stream):
        return L.fl_scan_exclusive_u32_noalloc(src.ptr, dst.ptr, ctypes.c_size_t(n), tot.ptr, stream)

    g = G.Graph(ctx)
    g.add(G.KERNEL, "scan", reads=["x"], writes=["y"], fn=scan)
    g.add(G.BARRIER, "done", reads=["y"])
    g.analyze()
    g.build()
    g.set_profiling(True)
    g.execute(cuda_graphs=False)
    ctx.sync()
    ref = np.concatenate([[0], np.cumsum(x)[:-1]]).astype(np.uint32)
    np.testing.assert_array_equal(dst.to_host(), ref)
    assert int(tot.to_host()[0]) == int(x.sum())
    count, ms = g.stats(0)
    assert count == 1 and ms > 0.0
