"""Parity at the benchmark configurations, on the GPU against the oracle.

Config 1: the lid-driven cavity (32^3 sites, max level 2, lid 0.05 +x on the top
  z face, tau 0.56), 200 steps with a vorticity regrid every 20: bricks,
  neighbour rows and populations equal at steps 20, 100 and 200; the FP32
  populations' error against an FP64 run of the next steps is bounded.
Config 2: the flow past a sphere at full size (128x64x64 base, 3 levels, r = 8
  at (32,32,32), inlet 0.04, tau 0.56): 25 steps, a regrid, one more step, all
  equal.
Config 3: the regrid microbenchmark's two-regrid blob octree (microbench_mesh):
  exact against the oracle at 2^18 leaves (the oracle's single-threaded
  balance takes seconds there, hours at 2^24), and at the full 2^24 leaves
  the size-independent properties: the output tiles the domain in strictly
  increasing key order, every leaf's 26 neighbours are within one level,
  balance iterated to a fixed point (a second balance marks nothing), and a
  second run is bitwise identical."""
import ctypes

import numpy as np
import pytest

from fluidloom_gb300.lbm import Pool, cavity
from tests import _oracle as O

pytestmark = pytest.mark.gpu


def _same_bricks(gp, op):
    g, o = gp.bricks(), op.bricks()
    for k in ("x", "y", "z", "level", "case_id"):
        assert np.array_equal(g[k], o[k]), k


def test_config1_cavity_200_steps(ctx):
    case = cavity(32, 2, u_lid=0.05, tau=0.56)
    gp, op = Pool(ctx, [case]), O.OraclePool([case])
    for s in range(1, 201):
        gp.step(1)
        op.step(1)
        if s % 20 == 0:
            gp.regrid()
            op.regrid()
        if s in (20, 100, 200):
            _same_bricks(gp, op)
            assert np.array_equal(gp.nbr(), op.nbr())
            g, o = gp.populations(), op.populations()
            np.testing.assert_allclose(g, o, rtol=1e-5, atol=0)   # FP32 vs FP32 oracle (observed: equal)
            assert np.array_equal(g, o)
    levels = np.bincount(gp.bricks()["level"], minlength=3)
    assert (levels > 0).all()  # all three levels present after the vorticity regrids
    # FP32 against FP64 on the developed mesh: the next 10 steps
    ref = op.fp64_steps(10)
    gp.step(10)
    f = gp.populations().astype(np.float64)
    err = float(np.max(np.abs(f - ref) / np.maximum(np.abs(ref), 1e-30)))
    assert err < 2e-5, err
    gp.close()


def test_config2_sphere_full_size(ctx):
    from bench import sphere_case
    case = sphere_case()
    gp, op = Pool(ctx, [case]), O.OraclePool([case])
    _same_bricks(gp, op)
    gp.step(25)
    op.step(25)
    assert np.array_equal(gp.populations(), op.populations())
    gp.regrid()
    op.regrid()
    _same_bricks(gp, op)
    assert np.array_equal(gp.nbr(), op.nbr())
    gp.step(1)
    op.step(1)
    g, o = gp.populations(), op.populations()
    np.testing.assert_allclose(g, o, rtol=1e-5, atol=0)
    assert np.array_equal(g, o)
    np.testing.assert_allclose(gp.conservation(), op.conservation(), rtol=1e-12, atol=1e-9)
    gp.close()


def test_config2_half_resolution_developing_mesh(ctx):
    """The sphere case with the benchmark's vorticity thresholds at half resolution (64x32x32
    base, 3 levels, r=4) for 100 steps, a regrid every 25: the wake starts to refine (the mesh
    grows past its band refinement) and the GPU pool -- whose regrids after the first state
    their input balanced -- equals the oracle, which probes every leaf, bit for bit at every
    regrid: bricks, neighbour rows, populations."""
    from bench import sphere_case
    case = sphere_case(2)
    gp, op = Pool(ctx, [case]), O.OraclePool([case])
    n0 = gp.info().num_bricks
    for s in range(1, 101):
        gp.step(1)
        op.step(1)
        if s % 25 == 0:
            gp.regrid()
            op.regrid()
            _same_bricks(gp, op)
            assert np.array_equal(gp.nbr(), op.nbr()), s
            assert np.array_equal(gp.populations(), op.populations()), s
    assert gp.info().num_bricks > n0  # the vorticity-driven refinement happened
    np.testing.assert_allclose(gp.conservation(), op.conservation(), rtol=1e-12, atol=1e-9)
    gp.close()


def test_config2_sphere_bulk_staged_equals_register_kernels(ctx):
    """Full-size sphere: the bulk-staged collide kernels (both staging modes) equal the
    register kernels bit for bit over 6 level-0 steps (48 level-3 sub-steps)."""
    from bench import sphere_case
    case = sphere_case()
    ref = Pool(ctx, [case])
    ref.step(6)
    f0 = ref.populations()
    ref.close()
    for mode in (1, 2):
        p = Pool(ctx, [case])
        p.set_options(staging=mode)
        p.step(6)
        assert np.array_equal(p.populations(), f0), mode
        p.close()


# ----------------------------------------------------------------- config 3


def _adapt_gpu(ctx, m, cfg):
    from fluidloom_gb300.amr import AdaptStats
    st = AdaptStats()
    fp = ctypes.c_void_p(0)
    ctx.call("fl_adapt", ctypes.byref(m.m), ctypes.byref(cfg), ctypes.byref(fp), 0, ctypes.byref(st))
    return st


def _gpu_two_regrids(ctx, L, hint=True):
    """The microbenchmark's octree on the GPU: the first regrid from the uniform level-L
    mesh, the second (the timed regrid of the benchmark) from its output -- stated balanced
    when hint is set and the first regrid's balance converged, as the benchmark does."""
    from bench import microbench_mesh
    from fluidloom_gb300.amr import AdaptConfig, Mesh
    mb = microbench_mesh(L)
    m = Mesh(ctx, mb["start"], capacity=1 << (3 * L))
    stats = []
    for blobs, lo, hi, ml in mb["regrids"]:
        ctx.call("fl_flags_from_blobs", ctypes.byref(m.m), blobs.ctypes.data_as(ctypes.c_void_p), len(blobs),
                 ctypes.c_float(lo), ctypes.c_float(hi), ml)
        balanced = hint and bool(stats) and stats[-1].balance.converged == 1
        stats.append(_adapt_gpu(ctx, m, AdaptConfig.make(max_level=ml, min_level=0, balance_mode=1,
                                                         input_balanced=balanced)))
    return m, stats, mb


@pytest.mark.parametrize("hint", [False, True])
def test_config3_microbench_octree_exact_at_2_18(ctx, hint):
    L = 6
    m, stats, mb = _gpu_two_regrids(ctx, L, hint)
    g = m.download()
    c = {k: v.copy() for k, v in mb["start"].items()}
    dom = O.domain(max_level=L + 2)
    for (blobs, lo, hi, ml), gst in zip(mb["regrids"], stats):
        c["flags"] = O.blob_flags(c, blobs, lo, hi, ml)
        c, st, *_ = O.adapt(c, dict(max_level=ml, min_level=0, balance_mode=1, max_balance_iterations=10,
                                    enforce_balance=1, averaging_rule=0), dom)
        c = {k: v.copy() for k, v in c.items()}
        assert (gst.num_split, gst.num_groups, gst.balance.iterations, gst.balance.total_cells_marked_for_balance) == \
            (st.num_split, st.num_groups, st.balance.iterations, st.balance.marked)
    assert stats[1].balance.iterations > 1 and stats[1].balance.total_cells_marked_for_balance > 0
    for k in ("x", "y", "z", "level", "state", "material"):
        assert np.array_equal(g[k], c[k]), k
    # neighbour table of the result (one sub-slot), against the oracle's
    from fluidloom_gb300 import DeviceArray
    from fluidloom_gb300.amr import AdaptConfig
    nbr = DeviceArray(ctx, (m.n * 26,), np.uint32)
    ctx.call("fl_neighbour_rebuild", ctypes.byref(m.m), ctypes.byref(AdaptConfig.make(max_level=L + 2)), 1, nbr.ptr)
    assert np.array_equal(nbr.to_host(), O.neighbours(c, dom, 1))
    m.free()


def test_config3_microbench_octree_properties_at_2_24(ctx):
    from fluidloom_gb300 import DeviceArray
    from fluidloom_gb300.amr import AdaptConfig
    L = 8
    m, stats, _ = _gpu_two_regrids(ctx, L)
    n = m.n
    assert stats[1].balance.iterations > 1 and stats[1].balance.total_cells_marked_for_balance > 0
    cols = m.download()
    A = 21
    # tiling in key order: each leaf's Hilbert run [key, key + 8^(A - level)) starts where the previous one ends
    keys = DeviceArray(ctx, (n,), np.uint64)
    ctx.call("fl_cell_keys", m.m.x, m.m.y, m.m.z, m.m.level, None, 21, A, keys.ptr, ctypes.c_size_t(n))
    span = np.left_shift(np.uint64(1), (3 * (A - cols["level"].astype(np.int64))).astype(np.uint64))
    start = keys.to_host() & ~(span - np.uint64(1))   # the run of a leaf starts at its key with the low bits cleared
    assert start[0] == 0 and int(start[-1]) + int(span[-1]) == 1 << (3 * A)
    assert np.array_equal(start[1:], start[:-1] + span[:-1])
    # 2:1 over faces, edges and corners
    nbr = DeviceArray(ctx, (n * 26,), np.uint32)
    ctx.call("fl_neighbour_rebuild", ctypes.byref(m.m), ctypes.byref(AdaptConfig.make(max_level=L + 2)), 1, nbr.ptr)
    nb = nbr.to_host().reshape(n, 26)
    lv = cols["level"].astype(np.int8)
    for d in range(26):
        j = nb[:, d]
        ok = j != 0xFFFFFFFF
        assert (np.abs(lv[j[ok]] - lv[ok]) <= 1).all(), d
    del nb
    nbr.free()
    # a second balance of the result marks nothing
    from fluidloom_gb300.amr import BalanceResult
    m2cols = dict(cols, flags=np.zeros(n, np.int32))
    from fluidloom_gb300.amr import Mesh
    m2 = Mesh(ctx, m2cols)
    r = BalanceResult()
    ctx.call("fl_balance_enforce", ctypes.byref(m2.m), ctypes.byref(AdaptConfig.make(max_level=L + 2, balance_mode=1)),
             ctypes.byref(r))
    assert r.converged == 1 and r.total_cells_marked_for_balance == 0
    m2.free()
    # run twice: bitwise the same leaves
    m3, stats3, _ = _gpu_two_regrids(ctx, L)
    c3 = m3.download()
    for key in ("x", "y", "z", "level"):
        assert np.array_equal(c3[key], cols[key]), key
    m3.free()
    m.free()
