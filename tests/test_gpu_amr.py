"""GPU regrid (balance, split, merge, rebuild, neighbour table) vs the oracle."""
import ctypes

import numpy as np
import pytest

from tests import _oracle as O

pytestmark = pytest.mark.gpu


def cfg(**kw):
    from fluidloom_gb300.amr import AdaptConfig
    return AdaptConfig.make(**kw)


def mesh(ctx, cols, capacity=None):
    from fluidloom_gb300.amr import Mesh
    return Mesh(ctx, cols, capacity=capacity)


def one(x, y, z, level, flag):
    return {"x": np.array(x, np.int32), "y": np.array(y, np.int32), "z": np.array(z, np.int32),
            "level": np.array(level, np.uint8), "state": np.zeros(len(x), np.uint8),
            "flags": np.array(flag, np.int32), "material": np.zeros(len(x), np.uint32)}


def run_adapt(ctx, cols, c, fields=None, C=0):
    from fluidloom_gb300 import DeviceArray
    from fluidloom_gb300.amr import AdaptStats
    m = mesh(ctx, cols)
    st = AdaptStats()
    fp = ctypes.c_void_p(0)
    keep = None
    if C:
        keep = DeviceArray.from_host(ctx, np.ascontiguousarray(fields, np.float32))
        # ownership passes to the library (it frees the old field buffer)
        fp = ctypes.c_void_p(keep.ptr.value)
        keep.ptr = None
    rc = ctx.lib.fl_adapt(ctx.handle, ctypes.byref(m.m), ctypes.byref(c), ctypes.byref(fp), C, ctypes.byref(st))
    out = m.download()
    of = None
    if C:
        of = np.empty((m.n, C), np.float32)
        ctx.call("fl_memcpy_d2h", of.ctypes.data_as(ctypes.c_void_p), fp, ctypes.c_size_t(of.nbytes))
        ctx.lib.fl_device_free(ctx.handle, fp)
    return rc, out, st, of


def test_reference_kats(ctx):
    # SplitEngineTest.cpp:35-63, MergeEngineTest.cpp:35-71, AdaptationIntegrationTest.cpp:62-128
    rc, out, st, _ = run_adapt(ctx, one([0], [0], [0], [0], [1]), cfg(balance_mode=1))
    assert rc == 0 and len(out["x"]) == 8 and (out["level"] == 1).all() and st.num_split == 1
    out["flags"][:] = -1
    rc, out2, st2, _ = run_adapt(ctx, out, cfg(balance_mode=1))
    assert rc == 0 and len(out2["x"]) == 1 and out2["level"][0] == 0 and st2.num_groups == 1
    # BalanceEnforcerTest.cpp:37-93 (8-level anchors)
    from fluidloom_gb300.amr import BalanceResult
    m = mesh(ctx, one([0, 4], [0, 0], [0, 0], [1, 3], [0, 0]))
    r = BalanceResult()
    ctx.call("fl_balance_enforce", ctypes.byref(m.m), ctypes.byref(cfg(max_level=8, anchor=8, balance_mode=0)),
             ctypes.byref(r))
    assert r.converged == 1 and r.total_violations_detected > 0 and r.total_cells_marked_for_balance > 0
    assert m.download()["flags"].tolist() == [1, 0]


@pytest.mark.parametrize("seed,mode,shuffled", [(1, 0, False), (2, 0, False), (3, 1, False), (4, 1, False),
                                                (5, 1, False), (6, 0, True), (7, 1, True), (8, 1, True)])
def test_adapt_vs_oracle(ctx, seed, mode, shuffled):
    """Shuffled meshes exercise the locator's own sort and the key-order emission."""
    cols = O.random_octree(seed, ext=(2, 2, 1), rounds=4, max_level=6, frac=0.3, balanced=True)
    rng = np.random.default_rng(seed)
    n = len(cols["x"])
    cols["flags"] = rng.choice([-1, 0, 1, 2], n, p=[0.55, 0.25, 0.15, 0.05]).astype(np.int32)
    cols["state"] = (rng.random(n) < 0.03).astype(np.uint8)
    C = 5
    f = rng.standard_normal((n, C)).astype(np.float32)
    if shuffled:
        perm = rng.permutation(n)
        cols = {k: np.ascontiguousarray(v[perm]) for k, v in cols.items()}
        f = np.ascontiguousarray(f[perm])
    kw = dict(max_level=6, min_level=1, balance_mode=mode, max_balance_iterations=10, enforce_balance=1,
              averaging_rule=seed % 2)
    want, wst, wf, *_ = O.adapt(cols, kw, O.domain(ext=(2, 2, 1), max_level=6), f, C)
    rc, got, st, gf = run_adapt(ctx, cols, cfg(max_level=6, min_level=1, balance_mode=mode, rule=seed % 2,
                                               ext=(2, 2, 1)), f, C)
    assert rc in (0, -5)
    for k in ("x", "y", "z", "level", "state", "flags", "material"):
        np.testing.assert_array_equal(got[k], want[k], err_msg=k)
    np.testing.assert_array_equal(gf, wf)  # bit-exact: same copies and the same ordered sums
    assert (st.num_split, st.num_groups, st.num_survivors) == (wst.num_split, wst.num_groups, wst.num_survivors)
    assert st.balance.converged == wst.balance.converged
    assert st.balance.total_violations_detected == wst.balance.violations
    assert st.balance.total_cells_marked_for_balance == wst.balance.marked


@pytest.mark.parametrize("seed,shuffled", [(21, False), (22, False), (23, True)])
def test_input_balanced_hint_equals_full_probing(ctx, seed, shuffled):
    """An adapt whose FULL26 balance converged leaves no two touching leaves more than one
    level apart.  A second adapt of its output with input_balanced set (the first round
    probes only from the leaves that will split) equals the same adapt without it -- leaves,
    flags and every statistic -- and both equal the oracle."""
    cols = O.random_octree(seed, ext=(2, 2, 1), rounds=4, max_level=6, frac=0.3, balanced=True)
    rng = np.random.default_rng(seed)
    cols["flags"] = rng.choice([-1, 0, 1], len(cols["x"]), p=[0.3, 0.4, 0.3]).astype(np.int32)
    # a balanced start below the maximum level: every violator can split, the balance converges
    rc, out, st, _ = run_adapt(ctx, cols, cfg(max_level=8, balance_mode=1, ext=(2, 2, 1)))
    assert rc == 0 and st.balance.converged == 1
    n = len(out["x"])
    out["flags"] = rng.choice([-1, 0, 1], n, p=[0.45, 0.35, 0.2]).astype(np.int32)
    if shuffled:
        perm = rng.permutation(n)
        out = {k: np.ascontiguousarray(v[perm]) for k, v in out.items()}
    runs = []
    for hint in (False, True):
        rc, got, gst, _ = run_adapt(ctx, {k: v.copy() for k, v in out.items()},
                                    cfg(max_level=8, balance_mode=1, ext=(2, 2, 1), input_balanced=hint))
        assert rc == 0
        runs.append((got, gst))
    (a, sa), (b, sb) = runs
    for k in ("x", "y", "z", "level", "state", "flags", "material"):
        np.testing.assert_array_equal(b[k], a[k], err_msg=k)
    assert (sb.num_split, sb.num_groups, sb.num_survivors) == (sa.num_split, sa.num_groups, sa.num_survivors)
    assert (sb.balance.converged, sb.balance.iterations, sb.balance.total_violations_detected,
            sb.balance.total_cells_marked_for_balance) == (sa.balance.converged, sa.balance.iterations,
                                                           sa.balance.total_violations_detected,
                                                           sa.balance.total_cells_marked_for_balance)
    assert sa.balance.total_cells_marked_for_balance > 0  # the balance has work to do
    kw = dict(max_level=8, min_level=0, balance_mode=1, max_balance_iterations=10, enforce_balance=1,
              averaging_rule=0)
    want, wst, *_ = O.adapt(out, kw, O.domain(ext=(2, 2, 1), max_level=8))
    for k in ("x", "y", "z", "level", "state", "flags", "material"):
        np.testing.assert_array_equal(b[k], want[k], err_msg=k)
    assert sb.balance.total_cells_marked_for_balance == wst.balance.marked


@pytest.mark.parametrize("mode,shuffled", [(0, False), (1, False), (1, True)])
def test_balance_vs_oracle(ctx, mode, shuffled):
    from fluidloom_gb300.amr import BalanceResult
    cols = O.random_octree(10 + mode, ext=(2, 1, 1), rounds=3, max_level=6, frac=0.3, balanced=False)
    rng = np.random.default_rng(mode)
    cols["flags"] = (rng.random(len(cols["x"])) < 0.2).astype(np.int32)
    if shuffled:
        perm = rng.permutation(len(cols["x"]))
        cols = {k: np.ascontiguousarray(v[perm]) for k, v in cols.items()}
    wf, wst = O.balance(cols, O.domain(ext=(2, 1, 1), max_level=7), mode, 7)
    m = mesh(ctx, cols)
    r = BalanceResult()
    rc = ctx.lib.fl_balance_enforce(ctx.handle, ctypes.byref(m.m),
                                    ctypes.byref(cfg(max_level=7, balance_mode=mode, ext=(2, 1, 1))), ctypes.byref(r))
    assert rc in (0, -5)
    np.testing.assert_array_equal(m.download()["flags"], wf)
    assert (r.converged, r.iterations, r.total_violations_detected, r.total_cells_marked_for_balance) == \
        (wst.converged, wst.iterations, wst.violations, wst.marked)


@pytest.mark.parametrize("order", ["key order", "shuffled"])
@pytest.mark.parametrize("sub,periodic", [(1, (0, 0, 0)), (4, (0, 0, 0)), (4, (1, 0, 1))])
def test_neighbours_vs_oracle(ctx, sub, periodic, order):
    """The locator sorts the leaves' key runs itself when the mesh is not in key order."""
    from fluidloom_gb300 import DeviceArray
    cols = O.random_octree(20 + sub, ext=(2, 2, 2), rounds=3, max_level=5, frac=0.25, balanced=True)
    if order == "shuffled":  # random_octree builds its leaves in key order
        perm = np.random.default_rng(7).permutation(len(cols["x"]))
        cols = {k: np.ascontiguousarray(v[perm]) for k, v in cols.items()}
    want = O.neighbours(cols, O.domain(ext=(2, 2, 2), max_level=5, periodic=periodic), sub)
    m = mesh(ctx, cols)
    nbr = DeviceArray(ctx, (len(cols["x"]) * 26 * sub,), np.uint32)
    ctx.call("fl_neighbour_rebuild", ctypes.byref(m.m),
             ctypes.byref(cfg(max_level=5, ext=(2, 2, 2), periodic=periodic)), sub, nbr.ptr)
    np.testing.assert_array_equal(nbr.to_host(), want)


def test_adapt_empty_and_growth(ctx):
    rc, out, st, _ = run_adapt(ctx, one([], [], [], [], []), cfg())
    assert rc == 0 and len(out["x"]) == 0
    c = O.uniform_mesh(2, (1, 1, 1))
    c["flags"][:] = 1
    from fluidloom_gb300.amr import Mesh, AdaptStats
    m = Mesh(ctx, c, capacity=64)
    st = AdaptStats()
    fp = ctypes.c_void_p(0)
    ctx.call("fl_adapt", ctypes.byref(m.m), ctypes.byref(cfg(balance_mode=1)), ctypes.byref(fp), 0, ctypes.byref(st))
    assert m.n == 512 and m.m.capacity == max(int(512 * 1.5), 512 + 1024)
