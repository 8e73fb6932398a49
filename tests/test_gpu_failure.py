"""Failure detection without a GPU fault: a bounded device wait that nothing
releases runs out, the call reports FL_E_DEVICE_TIMEOUT, and the context keeps
working; host-side bad inputs are rejected before any launch."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_lookback_wait_runs_out_and_context_survives(ctx):
    st = ctx.lib.fl_lookback_timeout_probe(ctx.handle, 2000)
    assert st == -6  # FL_E_DEVICE_TIMEOUT
    from fluidloom_gb300 import DeviceArray
    a = np.arange(100000, dtype=np.uint32)
    d, o = DeviceArray.from_host(ctx, a), DeviceArray(ctx, (100000,), np.uint32)
    ctx.call("fl_scan_exclusive_u32", d.ptr, o.ptr, 100000, None)
    np.testing.assert_array_equal(o.to_host(), np.concatenate([[0], np.cumsum(a[:-1])]).astype(np.uint32))


def test_invalid_inputs_rejected(ctx):
    L = ctx.lib
    assert L.fl_sort_pairs_u64_u32(ctx.handle, None, None, 10, 0, 64) == -1
    assert L.fl_sort_pairs_u64_u32(ctx.handle, None, None, 10, 8, 4) == -1
    assert L.fl_lookback_timeout_probe(ctx.handle, 0) == -1


# ---- allocation failure injected on the host (fl_ctx_inject_alloc_failure) --
# The countdown makes the library's k-th next device allocation fail as out of
# memory without calling CUDA: every k below the call's allocation count hits a
# different allocation site.  Each failing call must return FL_E_OOM (-2) and
# leave the context usable.

FL_E_OOM = -2


def _pool_create(ctx, cases):
    import ctypes
    from fluidloom_gb300.lbm import LbmCase
    arr = (LbmCase * len(cases))(*cases)
    h = ctypes.c_void_p()
    return ctx.lib.fl_pool_create(ctx.handle, arr, len(cases), ctypes.byref(h)), h


def test_pool_create_out_of_memory_at_every_allocation(ctx):
    from fluidloom_gb300.lbm import Pool, cavity
    from tests import _oracle as O
    case = cavity(16, 1)
    failures = 0
    for k in range(200):
        ctx.lib.fl_ctx_inject_alloc_failure(ctx.handle, k)
        rc, h = _pool_create(ctx, [case])
        ctx.lib.fl_ctx_inject_alloc_failure(ctx.handle, -1)
        if rc == 0:
            ctx.lib.fl_pool_destroy(ctx.handle, h)
            break
        assert rc == FL_E_OOM, (k, rc, ctx.lib.fl_last_error(ctx.handle))
        failures += 1
    assert failures > 10 and rc == 0  # every allocation of the creation failed once, then it succeeded
    # the context still works: a pool steps and equals the oracle
    gp, op = Pool(ctx, [case]), O.OraclePool([case])
    gp.step(3)
    op.step(3)
    assert np.array_equal(gp.populations(), op.populations())
    gp.close()


def test_add_cases_out_of_memory(ctx):
    """Every allocation of fl_pool_add_cases fails once.  A failure before the new
    bricks are appended leaves the pool as it was (it keeps stepping like the
    oracle); a failure after it leaves the pool marked unusable, and then every
    call on it is refused on the host without launching anything."""
    from fluidloom_gb300 import FluidLoomError
    from fluidloom_gb300.lbm import Pool, cavity
    from tests import _oracle as O
    a, b = cavity(16, 1, u_lid=0.05), cavity(24, 1, u_lid=0.03)
    outcomes = {"kept": 0, "unusable": 0}
    for k in range(400):
        gp = Pool(ctx, [a])
        gp.step(2)
        ctx.lib.fl_ctx_inject_alloc_failure(ctx.handle, k)
        try:
            gp.add_cases([b])
            ok = True
        except FluidLoomError as e:
            assert e.status == FL_E_OOM, e
            ok = False
        finally:
            ctx.lib.fl_ctx_inject_alloc_failure(ctx.handle, -1)
        if ok:
            break
        if gp.info().usable:
            outcomes["kept"] += 1
            op = O.OraclePool([a])
            op.step(3)
            gp.step(1)
            assert gp.info().num_active_cases == 1
            assert np.array_equal(gp.case_state(0)[1], op.populations()), k
        else:
            outcomes["unusable"] += 1
            for call in (lambda: gp.step(1), gp.populations, gp.regrid, lambda: gp.add_cases([b])):
                with pytest.raises(FluidLoomError) as ei:
                    call()
                assert ei.value.status == -1
        gp.close()
    assert ok and outcomes["kept"] > 0 and outcomes["unusable"] > 0, outcomes
    # the successful add: the resident case untouched, the added one as it would start alone
    op_a, op_b = O.OraclePool([a]), O.OraclePool([b])
    op_a.step(2)
    gp.step(2)
    op_a.step(2)
    op_b.step(2)
    assert np.array_equal(gp.case_state(0)[1], op_a.populations())
    assert np.array_equal(gp.case_state(1)[1], op_b.populations())
    gp.close()


def test_adapt_out_of_memory_leaves_the_mesh(ctx):
    import ctypes
    from fluidloom_gb300.amr import AdaptConfig, AdaptStats, Mesh
    from tests import _oracle as O
    cols = O.random_octree(3, ext=(2, 2, 2), rounds=2, max_level=5, frac=0.3)
    rng = np.random.default_rng(3)
    cols["flags"] = rng.choice([-1, 0, 1], len(cols["x"])).astype(np.int32)
    cfg = AdaptConfig.make(max_level=6, balance_mode=1, ext=(2, 2, 2))
    failures = 0
    for k in range(200):
        m = Mesh(ctx, cols)
        st = AdaptStats()
        fp = ctypes.c_void_p(0)
        ctx.lib.fl_ctx_inject_alloc_failure(ctx.handle, k)
        rc = ctx.lib.fl_adapt(ctx.handle, ctypes.byref(m.m), ctypes.byref(cfg), ctypes.byref(fp), 0, ctypes.byref(st))
        ctx.lib.fl_ctx_inject_alloc_failure(ctx.handle, -1)
        if rc == 0:
            m.free()
            break
        assert rc == FL_E_OOM, (k, rc, ctx.lib.fl_last_error(ctx.handle))
        failures += 1
        # the mesh is the input as it was: a regrid now gives the oracle's result
        assert m.n == len(cols["x"])
        st = AdaptStats()
        ctx.call("fl_adapt", ctypes.byref(m.m), ctypes.byref(cfg), ctypes.byref(fp), 0, ctypes.byref(st))
        out = m.download()
        ref, *_ = O.adapt(cols, dict(max_level=6, min_level=0, balance_mode=1, max_balance_iterations=10,
                                     enforce_balance=1, averaging_rule=0), O.domain(ext=(2, 2, 2), max_level=6))
        for key in ("x", "y", "z", "level"):
            assert np.array_equal(out[key], ref[key]), (k, key)
        m.free()
    assert failures > 0 and rc == 0
