"""Small exhaustive cases and determinism on the GPU (device race checks without
a sanitizer).  Every leaf set of one root cell down to level 2 whose level-1
cells are each a leaf or split (256 sets), in key order and shuffled:
neighbour tables, FULL26 balance and a regrid against the oracle.  Then the
same work run twice gives bitwise the same results (sort with ties, regrid,
pool steps)."""
import ctypes

import numpy as np
import pytest

from tests import _oracle as O
from tests.test_gpu_amr import cfg, mesh, run_adapt

pytestmark = pytest.mark.gpu


def octree(bits):
    """Level-1 cell c (bit order x, y, z) is split into 8 level-2 cells when bit c of `bits` is set."""
    x, y, z, lv = [], [], [], []
    for c in range(8):
        cx, cy, cz = c & 1, (c >> 1) & 1, (c >> 2) & 1
        if (bits >> c) & 1:
            for k in range(8):
                x.append(2 * cx + (k & 1)); y.append(2 * cy + ((k >> 1) & 1)); z.append(2 * cz + ((k >> 2) & 1))
                lv.append(2)
        else:
            x.append(cx); y.append(cy); z.append(cz); lv.append(1)
    n = len(x)
    return {"x": np.array(x, np.int32), "y": np.array(y, np.int32), "z": np.array(z, np.int32),
            "level": np.array(lv, np.uint8), "state": np.zeros(n, np.uint8), "flags": np.zeros(n, np.int32),
            "material": np.zeros(n, np.uint32)}


def _permute(cols, rng):
    p = rng.permutation(len(cols["x"]))
    return {k: np.ascontiguousarray(v[p]) for k, v in cols.items()}


def test_every_two_level_octree(ctx):
    from fluidloom_gb300 import DeviceArray
    from fluidloom_gb300.amr import BalanceResult
    rng = np.random.default_rng(11)
    for bits in range(256):
        cols = octree(bits)
        if bits % 3 == 1:
            cols = _permute(cols, rng)
        n = len(cols["x"])
        periodic = (bits & 1, (bits >> 1) & 1, 0)
        # neighbour tables, 1 and 4 sub-slots
        for sub in (1, 4):
            want = O.neighbours(cols, O.domain(ext=(1, 1, 1), max_level=4, periodic=periodic), sub)
            m = mesh(ctx, cols)
            nbr = DeviceArray(ctx, (n * 26 * sub,), np.uint32)
            ctx.call("fl_neighbour_rebuild", ctypes.byref(m.m),
                     ctypes.byref(cfg(max_level=4, periodic=periodic)), sub, nbr.ptr)
            np.testing.assert_array_equal(nbr.to_host(), want, err_msg="octree %d sub %d" % (bits, sub))
        # FULL26 balance with some level-2 cells flagged to split
        flagged = dict(cols)
        flagged["flags"] = ((np.arange(n) * 7 + bits) % 5 == 0).astype(np.int32) * (cols["level"] == 2)
        wf, wst = O.balance(flagged, O.domain(ext=(1, 1, 1), max_level=4), 1, 4)
        m = mesh(ctx, flagged)
        r = BalanceResult()
        rc = ctx.lib.fl_balance_enforce(ctx.handle, ctypes.byref(m.m),
                                        ctypes.byref(cfg(max_level=4, balance_mode=1)), ctypes.byref(r))
        assert rc in (0, -5)
        np.testing.assert_array_equal(m.download()["flags"], wf, err_msg="octree %d balance" % bits)
        # a regrid: the flagged cells split, level-2 octets flagged -1 merge where allowed
        mixed = dict(flagged)
        mixed["flags"] = np.where(cols["level"] == 2, np.where(flagged["flags"] > 0, 1, -1), 0).astype(np.int32)
        kw = dict(max_level=4, min_level=0, balance_mode=1, max_balance_iterations=10, enforce_balance=1,
                  averaging_rule=0)
        want, wst2, *_ = O.adapt(mixed, kw, O.domain(ext=(1, 1, 1), max_level=4))
        rc, got, st, _ = run_adapt(ctx, mixed, cfg(max_level=4, min_level=0, balance_mode=1))
        assert rc in (0, -5)
        for k in ("x", "y", "z", "level"):
            np.testing.assert_array_equal(got[k], want[k], err_msg="octree %d adapt %s" % (bits, k))


def test_same_work_twice_is_bitwise_identical(ctx):
    from fluidloom_gb300 import DeviceArray, lbm
    from fluidloom_gb300.lbm import Pool
    rng = np.random.default_rng(2)
    # sort with many ties
    n = 3_000_000
    keys = (rng.integers(0, 1 << 20, n) << 40).astype(np.uint64)
    outs = []
    for _ in range(2):
        k = DeviceArray.from_host(ctx, keys)
        v = DeviceArray.from_host(ctx, np.arange(n, dtype=np.uint32))
        ctx.call("fl_sort_pairs_u64_u32", k.ptr, v.ptr, ctypes.c_size_t(n), 0, 64)
        outs.append((k.to_host(), v.to_host()))
    np.testing.assert_array_equal(outs[0][0], outs[1][0])
    np.testing.assert_array_equal(outs[0][1], outs[1][1])
    # a regrid of a random octree
    cols = O.random_octree(31, ext=(2, 2, 2), rounds=3, max_level=6, frac=0.3)
    cols["flags"] = rng.choice([-1, 0, 1], len(cols["x"]), p=[0.5, 0.3, 0.2]).astype(np.int32)
    a = run_adapt(ctx, cols, cfg(max_level=6, balance_mode=1, ext=(2, 2, 2)))[1]
    b = run_adapt(ctx, cols, cfg(max_level=6, balance_mode=1, ext=(2, 2, 2)))[1]
    for k in ("x", "y", "z", "level"):
        np.testing.assert_array_equal(a[k], b[k])
    # pool steps with regrids (dependency graph over two streams, graph replay)
    c = lbm.sphere_channel(64, 32, 32, 2, radius=4.0, centre=(16.0, 16.0, 16.0), u_in=0.04, band=3.0)
    pools = [Pool(ctx, [c]) for _ in range(2)]
    for p in pools:
        for _ in range(3):
            p.step(7)
            p.regrid()
    np.testing.assert_array_equal(pools[0].populations(), pools[1].populations())
