"""The oracle against the reference's own regrid and hash-table kernels.

The reference's OpenCL kernels (split_cells.cl, merge_cells.cl,
balance_enforce.cl, compact_cells.cl, hash_build.cl, hash_query.cl,
halo_pack.cl) are compiled unmodified as C++ through an OpenCL C built-ins shim
(oracle/Makefile.ref, oracle/shim/opencl_c.h) and run by a CPU NDRange runner
(oracle/ndrange.cpp) under the reference engines' host steps restated in
oracle/ref_kernels.cpp.  Every deterministic output is compared with the oracle
restatement; where the oracle deliberately deviates (its deviation ledger), the
test shows the two differ exactly there.  Skipped where the reference tree is
absent (the in-place build needs it)."""
import ctypes
import os

import numpy as np
import pytest

from tests import _oracle as O

P = ctypes.c_void_p
INV = 0xFFFFFFFF


def _lib():
    from oracle import build as ob
    d = ob.build_reference()
    if d is None:
        pytest.skip("reference tree not present: the reference kernels cannot be compiled in place")
    L = ctypes.CDLL(os.path.join(d, "libfl_ref_kernels.so"))
    L.rk_balance.argtypes = [P] * 6 + [ctypes.c_size_t, ctypes.c_uint32, ctypes.c_uint32, P]
    L.rk_split.restype = ctypes.c_uint32
    L.rk_split.argtypes = [P] * 7 + [ctypes.c_size_t, P, ctypes.c_uint32] + [P] * 10
    L.rk_merge.restype = ctypes.c_uint32
    L.rk_merge.argtypes = [P] * 7 + [ctypes.c_size_t, P, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32,
                                     ctypes.c_int] + [P] * 9
    L.rk_exclusive_scan.restype = ctypes.c_uint32
    L.rk_exclusive_scan.argtypes = [P, P, ctypes.c_size_t]
    L.rk_adapt.restype = ctypes.c_size_t
    L.rk_adapt.argtypes = [P] * 7 + [ctypes.c_size_t, P, ctypes.c_uint32, ctypes.c_int, ctypes.c_uint32,
                                     ctypes.c_uint32, ctypes.c_uint32, ctypes.c_float] + [P] * 9
    L.rk_hash.argtypes = [P, P, ctypes.c_size_t, ctypes.c_uint64, P, ctypes.c_size_t, P, P, P]
    L.rk_pack_unpack.argtypes = [P, ctypes.c_size_t, ctypes.c_uint64, P, P]
    return L


@pytest.fixture(scope="module")
def rk():
    return _lib()


class BalStats(ctypes.Structure):
    _fields_ = [("converged", ctypes.c_int32), ("iterations", ctypes.c_uint32), ("violations", ctypes.c_uint32),
                ("marked", ctypes.c_uint32), ("per_iter_violations", ctypes.c_uint32 * 64),
                ("per_iter_marked", ctypes.c_uint32 * 64), ("table_max_displacement", ctypes.c_uint32)]


class AdaptStats(ctypes.Structure):
    _fields_ = [("num_children", ctypes.c_uint32), ("num_groups", ctypes.c_uint32),
                ("num_survivors", ctypes.c_uint32), ("num_out", ctypes.c_uint32), ("balance", BalStats),
                ("merge_table_max_displacement", ctypes.c_uint32)]


def p(a):
    return O.ptr(a)


def cols_c(c):
    return {k: np.ascontiguousarray(v) for k, v in c.items()}


# Reference kernels read 8-level coordinates (MAX_REFINEMENT_LEVEL 8 in every
# kernel file); the oracle runs the same meshes in a one-root domain with
# anchors at level 8.
DOM8 = dict(depth=21, anchor=8, max_level=8)
# Host lookup tables of at least 2^24 slots (every 8-level key) hold each key
# in its home slot: the kernels' lookups are then exact on any mesh, and the
# comparisons test the kernels' semantics; the engines' own table sizing
# (TABLE_ENGINE) is shown apart, in the probe-cap deviation test.
TABLE_EXACT = 1 << 24
TABLE_ENGINE = 0


def deep_mesh(seed, block=8, base=6, rounds=((0.3, 6), (0.3, 7)), states=False):
    """A leaf set confined to a corner block of the 256^3 anchor domain: a
    uniform block of `base`-level cells, then unbalanced random splits of the
    given fraction of cells at the given level.  Deep levels keep the engines'
    host lookup tables (slot = Morton key % size) free of long probe chains,
    so the kernels' probe caps (64) do not bite: once the table (a power of two
    >= 2n) is at least 8^b for a block of 2^b anchors, every key sits in its
    home slot."""
    rng = np.random.default_rng(seed)
    g = np.stack(np.meshgrid(*[np.arange(block)] * 3, indexing="ij"), -1).reshape(-1, 3)
    n = len(g)
    c = {"x": g[:, 0].astype(np.int32), "y": g[:, 1].astype(np.int32), "z": g[:, 2].astype(np.int32),
         "level": np.full(n, base, np.uint8), "state": np.zeros(n, np.uint8), "flags": np.zeros(n, np.int32),
         "material": rng.integers(0, 5, n).astype(np.uint32)}
    cfg = dict(max_level=8, min_level=0, balance_mode=0, max_balance_iterations=10, enforce_balance=0,
               averaging_rule=0)
    for frac, lv in rounds:
        m = len(c["x"])
        c["flags"] = np.where((rng.random(m) < frac) & (c["level"] == lv), 1, 0).astype(np.int32)
        c, *_ = O.adapt(c, cfg, O.domain(**DOM8))
        c = {k: v.copy() for k, v in c.items()}
    if states:
        c["state"] = np.where(rng.random(len(c["x"])) < 0.05, 1, 0).astype(np.uint8)
    return c


def anchors(c):
    sh = 8 - c["level"].astype(np.int32)
    return [(c[a].astype(np.int64) << sh).astype(np.int32) for a in ("x", "y", "z")]


# ----------------------------------------------------------------- 2:1 balance


@pytest.mark.parametrize("seed", [1, 2, 3, 4])
def test_balance_face6_equals_reference_kernels(rk, seed):
    """detect_balance_violations + mark_cascading_refinement under
    BalanceEnforcer::enforce vs the oracle's FACE6 mode: flags, convergence,
    iteration count, violation and mark totals."""
    c = deep_mesh(seed, rounds=((0.45, 6), (0.6, 7)))
    rng = np.random.default_rng(seed + 100)
    c["flags"] = rng.choice([0, 0, 0, 1, -1], len(c["x"])).astype(np.int32)
    c["state"] = np.where(rng.random(len(c["x"])) < 0.03, 1, 0).astype(np.uint8)
    c = cols_c(c)
    ax, ay, az = anchors(c)
    rflags = c["flags"].copy()
    st = BalStats()
    rk.rk_balance(p(ax), p(ay), p(az), p(c["level"]), p(c["state"]), p(rflags), len(ax), 10, TABLE_EXACT,
                  ctypes.byref(st))
    assert st.table_max_displacement < 64, "reference probe cap would bite on this mesh"
    oflags, ost = O.balance(c, O.domain(**DOM8), 0, 8, 10)
    assert st.violations > 0 and st.marked > 0  # the case exercises the kernels
    np.testing.assert_array_equal(rflags, oflags)
    assert (st.converged, st.iterations, st.violations, st.marked) == \
        (ost.converged, ost.iterations, ost.violations, ost.marked)
    for it in range(st.iterations - (1 if st.converged else 0)):
        assert st.per_iter_violations[it] == ost.per_iter_violations[it]
        assert st.per_iter_marked[it] == ost.per_iter_marked[it]


def test_balance_known_answer_through_reference_kernels(rk):
    """tests/unit/adaptation/BalanceEnforcerTest.cpp:37-93 on the compiled
    kernels: anchors x = {0, 128}, levels {1, 3} -> cell 0 flagged, converged."""
    ax = np.array([0, 128], np.int32)
    zz = np.zeros(2, np.int32)
    lv = np.array([1, 3], np.uint8)
    fl = np.zeros(2, np.int32)
    st = BalStats()
    rk.rk_balance(p(ax), p(zz), p(zz), p(lv), p(np.zeros(2, np.uint8)), p(fl), 2, 10, TABLE_ENGINE,
                  ctypes.byref(st))
    assert st.converged == 1 and st.violations > 0 and fl.tolist() == [1, 0]


def test_balance_probe_cap_deviation(rk):
    """Deviation 8: on a regular coarse grid the engines' table (slot = Morton
    key % size) puts every level-4 anchor (key low 12 bits zero) into a handful
    of home slots; past 64 probes the kernel stops looking and the violation
    is missed.  The oracle's exact lookups find it."""
    c = O.uniform_mesh(4)                     # 16^3 level-4 cells
    # refine one cell twice: level-6 cells next to level-4 neighbours
    c["flags"][:] = 0
    c["flags"][np.flatnonzero((c["x"] == 7) & (c["y"] == 7) & (c["z"] == 7))] = 1
    cfg = dict(max_level=8, min_level=0, balance_mode=0, max_balance_iterations=10, enforce_balance=0,
               averaging_rule=0)
    c, *_ = O.adapt(c, cfg, O.domain(**DOM8))
    c = {k: v.copy() for k, v in c.items()}
    c["flags"] = np.where(c["level"] == 5, 1, 0).astype(np.int32)
    c, *_ = O.adapt(c, cfg, O.domain(**DOM8))
    c = cols_c({k: v.copy() for k, v in c.items()})
    c["flags"][:] = 0
    ax, ay, az = anchors(c)
    rflags = c["flags"].copy()
    st = BalStats()
    rk.rk_balance(p(ax), p(ay), p(az), p(c["level"]), p(c["state"]), p(rflags), len(ax), 10, TABLE_ENGINE,
                  ctypes.byref(st))
    oflags, ost = O.balance(c, O.domain(**DOM8), 0, 8, 10)
    assert st.table_max_displacement >= 64
    assert ost.marked > 0 and (oflags == 1).sum() > (rflags == 1).sum()


# ----------------------------------------------------------------- split


@pytest.mark.parametrize("seed", [5, 6, 7])
def test_split_equals_reference_kernels(rk, seed):
    """split_count_and_allocate (barrier kernel, run as fibers) + host scan +
    split_generate_children + interpolate_split_fields vs the oracle regrid's
    children: same split set, same children (coordinates, level, state,
    material) in the reference's parent-major order, same copied fields, and
    the kernels' 8-level child keys equal the Morton codec."""
    c = cols_c(deep_mesh(seed, block=6, base=5, rounds=((0.3, 5), (0.3, 6))))
    n = len(c["x"])
    rng = np.random.default_rng(seed)
    c["flags"] = rng.choice([0, 1, 1, -1], n).astype(np.int32)
    c["flags"][c["level"] == 8] = 0
    C = 3
    f = rng.standard_normal((n, C)).astype(np.float32)
    cbs = np.zeros(n, np.uint32)
    m = 8 * n
    cx, cy, cz = (np.zeros(m, np.int32) for _ in range(3))
    cl, cs = np.zeros(m, np.uint8), np.zeros(m, np.uint8)
    cm = np.zeros(m, np.uint32)
    ch = np.zeros(m, np.uint64)
    cf = np.zeros(m * C, np.float32)
    kcbs = np.zeros(n, np.uint32)
    nc = rk.rk_split(p(c["x"]), p(c["y"]), p(c["z"]), p(c["level"]), p(c["state"]), p(c["flags"]), p(c["material"]),
                     n, p(f), C, p(cbs), p(cx), p(cy), p(cz), p(cl), p(cs), p(cm), p(ch), p(cf), p(kcbs))
    # the barrier kernel's own block starts ((inclusive count - 1) * 8) equal the engine's host scan
    np.testing.assert_array_equal(kcbs, cbs)
    out, st, of, src, kind, mem, _ = O.adapt(c, dict(max_level=8, min_level=0, balance_mode=0,
                                                     max_balance_iterations=10, enforce_balance=0,
                                                     averaging_rule=0), O.domain(**DOM8), f, C)
    sel = kind < 8
    order = np.lexsort((kind[sel], src[sel]))  # parent-major, child index minor
    assert nc == 8 * st.num_split and nc == sel.sum() and nc > 0
    for k, ref in (("x", cx), ("y", cy), ("z", cz), ("level", cl), ("state", cs), ("material", cm)):
        np.testing.assert_array_equal(out[k][sel][order], ref[:nc], err_msg=k)
    np.testing.assert_array_equal(of[sel][order], cf[:nc * C].reshape(nc, C))
    # the split set and the block starts (8 x rank among split parents)
    split_parents = np.unique(src[sel])
    assert (cbs[split_parents] == 8 * np.arange(len(split_parents))).all()
    assert (np.delete(cbs, split_parents) == INV).all()
    np.testing.assert_array_equal(ch[:nc], O.morton8(cx[:nc], cy[:nc], cz[:nc]))


# ----------------------------------------------------------------- merge


def _block(level, lo, hi):
    g = np.stack(np.meshgrid(*[np.arange(a, b) for a, b in zip(lo, hi)], indexing="ij"), -1).reshape(-1, 3)
    return g, np.full(len(g), level, np.uint8)


def _merge_mesh(seed):
    """Three uniform blocks at levels 8, 7 and 6 whose NATIVE coordinates never
    coincide (the merge engine keys its host table on native coordinates
    without the level, so equal coordinates of different levels would share a
    key and chain): level 8 at native [0,16)^3, level 7 at x in [16,24),
    level 6 at y in [16,24); the blocks are disjoint in space too.  Random
    octets are flagged -1, a few single cells unflagged (incomplete octets)
    and a few cells made SOLID."""
    parts = [_block(8, (0, 0, 0), (16, 16, 16)), _block(7, (16, 0, 0), (24, 8, 8)), _block(6, (0, 16, 0), (8, 24, 8))]
    g = np.concatenate([a for a, _ in parts])
    lv = np.concatenate([b for _, b in parts])
    rng = np.random.default_rng(seed)
    perm = rng.permutation(len(g))         # the engines do not rely on any cell order
    g, lv = g[perm], lv[perm]
    n = len(g)
    c = {"x": g[:, 0].astype(np.int32), "y": g[:, 1].astype(np.int32), "z": g[:, 2].astype(np.int32),
         "level": lv, "state": np.zeros(n, np.uint8), "flags": np.zeros(n, np.int32),
         "material": rng.integers(0, 5, n).astype(np.uint32)}
    key = (c["x"] >> 1).astype(np.int64) * 1_000_003 + (c["y"] >> 1) * 1009 + (c["z"] >> 1) + \
        c["level"].astype(np.int64) * 10 ** 9
    u, inv = np.unique(key, return_inverse=True)
    pick = rng.random(len(u)) < 0.5
    c["flags"] = np.where(pick[inv], -1, 0).astype(np.int32)
    c["flags"][rng.random(n) < 0.05] = 0
    c["state"] = np.where(rng.random(n) < 0.01, 1, 0).astype(np.uint8)
    return cols_c(c)


@pytest.mark.parametrize("seed", [11, 12, 13])
@pytest.mark.parametrize("rule", [0, 1])
def test_merge_equals_reference_kernels(rk, seed, rule):
    """mark_sibling_groups + create_parent_cells + merge_fields under
    MergeEngine::merge vs the oracle regrid's merge: the groups as sets of
    member sets (atomic_inc ids are device-order dependent), each group's
    parent cell, and its restricted field.  Deviation 5: the reference adds
    the children's contributions in cell-index order with float CAS atomics,
    the oracle sums children 0..7 in order; the values equal a sum taken in
    the reference's order bit for bit and the oracle's to rounding."""
    c = _merge_mesh(seed)
    n = len(c["x"])
    C = 4
    rng = np.random.default_rng(seed + 7)
    f = (rng.standard_normal((n, C)) * 3).astype(np.float32)
    gid = np.zeros(n, np.uint32)
    px, py, pz = (np.zeros(n, np.int32) for _ in range(3))
    pl, ps, pm = np.zeros(n, np.uint8), np.zeros(n, np.uint8), np.zeros(n, np.uint32)
    pf = np.zeros(n * C, np.float32)
    md = ctypes.c_uint32(0)
    ng = rk.rk_merge(p(c["x"]), p(c["y"]), p(c["z"]), p(c["level"]), p(c["state"]), p(c["flags"]), p(c["material"]),
                     n, p(f), C, rule, TABLE_EXACT, 0, p(gid), p(px), p(py), p(pz), p(pl), p(ps), p(pm), p(pf),
                     ctypes.byref(md))
    assert md.value < 64, "reference probe cap would bite on this mesh"
    out, st, of, src, kind, mem, _ = O.adapt(c, dict(max_level=8, min_level=0, balance_mode=0,
                                                     max_balance_iterations=10, enforce_balance=0,
                                                     averaging_rule=rule), O.domain(**DOM8), f, C)
    assert ng == st.num_groups and ng > 0
    ref_groups = {}
    for i in np.flatnonzero(gid != INV):
        ref_groups.setdefault(int(gid[i]), []).append(int(i))
    ora = mem.reshape(-1, 8)
    assert {frozenset(g) for g in ref_groups.values()} == {frozenset(g.tolist()) for g in ora}
    # parents: match each oracle group to the reference group with the same members
    by_members = {frozenset(v): k for k, v in ref_groups.items()}
    pf = pf[:ng * C].reshape(ng, C)
    sel = np.flatnonzero(kind == 9)
    for j in sel:
        g = int(src[j])
        r = by_members[frozenset(ora[g].tolist())]
        assert (px[r], py[r], pz[r], pl[r], ps[r], pm[r]) == \
            (out["x"][j], out["y"][j], out["z"][j], out["level"][j], out["state"][j], out["material"][j])
        # the reference's value = contributions added in cell-index order
        s = np.zeros(C, np.float32)
        for i in sorted(ref_groups[r]):
            v = f[i] * np.float32(0.125) if rule == 0 else f[i]
            s = (s + v).astype(np.float32)
        np.testing.assert_array_equal(pf[r], s)
        np.testing.assert_allclose(pf[r], of[j], rtol=2e-6, atol=1e-6)


def test_merge_level_zero_deviation(rk):
    """Deviation 9: eight level-0 cells flagged -1 merge into a level-255 parent
    on the reference kernels; the oracle stops at min_level (0)."""
    c = cols_c(O.uniform_mesh(0, (2, 2, 2)))
    c["flags"][:] = -1
    n = 8
    gid = np.zeros(n, np.uint32)
    px, py, pz = (np.zeros(n, np.int32) for _ in range(3))
    pl, ps, pm = np.zeros(n, np.uint8), np.zeros(n, np.uint8), np.zeros(n, np.uint32)
    ng = rk.rk_merge(p(c["x"]), p(c["y"]), p(c["z"]), p(c["level"]), p(c["state"]), p(c["flags"]), p(c["material"]),
                     n, None, 0, 0, TABLE_ENGINE, 0, p(gid), p(px), p(py), p(pz), p(pl), p(ps), p(pm), None, None)
    assert ng == 1 and pl[0] == 255
    out, st, *_ = O.adapt(c, dict(max_level=8, min_level=0, balance_mode=0, max_balance_iterations=10,
                                  enforce_balance=0, averaging_rule=0), O.domain(ext=(2, 2, 2)))
    assert st.num_groups == 0


# ----------------------------------------------------------------- scan + compaction


@pytest.mark.parametrize("n", [1, 7, 255, 256, 257, 4097, 65535, 65536])
def test_scan_equals_reference_kernels(rk, n):
    """AdaptationEngine::exclusiveScan over scan_local (barrier kernel with
    __local memory, run as fibers) and scan_add_sums vs the oracle's scan."""
    a = np.random.default_rng(n).integers(0, 3, n).astype(np.uint32)
    r = np.zeros(n, np.uint32)
    o = np.zeros(n, np.uint32)
    tr = rk.rk_exclusive_scan(p(a), p(r), n)
    to = O.load().or_scan_exclusive_u32(p(a), p(o), n)
    np.testing.assert_array_equal(r, o)
    assert tr == to


def test_scan_limit_deviation(rk):
    """Deviation 6: the block sums are scanned by one 256-wide group, so the
    reference's scan is wrong from element 65,536 on; the oracle's is exact."""
    n = 70000
    a = np.ones(n, np.uint32)
    r = np.zeros(n, np.uint32)
    rk.rk_exclusive_scan(p(a), p(r), n)
    np.testing.assert_array_equal(r[:65536], np.arange(65536))
    assert (r[65536:] != np.arange(65536, n)).any()


def _to_reference_order(out, src, kind):
    """Oracle regrid output (key order) permuted into the reference rebuild's
    order: survivors by old index, children parent-major, parents by group."""
    surv = np.flatnonzero(kind == 8)
    surv = surv[np.argsort(src[surv], kind="stable")]
    ch = np.flatnonzero(kind < 8)
    ch = ch[np.lexsort((kind[ch], src[ch]))]
    par = np.flatnonzero(kind == 9)
    par = par[np.argsort(src[par], kind="stable")]
    return np.concatenate([surv, ch, par]), len(surv), len(ch)


@pytest.mark.parametrize("mesh", ["merge", "balance"])
@pytest.mark.parametrize("seed", [21, 22, 23])
def test_adapt_equals_reference_rebuild(rk, seed, mesh):
    """The whole reference regrid -- BalanceEnforcer (FACE6), SplitEngine,
    MergeEngine, then compactAndRebuildGPU's mark_valid_cells, exclusive scan,
    compact_cells and append_cells -- vs the oracle regrid put into the
    reference's output order (deviation 1: the oracle sorts by key).  Cells
    and survivor/parent fields are equal; children carry no fields in the
    reference rebuild (deviation 2) and the oracle copies the parent's.
    "merge": the three-block mesh with merges and splits, balance on (it finds
    nothing to do there); "balance": an unbalanced random octree with splits
    and FACE6 violations, no merges."""
    rng = np.random.default_rng(seed)
    if mesh == "merge":
        c = _merge_mesh(seed)
        balance = 1
    else:
        c = cols_c(deep_mesh(seed, rounds=((0.45, 6), (0.6, 7))))
        c["flags"][:] = 0
        balance = 1
    n = len(c["x"])
    split = (rng.random(n) < 0.15) & (c["level"] < 8)
    c["flags"][split] = 1
    c["state"][:] = 0  # deviation 13 (flagged cells that cannot split) has its own test
    C = 2
    f = rng.standard_normal((n, C)).astype(np.float32)
    m = 8 * n + 8
    ox, oy, oz = (np.zeros(m, np.int32) for _ in range(3))
    ol, os_, om = np.zeros(m, np.uint8), np.zeros(m, np.uint8), np.zeros(m, np.uint32)
    of = np.zeros(m * C, np.float32)
    fab = np.zeros(n, np.int32)
    st = AdaptStats()
    fill = np.float32(-12345.0)
    M = rk.rk_adapt(p(c["x"]), p(c["y"]), p(c["z"]), p(c["level"]), p(c["state"]), p(c["flags"]), p(c["material"]),
                    n, p(f), C, balance, 10, 0, TABLE_EXACT, fill, p(ox), p(oy), p(oz), p(ol), p(os_), p(om), p(of), p(fab),
                    ctypes.byref(st))
    assert st.merge_table_max_displacement < 64 or not (c["flags"] == -1).any()
    assert st.balance.table_max_displacement < 64
    if mesh == "balance":
        assert st.balance.violations > 0 and st.num_children > 0
    else:
        assert st.num_groups > 0 and st.num_children > 0
    out, ost, oof, src, kind, mem, keep = O.adapt(c, dict(max_level=8, min_level=0, balance_mode=0,
                                                         max_balance_iterations=10, enforce_balance=balance,
                                                         averaging_rule=0), O.domain(**DOM8), f, C)
    np.testing.assert_array_equal(fab, keep["flags"])  # flags after balance
    assert M == len(out["x"]) and st.num_groups == ost.num_groups and st.num_children == ost.num_children
    perm, ns, nch = _to_reference_order(out, src, kind)
    assert st.num_survivors == ns
    for k, ref in (("x", ox), ("y", oy), ("z", oz), ("level", ol), ("state", os_), ("material", om)):
        np.testing.assert_array_equal(out[k][perm], ref[:M], err_msg=k)
    of = of[:M * C].reshape(M, C)
    oo = oof[perm]
    np.testing.assert_array_equal(oo[:ns], of[:ns])                         # survivors copied
    assert (of[ns:ns + nch] == fill).all()                                   # children: no fields (ref)
    np.testing.assert_array_equal(oo[ns:ns + nch], f[src[perm][ns:ns + nch]])  # children: parent's (oracle)
    np.testing.assert_allclose(oo[ns + nch:], of[ns + nch:], rtol=2e-6, atol=1e-6)  # parents (deviation 5)


def test_flagged_cell_that_cannot_split_deviation(rk):
    """Deviation 13: mark_valid_cells drops every cell with flag > 0, but the
    split kernels split only FLUID cells below level 8, so a flagged SOLID cell
    vanishes from the reference's rebuilt mesh.  The oracle keeps it."""
    c = cols_c(deep_mesh(31, block=4, base=6, rounds=()))
    n = len(c["x"])
    c["state"][:5] = 1
    c["flags"][:5] = 1
    c["flags"][5:9] = 1
    m = 8 * n + 8
    bufs = [np.zeros(m, np.int32) for _ in range(3)] + [np.zeros(m, np.uint8) for _ in range(2)] + \
        [np.zeros(m, np.uint32)]
    st = AdaptStats()
    M = rk.rk_adapt(p(c["x"]), p(c["y"]), p(c["z"]), p(c["level"]), p(c["state"]), p(c["flags"]), p(c["material"]),
                    n, None, 0, 0, 10, 0, TABLE_EXACT, 0.0, *[p(b) for b in bufs], None, None, ctypes.byref(st))
    out, ost, *_ = O.adapt(c, dict(max_level=8, min_level=0, balance_mode=0, max_balance_iterations=10,
                                   enforce_balance=0, averaging_rule=0), O.domain(**DOM8))
    assert M == len(out["x"]) - 5
    solid = {(int(x), int(y), int(z)) for x, y, z in zip(c["x"][:5], c["y"][:5], c["z"][:5])}
    ref_cells = {(int(x), int(y), int(z), int(l)) for x, y, z, l in zip(bufs[0][:M], bufs[1][:M], bufs[2][:M],
                                                                       bufs[3][:M])}
    assert not any((x, y, z, 6) in ref_cells for x, y, z in solid)
    ora_cells = {(int(x), int(y), int(z), int(l)) for x, y, z, l in zip(out["x"], out["y"], out["z"], out["level"])}
    assert all((x, y, z, 6) in ora_cells for x, y, z in solid)


# ----------------------------------------------------------------- hash table


def _hash_run(rk, keys, vals, queries):
    cap = int(O.load().or_hash_capacity(len(keys)))
    res = np.zeros(len(queries), np.uint32)
    qp = np.zeros(len(queries), np.uint32)
    bp = np.zeros(len(keys), np.uint32)
    rk.rk_hash(p(keys), p(vals), len(keys), cap, p(queries), len(queries), p(res), p(qp), p(bp))
    tk = np.zeros(cap, np.uint64)
    tv = np.zeros(cap, np.uint32)
    L = O.load()
    L.or_hash_build(p(keys), p(vals), len(keys), cap, p(tk), p(tv))
    ores = np.zeros(len(queries), np.uint32)
    L.or_hash_query(p(tk), p(tv), cap, p(queries), p(ores), len(queries))
    return res, ores, bp


@pytest.mark.parametrize("n", [1, 1000, 300_000])
def test_hash_equals_reference_kernels(rk, n):
    """hash_clear + hash_build + hash_validate vs the oracle's table: the same
    query results for present and absent keys (random 63-bit keys, where the
    reference's 32-probe cap does not bite), and for repeated keys the last
    input's value (the runner executes work-items in order)."""
    rng = np.random.default_rng(n)
    keys = rng.integers(0, 1 << 63, n, dtype=np.uint64)
    keys = np.concatenate([keys, keys[: n // 10]])            # repeats
    vals = np.arange(len(keys), dtype=np.uint32)
    q = np.concatenate([keys, rng.integers(0, 1 << 63, n, dtype=np.uint64), np.array([~np.uint64(0)])])
    res, ores, bp = _hash_run(rk, keys, vals, q)
    assert (bp < 32).all()
    np.testing.assert_array_equal(res, ores)
    assert (res[:len(keys)] != INV).all()


def test_hash_low_bits_deviation(rk):
    """Deviation 10: the reference's slot is the LOW bits of key * 2^64/phi.
    12-state keys of level-3 anchors (21-level codec) have their low 54 bits
    set by the curve's digits for zero sub-coordinates, so all of them fall
    into a handful of slots; past 32 probes hash_build silently drops the pair
    and the query misses.  The oracle's high-bit slot keeps every key."""
    c = O.uniform_mesh(3)
    keys = O.hilbert_encode(c["x"].astype(np.int64) << 18, c["y"].astype(np.int64) << 18,
                            c["z"].astype(np.int64) << 18, 21)
    vals = np.arange(len(keys), dtype=np.uint32)
    res, ores, bp = _hash_run(rk, keys, vals, keys)
    assert (bp == 32).any() and (res == INV).any()
    np.testing.assert_array_equal(ores, vals)


def test_halo_pack_unpack_identity(rk):
    """pack_fields / unpack_fields (kernels/halo_pack.cl) round trip at a byte
    offset, as test_halo_exchanger.cpp:82-123 checks."""
    f = np.random.default_rng(0).standard_normal(1000).astype(np.float32)
    buf = np.zeros(4096 + 4000, np.uint8)
    back = np.zeros(1000, np.float32)
    rk.rk_pack_unpack(p(f), 1000, 4096, p(buf), p(back))
    np.testing.assert_array_equal(back, f)
    np.testing.assert_array_equal(buf[4096:].view(np.float32), f)


def test_merge_group_id_race(rk):
    """mark_sibling_groups clears its own work-item's group id (merge_cells.cl:29)
    in the launch in which leaders store their siblings' ids (:101-104).  Under
    the in-order schedule every sibling after its leader is cleared again, so
    create_parent_cells still makes every parent but merge_fields misses those
    children; under the all-fibers schedule (every clear before any leader's
    stores) every member keeps its id.  The oracle follows the latter."""
    c = _merge_mesh(41)
    n = len(c["x"])
    res = {}
    for seq in (0, 1):
        gid = np.zeros(n, np.uint32)
        px, py, pz = (np.zeros(n, np.int32) for _ in range(3))
        pl, ps, pm = np.zeros(n, np.uint8), np.zeros(n, np.uint8), np.zeros(n, np.uint32)
        ng = rk.rk_merge(p(c["x"]), p(c["y"]), p(c["z"]), p(c["level"]), p(c["state"]), p(c["flags"]),
                         p(c["material"]), n, None, 0, 0, TABLE_EXACT, seq, p(gid), p(px), p(py), p(pz), p(pl),
                         p(ps), p(pm), None, None)
        res[seq] = (ng, gid.copy(), px[:ng].copy())
    (ng0, g0, p0), (ng1, g1, p1) = res[0], res[1]
    assert ng0 == ng1 > 0
    np.testing.assert_array_equal(p0, p1)               # parents do not depend on the schedule
    assert (g0 != INV).sum() == 8 * ng0                  # every member keeps its id
    assert (g1 != INV).sum() < 8 * ng1                   # in order: later siblings lose theirs
    leaders = (c["x"] & 1 | c["y"] & 1 | c["z"] & 1) == 0
    np.testing.assert_array_equal((g1 != INV) & leaders, (g0 != INV) & leaders)
