"""Oracle regrid vs the reference's own AMR tests (read as text: the reference
needs OpenCL, absent here) and structural properties."""
import numpy as np
import pytest

from tests import _oracle as O

CFG = dict(max_level=8, min_level=0, balance_mode=0, max_balance_iterations=10, enforce_balance=1, averaging_rule=0)


def one(x, y, z, level, flag):
    return {"x": np.array(x, np.int32), "y": np.array(y, np.int32), "z": np.array(z, np.int32),
            "level": np.array(level, np.uint8), "state": np.zeros(len(x), np.uint8),
            "flags": np.array(flag, np.int32), "material": np.zeros(len(x), np.uint32)}


def test_split_single_cell():
    # tests/unit/adaptation/SplitEngineTest.cpp:35-63: 1 cell, flag 1 -> 8 children at level 1
    out, st, *_ = O.adapt(one([0], [0], [0], [0], [1]), CFG, O.domain())
    assert st.num_split == 1 and st.num_children == 8 and len(out["x"]) == 8
    assert (out["level"] == 1).all()
    assert sorted(zip(out["x"], out["y"], out["z"])) == [(i & 1, (i >> 1) & 1, i >> 2) for i in range(8)] or \
        set(zip(out["x"], out["y"], out["z"])) == {(i & 1, (i >> 1) & 1, i >> 2) for i in range(8)}


def test_merge_siblings():
    # tests/unit/adaptation/MergeEngineTest.cpp:35-71: 8 siblings at level 1, flag -1 -> one parent
    i = np.arange(8)
    out, st, *_ = O.adapt(one(i & 1, (i >> 1) & 1, i >> 2, [1] * 8, [-1] * 8), CFG, O.domain())
    assert st.num_groups == 1 and st.num_merged == 8
    assert len(out["x"]) == 1 and out["level"][0] == 0 and out["x"][0] == 0


def test_balance_detects_violation():
    # tests/unit/adaptation/BalanceEnforcerTest.cpp:37-93: finest-anchor coords x={0,128},
    # levels {1,3} (8-level anchors) -> cell 0 flagged, converged
    cols = one([0, 128 >> 5], [0, 0], [0, 0], [1, 3], [0, 0])
    flags, st = O.balance(cols, O.domain(depth=21, anchor=8, max_level=8), 0, 8)
    assert st.converged == 1 and st.violations > 0 and st.marked > 0
    assert flags.tolist() == [1, 0]


def test_split_merge_cycle():
    # tests/integration/adaptation/AdaptationIntegrationTest.cpp:62-128
    out, st, *_ = O.adapt(one([0], [0], [0], [0], [1]), dict(CFG, balance_mode=1), O.domain())
    assert len(out["x"]) == 8 and (out["level"] == 1).all() and (out["flags"] == 0).all()
    out["flags"] = np.full(8, -1, np.int32)
    out2, st2, *_ = O.adapt(out, dict(CFG, balance_mode=1), O.domain())
    assert len(out2["x"]) == 1 and out2["level"][0] == 0


def test_merge_stops_at_min_level():
    # deviation guard: the reference would create a level-255 parent from level-0 cells
    c = O.uniform_mesh(0, (2, 2, 2))
    c["flags"][:] = -1
    out, st, *_ = O.adapt(c, CFG, O.domain(ext=(2, 2, 2)))
    assert st.num_groups == 0 and len(out["x"]) == 8


def _leaf_levels_grid(cols, L):
    """Level of the leaf covering each finest cell of a 2^L grid (single root)."""
    g = np.full((1 << L,) * 3, -1, np.int32)
    for x, y, z, l in zip(cols["x"], cols["y"], cols["z"], cols["level"]):
        s = 1 << (L - l)
        sl = g[x * s:(x + 1) * s, y * s:(y + 1) * s, z * s:(z + 1) * s]
        assert (sl == -1).all(), "overlapping leaves"
        sl[...] = l
    assert (g >= 0).all(), "holes"
    return g


def _balanced26(g):
    a = g.astype(np.int32)
    for dx in (-1, 0, 1):
        for dy in (-1, 0, 1):
            for dz in (-1, 0, 1):
                sh = np.roll(np.roll(np.roll(a, dx, 0), dy, 1), dz, 2)
                m = np.ones_like(a, bool)
                # ignore wrap-around
                if dx == 1: m[0] = False
                if dx == -1: m[-1] = False
                if dy == 1: m[:, 0] = False
                if dy == -1: m[:, -1] = False
                if dz == 1: m[:, :, 0] = False
                if dz == -1: m[:, :, -1] = False
                if (np.abs(sh - a)[m] > 1).any():
                    return False
    return True


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_full26_regrid_keeps_2to1_and_tiles_domain(seed):
    cols = O.random_octree(seed, ext=(1, 1, 1), rounds=4, max_level=5, frac=0.35, balanced=True)
    g = _leaf_levels_grid(cols, 5)
    assert _balanced26(g)
    # random split/merge flags, FULL26 regrid, still a balanced tiling
    rng = np.random.default_rng(seed)
    cols["flags"] = rng.choice([-1, 0, 1], len(cols["x"]), p=[0.5, 0.3, 0.2]).astype(np.int32)
    out, st, *_ = O.adapt(cols, dict(CFG, max_level=5, balance_mode=1), O.domain(max_level=5))
    g2 = _leaf_levels_grid(out, 5)
    assert _balanced26(g2)
    keys = O.cell_keys(out["x"], out["y"], out["z"], out["level"], None, 21, 21)
    assert (np.diff(keys.astype(np.uint64)) > 0).all()


def test_fields_prolong_and_restrict():
    c = O.uniform_mesh(1, (1, 1, 1))
    C = 3
    f = np.arange(8 * C, dtype=np.float32).reshape(8, C) * 0.37 + 1.0
    c["flags"][:] = -1
    out, st, of, src, kind, mem, _ = O.adapt(c, CFG, O.domain(), f, C)
    assert len(out["x"]) == 1
    s = np.zeros(C, np.float32)
    for q in range(8):
        s = (s + f[mem[q]]).astype(np.float32)
    np.testing.assert_array_equal(of[0], s * np.float32(0.125))
    c2 = O.uniform_mesh(0, (1, 1, 1))
    c2["flags"][:] = 1
    out, st, of, src, kind, mem, _ = O.adapt(c2, CFG, O.domain(), np.array([[1.5, -2.0, 3.25]], np.float32), 3)
    assert (of == np.array([1.5, -2.0, 3.25], np.float32)).all()


def test_neighbours_uniform_periodic():
    c = O.uniform_mesh(2, (1, 1, 1))
    nbr = O.neighbours(c, O.domain(max_level=4, periodic=(1, 1, 1)), 1).reshape(-1, 26)
    idx = {(x, y, z): i for i, (x, y, z) in enumerate(zip(c["x"], c["y"], c["z"]))}
    for i, (x, y, z) in enumerate(zip(c["x"], c["y"], c["z"])):
        for k in range(26):
            kk = k if k < 13 else k + 1
            d = (kk % 3 - 1, (kk // 3) % 3 - 1, kk // 9 - 1)
            assert nbr[i, k] == idx[((x + d[0]) % 4, (y + d[1]) % 4, (z + d[2]) % 4)]


def test_full26_flag_at_max_level_does_not_push_neighbours():
    """A flagged cell already at the maximum level will not split, so it must not
    make its one-level-coarser neighbours refine (FULL26 shadow levels)."""
    # level-1 octant of a unit domain refined once more: cells at level 2 in
    # [0, 2)^3 (level-1 cell 0 split), level 1 elsewhere
    l1 = O.uniform_mesh(1)
    keep = ~((l1["x"] == 0) & (l1["y"] == 0) & (l1["z"] == 0))
    l2 = O.uniform_mesh(2)
    inner = (l2["x"] < 2) & (l2["y"] < 2) & (l2["z"] < 2)
    cols = {k: np.concatenate([l1[k][keep], l2[k][inner]]) for k in l1}
    cols["flags"][:] = 0
    cols["flags"][cols["level"] == 2] = 1  # flagged, but level 2 is the maximum
    dom = O.domain(ext=(1, 1, 1))
    flags, st = O.balance(cols, dom, 1, 2)
    assert st.marked == 0 and (flags[cols["level"] == 1] == 0).all()
    # with a maximum of 3 the same flags do split, and the level-1 neighbours must follow
    flags3, st3 = O.balance(cols, dom, 1, 3)
    assert st3.marked > 0 and (flags3[cols["level"] == 1] == 1).any()
