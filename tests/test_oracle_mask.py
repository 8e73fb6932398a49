"""Solid masks in the CPU oracle pool (no GPU): an empty mask changes nothing,
a box of mask voxels removes exactly the sites that sample it (at a coarser and
at the same level), and bricks holding both solid and fluid sites are flagged
for refinement."""
import numpy as np

from fluidloom_gb300 import lbm
from tests import _oracle as O


def _box_mask(shape, lo, hi):
    m = np.zeros(shape, bool)
    m[lo[2]:hi[2], lo[1]:hi[1], lo[0]:hi[0]] = True
    return m


def _shape(case, level):
    return tuple((int(case.ext[a]) * 8) << level for a in (2, 1, 0))


def test_empty_mask_changes_nothing():
    c = lbm.cavity(16, 1, u_lid=0.06, tau=0.6)
    a, b = O.OraclePool([c]), O.OraclePool([c])
    b.set_mask(0, 1, lbm.pack_mask(np.zeros(_shape(c, 1), bool)))
    for p in (a, b):
        p.step(2)
        p.regrid()
        p.step(1)
    for k in ("x", "y", "z", "level", "case_id"):
        np.testing.assert_array_equal(a.bricks()[k], b.bricks()[k])
    np.testing.assert_array_equal(a.populations(), b.populations())


def test_box_removes_the_sites_that_sample_it():
    c = lbm.cavity(16, 0)
    p = O.OraclePool([c])
    full = p.lups()
    assert full == 16 ** 3
    # level 0: a 4^3 box of sites
    p.set_mask(0, 0, lbm.pack_mask(_box_mask(_shape(c, 0), (3, 5, 6), (7, 9, 10))))
    assert p.lups() == full - 64
    # level 1: a level-0 site samples voxel 2s + 1, so voxels [8, 16) hold sites 4..7
    p.set_mask(0, 1, lbm.pack_mask(_box_mask(_shape(c, 1), (8, 8, 8), (16, 16, 16))))
    assert p.lups() == full - 64
    # voxels [9, 16): 2s + 1 >= 9 leaves sites 4..7 as well; [8, 15) only 4..6
    p.set_mask(0, 1, lbm.pack_mask(_box_mask(_shape(c, 1), (9, 9, 9), (16, 16, 16))))
    assert p.lups() == full - 64
    p.set_mask(0, 1, lbm.pack_mask(_box_mask(_shape(c, 1), (8, 8, 8), (15, 15, 15))))
    assert p.lups() == full - 27
    p.set_mask(0, 0, None)
    assert p.lups() == full


def test_mixed_bricks_are_flagged():
    c = lbm.cavity(32, 1)
    c.refine_frac, c.coarsen_frac = 2.0, 0.0  # no vorticity flags: only the mask band
    p = O.OraclePool([c])
    lo, hi = (10, 10, 10), (20, 20, 20)  # level-0 sites; bricks 1..2 per axis touch it
    p.set_mask(0, 0, lbm.pack_mask(_box_mask(_shape(c, 0), lo, hi)))
    fl, _ = p.flags()
    b = p.bricks()
    for i in range(len(fl)):
        o = np.array([b["x"][i], b["y"][i], b["z"][i]]) * 8
        touches = all(o[a] - 1 < hi[a] and o[a] + 9 > lo[a] for a in range(3))
        inside = all(o[a] >= lo[a] and o[a] + 8 <= hi[a] for a in range(3))
        assert fl[i] == (1 if touches and not inside else 0), (i, o)
