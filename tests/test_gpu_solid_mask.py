"""Solid masks on the GPU pool vs the CPU oracle: a box of mask voxels at a
level coarser than, equal to and finer than the bricks (centre sampling and
containing-voxel sampling), a cylinder placed by the geometry kernels into a
sphere channel (mask OR sphere, periodic halo), and removal of the mask.
Populations compared with 1e-5 relative tolerance (expected difference zero:
the kernels are built without FMA contraction)."""
import numpy as np
import pytest

from fluidloom_gb300 import geometry, lbm
from tests import _oracle as O
from tests.test_gpu_lbm import assert_pool_equal

pytestmark = pytest.mark.gpu


def _channel():
    c = lbm.sphere_channel(64, 32, 32, 2, radius=4.0, centre=(16.0, 16.0, 16.0), u_in=0.04, band=3.0)
    c.has_sphere = 0
    return c


def _box(shape, lo, hi):
    m = np.zeros(shape, bool)
    m[lo[2]:hi[2], lo[1]:hi[1], lo[0]:hi[0]] = True
    return m


def _run_both(gp, op, rounds=2):
    for _ in range(rounds):
        gp.step(3)
        op.step(3)
        assert_pool_equal(gp, op)
        np.testing.assert_allclose(gp.conservation(), op.conservation(), rtol=1e-12, atol=1e-9)
        gfl, gwm = gp.flags()
        ofl, owm = op.flags()
        np.testing.assert_array_equal(gfl, ofl)
        np.testing.assert_array_equal(gwm, owm)
        gp.regrid()
        op.regrid()
        assert_pool_equal(gp, op)
        assert gp.info().fluid_lups_per_step == op.lups()


@pytest.mark.parametrize("level", [0, 1, 2])
def test_box_mask_vs_oracle(ctx, level):
    from fluidloom_gb300.lbm import Pool
    c = _channel()
    gp, op = Pool(ctx, [c]), O.OraclePool([c])
    s = 1 << level
    m = _box(gp.mask_shape(0, level), (20 * s + s // 2, 12 * s, 10 * s), (27 * s, 19 * s + s // 2, 22 * s))
    gp.set_solid_mask(0, level, m)
    op.set_mask(0, level, lbm.pack_mask(m))
    lv, back = gp.solid_mask(0)
    assert lv == level and np.array_equal(back, m)
    assert gp.info().fluid_lups_per_step == op.lups() < c.ext[0] * c.ext[1] * c.ext[2] * 512
    _run_both(gp, op)
    assert gp.bricks()["level"].max() == 2  # the mask band refined to max_level


def test_placed_cylinder_with_sphere_vs_oracle(ctx):
    from fluidloom_gb300.lbm import Pool
    c = lbm.sphere_channel(64, 32, 32, 2, radius=3.0, centre=(12.0, 16.0, 16.0), u_in=0.04, band=2.0)
    gp, op = Pool(ctx, [c]), O.OraclePool([c])
    # a cylinder along y at level 1 (voxel units), crossing the periodic y faces
    cyl = geometry.make(geometry.CYLINDER, translate=(80.0, 32.0, 30.0), radius=6.0, height=200.0)
    n = geometry.place(ctx, gp, 0, 1, [(cyl, None)])
    lv, m = gp.solid_mask(0)
    assert lv == 1 and m.sum() == n > 0
    z, y, x = np.meshgrid(*[np.arange(k, dtype=np.float32) for k in m.shape], indexing="ij")
    f = np.float32
    lx, lz = (x + f(0.5) - f(80.0)) / f(1.0), (z + f(0.5) - f(30.0)) / f(1.0)
    want = (lx * lx + lz * lz <= f(36.0)) & (np.abs((y + f(0.5) - f(32.0)) / f(1.0)) <= f(100.0))
    np.testing.assert_array_equal(m, want)
    op.set_mask(0, 1, lbm.pack_mask(m))
    assert gp.info().fluid_lups_per_step == op.lups()
    _run_both(gp, op)


def test_mask_removal(ctx):
    from fluidloom_gb300.lbm import Pool
    c = _channel()
    gp, op, fresh = Pool(ctx, [c]), O.OraclePool([c]), Pool(ctx, [c])
    m = _box(gp.mask_shape(0, 0), (24, 8, 8), (32, 24, 24))
    gp.set_solid_mask(0, 0, m)
    op.set_mask(0, 0, lbm.pack_mask(m))
    gp.step(2)
    op.step(2)
    gp.set_solid_mask(0, 0, None)
    op.set_mask(0, 0, None)
    assert gp.solid_mask(0) == (-1, None)
    assert gp.info().fluid_lups_per_step == fresh.info().fluid_lups_per_step == op.lups()
    _run_both(gp, op, rounds=1)


def test_masked_case_leaves_a_batch(ctx):
    from fluidloom_gb300.lbm import Pool
    a, b = lbm.cavity(16, 1, u_lid=0.06, tau=0.6), _channel()
    gp, ref = Pool(ctx, [a, b]), Pool(ctx, [a])
    gp.set_solid_mask(1, 0, _box(gp.mask_shape(1, 0), (24, 8, 8), (32, 24, 24)))
    gp.remove_cases([1])
    for p in (gp, ref):
        p.step(3)
        p.regrid()
        p.step(2)
    np.testing.assert_array_equal(gp.populations(), ref.populations())
    ids = gp.add_cases([b])  # the freed slot comes back without a mask
    assert ids == [1] and gp.solid_mask(1) == (-1, None)
