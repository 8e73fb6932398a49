"""Snapshot / restart and site fields on the GPU: a pool restored from a
snapshot continues bit for bit like the pool it was taken from (also with a
removed case); the macroscopic fields equal the FP32 moments of the populations;
the VTK file carries them."""
import numpy as np
import pytest

from fluidloom_gb300 import io

pytestmark = pytest.mark.gpu


def _cases():
    from fluidloom_gb300 import lbm
    cav = lbm.cavity(16, 1, u_lid=0.06, tau=0.6)
    sph = lbm.sphere_channel(32, 16, 16, 2, radius=2.0, centre=(8.0, 8.0, 8.0), u_in=0.04, band=2.0)
    cav2 = lbm.cavity(24, 2, u_lid=0.03, tau=0.55)
    return cav, sph, cav2


def _same(p, q):
    a, b = p.bricks(), q.bricks()
    for k in ("x", "y", "z", "level", "case_id"):
        np.testing.assert_array_equal(a[k], b[k])
    np.testing.assert_array_equal(p.populations(), q.populations())


def _advance(p):
    p.step(4)
    p.regrid()
    p.step(3)


def test_snapshot_restart_continues_bit_for_bit(ctx, tmp_path):
    from fluidloom_gb300.lbm import Pool
    cav, sph, cav2 = _cases()
    p = Pool(ctx, [cav, sph, cav2])
    _advance(p)
    p.remove_cases([0])
    p.step(1)  # an odd number of level-0 steps: level 0 ends on the other buffer
    path = io.save_snapshot(p, str(tmp_path / "snap.npz"))
    q = io.load_snapshot(ctx, path)
    _same(p, q)
    for r in (p, q):
        _advance(r)
    _same(p, q)
    np.testing.assert_array_equal(p.conservation()[1:], q.conservation()[1:])


def test_snapshot_keeps_solid_masks(ctx, tmp_path):
    from fluidloom_gb300.lbm import Pool
    cav, sph, _ = _cases()
    p = Pool(ctx, [cav, sph])
    m = np.zeros(p.mask_shape(1, 1), bool)
    m[10:20, 8:24, 40:50] = True
    p.set_solid_mask(1, 1, m)
    _advance(p)
    q = io.load_snapshot(ctx, io.save_snapshot(p, str(tmp_path / "masked.npz")))
    lv, back = q.solid_mask(1)
    assert lv == 1 and np.array_equal(back, m) and q.solid_mask(0) == (-1, None)
    assert q.info().fluid_lups_per_step == p.info().fluid_lups_per_step
    for r in (p, q):
        _advance(r)
    _same(p, q)


def _moments(f):
    """The kernels' FP32 moment order (rho, then j by pairs) in numpy float32."""
    r = f[0].copy()
    for q in range(1, 19):
        r = r + f[q]
    a = f[1] - f[2]
    for u, v in ((7, 8), (9, 10), (11, 12), (13, 14)):
        a = a + (f[u] - f[v])
    b = f[3] - f[4]
    for u, v in ((7, 8), (10, 9), (15, 16), (17, 18)):
        b = b + (f[u] - f[v])
    c = f[5] - f[6]
    for u, v in ((11, 12), (14, 13), (15, 16), (18, 17)):
        c = c + (f[u] - f[v])
    inv = np.float32(1.0) / r
    return r, a * inv, b * inv, c * inv


def test_macroscopic_fields_and_vtk(ctx, tmp_path):
    from fluidloom_gb300.lbm import Pool
    cav, _, _ = _cases()
    p = Pool(ctx, [cav])
    p.step(6)
    m = p.macroscopic()
    r, ux, uy, uz = _moments(p.populations())
    np.testing.assert_array_equal(m["density"], r)
    np.testing.assert_array_equal(m["velocity"][..., 0], ux)
    np.testing.assert_array_equal(m["velocity"][..., 1], uy)
    np.testing.assert_array_equal(m["velocity"][..., 2], uz)
    path = io.VTKWriter(str(tmp_path / "out")).write_snapshot(6, 0.0, p)
    a = io.read_vtp_arrays(path)
    n = p.info().num_bricks
    assert a["Points"].shape == (n * 512, 3)
    np.testing.assert_array_equal(a["Density"], m["density"].reshape(-1))
    np.testing.assert_array_equal(a["Level"], np.repeat(p.bricks()["level"].astype(np.int32), 512))


def test_sphere_sites_report_zero(ctx):
    from fluidloom_gb300.lbm import Pool
    _, sph, _ = _cases()
    p = Pool(ctx, [sph])
    p.step(2)
    m = p.macroscopic()
    solid = m["density"] == 0
    assert solid.any() and (m["velocity"][solid] == 0).all()
    assert np.isfinite(m["density"]).all() and (m["density"][~solid] > 0.5).all()
