"""Scripts run on the GPU: a cavity script gives exactly the populations of the
same case stepped and regridded directly; a sphere script's pre-refinement loop
refines the bricks near the sphere to the maximum level; the VTK output of
final_output is written."""
import os

import numpy as np
import pytest

from fluidloom_gb300 import dsl

pytestmark = pytest.mark.gpu
SCEN = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "fluidloom_gb300", "scenarios")


def test_cavity_script_equals_direct_pool(ctx, tmp_path):
    from fluidloom_gb300.lbm import Pool
    sc = dsl.Scenario(dsl.parse(open(os.path.join(SCEN, "cavity.fl")).read()), ext=(2, 2, 2), max_level=1)
    logs = []
    r = dsl.Runner(ctx, sc, str(tmp_path), log=logs.append)
    r.initial()
    r.run(45)
    r.final()
    ref = Pool(ctx, [sc.case()])
    for _ in range(2):
        ref.step(20)
        ref.regrid()
    ref.step(5)
    a, b = r.pool.bricks(), ref.bricks()
    for k in ("x", "y", "z", "level"):
        np.testing.assert_array_equal(a[k], b[k])
    np.testing.assert_array_equal(r.pool.populations(), ref.populations())
    assert r.regrids == 2 and logs[0].startswith("cells: ") and logs[-1] == "done"
    assert any(l.startswith("step 40, cells ") for l in logs)
    assert os.path.exists(os.path.join(str(tmp_path), "cavity_final.vtp"))


def test_sphere_script_prerefines_near_the_sphere(ctx, tmp_path):
    src = """
        import "d3q19.lattice"
        field velocity: vector
        field refine_flag: int
        initial_condition: {
            place_geometry(type = "sphere", center = (8.0, 8.0, 8.0), radius = 2.0)
            for i in 0..num_cells {
                velocity[i] = (0.04, 0.0, 0.0)
                vector p = cell_position(i)
                if distance(p, (8.0, 8.0, 8.0)) < 8.0 { refine_flag[i] = 2 }
            }
            adapt_mesh()
        }
        time_loop: {
            run lbm_collide_stream()
            run apply_inlet_velocity(velocity_inlet = (0.04, 0.0, 0.0))
            run apply_outlet_zero_gradient()
        }
    """
    sc = dsl.Scenario(dsl.parse(src), ext=(4, 2, 2), max_level=2)
    r = dsl.Runner(ctx, sc, str(tmp_path), log=lambda s: None)
    r.initial()
    b = r.pool.bricks()
    assert b["level"].max() == 2
    c = (b["x"] * 8 + 4.0) / (1 << b["level"].astype(np.int64))
    fine = b["level"] == 2
    assert np.all(np.abs(c[fine] - 8.0) < 8.0)
    secs = r.run(6)
    assert secs > 0 and r.lups > 0


def test_obstacle_script_equals_direct_pool(ctx, tmp_path):
    """Box and cylinder of a script become the case's solid mask (GPU voxelised),
    the mesh is pre-refined around them, and the run equals the same steps on a
    pool built directly."""
    from fluidloom_gb300 import geometry
    from fluidloom_gb300.lbm import Pool
    sc = dsl.Scenario(dsl.parse(open(os.path.join(SCEN, "obstacles.fl")).read()), ext=(8, 8, 8), max_level=1,
                      mask_level=1)
    r = dsl.Runner(ctx, sc, str(tmp_path), log=lambda *_: None)
    r.initial()
    r.run(30)
    ref = Pool(ctx, [sc.case()])
    n = geometry.place(ctx, ref, 0, 1, sc.solid_geometries())
    ref.regrid()
    ref.step(25)
    ref.regrid()
    ref.step(5)
    assert r.solid_cells == n > 0
    lv, m = r.pool.solid_mask(0)
    assert lv == 1 and m.sum() == n
    a, b = r.pool.bricks(), ref.bricks()
    for k in ("x", "y", "z", "level"):
        np.testing.assert_array_equal(a[k], b[k])
    assert (a["level"] == 1).any()
    np.testing.assert_array_equal(r.pool.populations(), ref.populations())
