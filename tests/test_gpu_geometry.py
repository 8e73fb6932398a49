"""Geometry placement on the GPU against the oracle (itself pinned to the
reference's geometry sources on the host): implicit evaluation of points and
cells, STL voxelisation, and processGeometry's candidates, materials and keys."""
import numpy as np
import pytest

from fluidloom_gb300 import geometry as G
from tests import _oracle as O
from tests.test_geometry_host import cube_mesh, descs, ico_mesh

pytestmark = pytest.mark.gpu


def test_implicit_points_and_cells(ctx):
    rng = np.random.default_rng(11)
    pts = rng.uniform(-10, 10, (50000, 3)).astype(np.float32)
    cells = rng.integers(-12, 12, (50000, 3)).astype(np.int32)
    for d in descs(rng):
        np.testing.assert_array_equal(G.inside(ctx, d, pts), O.geometry_inside(d, pts))
        np.testing.assert_array_equal(G.evaluate(ctx, d, cells), O.geometry_evaluate(d, cells))
        assert G.aabb(ctx, d) == list(O.geometry_aabb(d))


@pytest.mark.parametrize("mesh", ["cube", "ico"])
def test_stl_voxelize(ctx, mesh):
    tris = cube_mesh((-1.3, -0.7, 0.2), (2.1, 1.6, 3.05)) if mesh == "cube" else ico_mesh()
    for scale, trans, cell in (((1, 1, 1), (0, 0, 0), 0.25), ((1.5, 0.8, 1.2), (2.0, -1.0, 0.5), 0.1)):
        d = G.make(G.STL, translate=trans, scale=scale)
        got = G.voxelize(ctx, tris, d, cell)
        want = O.stl_voxelize(tris, d, cell)
        assert len(want) > 10
        np.testing.assert_array_equal(got, want)


def test_process_geometry(ctx):
    dom = [-4.0, -4.0, -4.0, 20.0, 20.0, 20.0]
    sph = G.make(G.SPHERE, translate=(6.0, 5.0, 7.0), radius=4.5, material_id=7)
    cells, mat, key = G.process(ctx, sph, 1.0, dom)
    want = O.geometry_candidates(sph, 1.0, dom)
    np.testing.assert_array_equal(cells, want)
    assert (mat == 7).all()
    np.testing.assert_array_equal(key, O.hilbert_encode(cells[:, 0], cells[:, 1], cells[:, 2], 8))
    tris = ico_mesh(r=2.5, c=(1.0, 1.0, 1.0))
    stl = G.make(G.STL, material_id=3)
    cells, mat, key = G.process(ctx, stl, 0.2, dom, tris=tris)
    np.testing.assert_array_equal(cells, O.stl_voxelize(tris, stl, 0.2))
    assert (mat == 3).all() and len(key) == len(cells)
