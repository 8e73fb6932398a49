"""Geometry oracle on the host: the implicit evaluator, AABBs and the STL
voxeliser against the reference's own ImplicitEvaluator.cpp and
SimpleSTLVoxelizer.cpp compiled in place (oracle/Makefile.ref; skipped where the
reference tree is absent), plus the reader of binary STL files."""
import ctypes
import os

import numpy as np
import pytest

from fluidloom_gb300 import geometry as G
from tests import _oracle as O

REF = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle", "_ref",
                   "libfl_ref_geometry.so")
P = ctypes.c_void_p


def ref():
    if not os.path.exists(REF):
        pytest.skip("reference geometry not built (reference tree absent)")
    L = ctypes.CDLL(REF)
    fl = ctypes.c_float
    L.ref_geometry_inside.argtypes = [ctypes.c_int, P, P, fl, fl, fl, fl, P, P, P, ctypes.c_size_t, P]
    L.ref_stl_voxelize.restype = ctypes.c_size_t
    L.ref_stl_voxelize.argtypes = [ctypes.c_char_p, P, P, fl, P, P, P, ctypes.c_size_t]
    L.ref_geometry_aabb.argtypes = [ctypes.c_int, P, P, fl, fl, fl, fl, P]
    return L


def descs(rng, n=12):
    out = []
    for k in range(n):
        kind = [G.BOX, G.SPHERE, G.CYLINDER, G.IMPLICIT][k % 4]
        out.append(G.make(kind, translate=rng.uniform(-5, 5, 3), scale=rng.uniform(0.5, 2.0, 3),
                          radius=float(rng.uniform(0.5, 4)), height=float(rng.uniform(0.5, 6)),
                          width=float(rng.uniform(0.5, 6)), length=float(rng.uniform(0.5, 6))))
    return out


def _args(d):
    t = np.array(d.translate, np.float32)
    s = np.array(d.scale, np.float32)
    return t, s


def test_implicit_and_aabb_match_reference():
    L = ref()
    rng = np.random.default_rng(7)
    pts = rng.uniform(-10, 10, (20000, 3)).astype(np.float32)
    cols = [np.ascontiguousarray(pts[:, a]) for a in range(3)]
    for d in descs(rng):
        t, s = _args(d)
        want = np.zeros(len(pts), np.uint8)
        L.ref_geometry_inside(d.type, O.ptr(t), O.ptr(s), d.radius, d.height, d.width, d.length,
                              *[O.ptr(c) for c in cols], len(pts), O.ptr(want))
        np.testing.assert_array_equal(O.geometry_inside(d, pts), want.astype(bool))
        b = np.zeros(6, np.float32)
        L.ref_geometry_aabb(d.type, O.ptr(t), O.ptr(s), d.radius, d.height, d.width, d.length, O.ptr(b))
        np.testing.assert_array_equal(O.geometry_aabb(d), b)


def cube_mesh(lo=(0.0, 0.0, 0.0), hi=(1.0, 1.0, 1.0)):
    """Closed axis-aligned box of 12 triangles."""
    x0, y0, z0 = lo
    x1, y1, z1 = hi
    v = np.array([[x0, y0, z0], [x1, y0, z0], [x1, y1, z0], [x0, y1, z0],
                  [x0, y0, z1], [x1, y0, z1], [x1, y1, z1], [x0, y1, z1]], np.float32)
    f = [(0, 2, 1), (0, 3, 2), (4, 5, 6), (4, 6, 7), (0, 1, 5), (0, 5, 4),
         (2, 3, 7), (2, 7, 6), (1, 2, 6), (1, 6, 5), (0, 4, 7), (0, 7, 3)]
    return np.stack([np.concatenate([v[a], v[b], v[c]]) for a, b, c in f]).astype(np.float32)


def ico_mesh(r=3.0, c=(0.3, -0.2, 0.1), sub=2):
    """Subdivided octahedron projected on a sphere."""
    v = [np.array(p, float) for p in ((1, 0, 0), (-1, 0, 0), (0, 1, 0), (0, -1, 0), (0, 0, 1), (0, 0, -1))]
    faces = [(0, 2, 4), (2, 1, 4), (1, 3, 4), (3, 0, 4), (2, 0, 5), (1, 2, 5), (3, 1, 5), (0, 3, 5)]
    tris = [(v[a], v[b], v[cc]) for a, b, cc in faces]
    for _ in range(sub):
        nt = []
        for a, b, cc in tris:
            ab, bc, ca = [(p + q) / np.linalg.norm(p + q) for p, q in ((a, b), (b, cc), (cc, a))]
            nt += [(a, ab, ca), (ab, b, bc), (ca, bc, cc), (ab, bc, ca)]
        tris = nt
    return np.array([np.concatenate([p * r + c for p in t]) for t in tris], np.float32)


@pytest.mark.parametrize("mesh", ["cube", "ico"])
def test_stl_voxelize_matches_reference(tmp_path, mesh):
    L = ref()
    tris = cube_mesh((-1.3, -0.7, 0.2), (2.1, 1.6, 3.05)) if mesh == "cube" else ico_mesh()
    path = str(tmp_path / "m.stl")
    G.write_stl(path, tris)
    np.testing.assert_array_equal(G.load_stl(path), tris)
    for scale, trans, cell in (((1, 1, 1), (0, 0, 0), 0.25), ((1.5, 0.8, 1.2), (2.0, -1.0, 0.5), 0.3)):
        d = G.make(G.STL, translate=trans, scale=scale)
        t, s = _args(d)
        cap = 1 << 20
        x, y, z = (np.zeros(cap, np.int32) for _ in range(3))
        n = L.ref_stl_voxelize(path.encode(), O.ptr(t), O.ptr(s), cell, O.ptr(x), O.ptr(y), O.ptr(z), cap)
        want = np.stack([x[:n], y[:n], z[:n]], -1)
        got = O.stl_voxelize(tris, d, cell)
        assert len(want) > 10
        np.testing.assert_array_equal(got, want)
