"""Geometry placement over the C ABI (fl_geometry_*, fl_stl_voxelize): implicit
spheres, boxes and cylinders and STL meshes, voxelised on the GPU.

Mirrors src/geometry (GeometryDescriptor, ImplicitEvaluator, SimpleSTLVoxelizer,
GeometryPlacer).  `load_stl` reads binary or ASCII STL the way
SimpleSTLVoxelizer::loadSTL does (binary first: 80-byte header, uint32 count,
then per triangle a normal, three vertices and a 2-byte attribute; else the
ASCII `vertex` lines of each facet).
"""
import ctypes
import struct

import numpy as np

from .runtime import DeviceArray

STL, IMPLICIT, BOX, SPHERE, CYLINDER = range(5)


class GeometryDesc(ctypes.Structure):
    _fields_ = [("type", ctypes.c_int32), ("material_id", ctypes.c_int32), ("translate", ctypes.c_float * 3),
                ("scale", ctypes.c_float * 3), ("rotate", ctypes.c_float * 3), ("radius", ctypes.c_float),
                ("height", ctypes.c_float), ("width", ctypes.c_float), ("length", ctypes.c_float)]


def make(kind, translate=(0.0, 0.0, 0.0), scale=(1.0, 1.0, 1.0), radius=1.0, height=1.0, width=1.0, length=1.0,
         material_id=1):
    d = GeometryDesc()
    d.type = kind
    d.material_id = material_id
    d.translate[:] = list(translate)
    d.scale[:] = list(scale)
    d.radius, d.height, d.width, d.length = radius, height, width, length
    return d


def load_stl(path):
    """Triangles of an STL file as float32 (ntri, 9) [v1, v2, v3]."""
    raw = open(path, "rb").read()
    if len(raw) >= 84:
        n = struct.unpack_from("<I", raw, 80)[0]
        if n and 84 + n * 50 <= len(raw):
            rec = np.frombuffer(raw, dtype=np.dtype([("f", "<f4", 12), ("a", "<u2")]), count=n, offset=84)
            return np.ascontiguousarray(rec["f"][:, 3:12], np.float32)
    verts = [list(map(float, line.split()[1:4])) for line in raw.decode(errors="replace").splitlines()
             if line.strip().startswith("vertex")]
    return np.asarray(verts, np.float32).reshape(-1, 9)


def write_stl(path, tris):
    """Binary STL of (ntri, 9) triangles (normals zero)."""
    tris = np.asarray(tris, np.float32).reshape(-1, 9)
    rec = np.zeros(len(tris), dtype=np.dtype([("f", "<f4", 12), ("a", "<u2")]))
    rec["f"][:, 3:12] = tris
    with open(path, "wb") as fh:
        fh.write(b"\0" * 80 + struct.pack("<I", len(tris)) + rec.tobytes())


def aabb(ctx, d):
    b = (ctypes.c_float * 6)()
    ctx.lib.fl_geometry_aabb(ctypes.byref(d), b)
    return list(b)


def inside(ctx, d, pts):
    pts = np.asarray(pts, np.float32).reshape(-1, 3)
    cols = [DeviceArray.from_host(ctx, np.ascontiguousarray(pts[:, a])) for a in range(3)]
    out = DeviceArray(ctx, (len(pts),), np.uint8)
    ctx.call("fl_geometry_inside", ctypes.byref(d), *[c.ptr for c in cols], ctypes.c_size_t(len(pts)), out.ptr)
    return out.to_host().astype(bool)


def evaluate(ctx, d, cells):
    cells = np.asarray(cells, np.int32).reshape(-1, 3)
    cols = [DeviceArray.from_host(ctx, np.ascontiguousarray(cells[:, a])) for a in range(3)]
    out = DeviceArray(ctx, (len(cells),), np.uint8)
    ctx.call("fl_geometry_evaluate", ctypes.byref(d), *[c.ptr for c in cols], ctypes.c_size_t(len(cells)), out.ptr)
    return out.to_host().astype(bool)


def voxelize(ctx, tris, d, cell_size, cap=1 << 22):
    """Cells (n, 3) of the mesh's voxelisation, in z, y, x order."""
    tris = np.ascontiguousarray(tris, np.float32).reshape(-1, 9)
    out = [DeviceArray(ctx, (cap,), np.int32) for _ in range(3)]
    n = ctypes.c_size_t()
    ctx.call("fl_stl_voxelize", tris.ctypes.data_as(ctypes.c_void_p), ctypes.c_size_t(len(tris)), ctypes.byref(d),
             ctypes.c_float(cell_size), *[o.ptr for o in out], ctypes.c_size_t(cap), ctypes.byref(n))
    return np.stack([o.to_host()[:n.value] for o in out], -1)


def process(ctx, d, cell_size, domain_box, tris=None, cap=1 << 22):
    """GeometryPlacer::processGeometry: cells (n, 3), material ids and level-8 keys."""
    t = np.ascontiguousarray(tris if tris is not None else np.zeros((0, 9)), np.float32).reshape(-1, 9)
    out = [DeviceArray(ctx, (cap,), np.int32) for _ in range(4)]
    key = DeviceArray(ctx, (cap,), np.uint64)
    box = (ctypes.c_float * 6)(*domain_box)
    n = ctypes.c_size_t()
    ctx.call("fl_geometry_process", ctypes.byref(d), t.ctypes.data_as(ctypes.c_void_p), ctypes.c_size_t(len(t)),
             ctypes.c_float(cell_size), box, *[o.ptr for o in out], key.ptr, ctypes.c_size_t(cap), ctypes.byref(n))
    k = n.value
    return np.stack([o.to_host()[:k] for o in out[:3]], -1), out[3].to_host()[:k], key.to_host()[:k]



def _cell_bound(ctx, d, t, dims):
    """Cells fl_geometry_process can return for one geometry on the grid `dims`."""
    if d.type == STL:  # the whole inclusive grid range of the transformed mesh bounds
        if not len(t):
            return 0
        v = t.reshape(-1, 3).astype(np.float64) * np.array(d.scale) + np.array(d.translate)
        lo, hi = v.min(0), v.max(0)
        return int(np.prod(np.ceil(hi) - np.floor(lo) + 2))
    b = np.array(aabb(ctx, d), np.float64)  # clipped to the grid, cells [floor, ceil)
    lo, hi = np.maximum(b[:3], 0.0), np.minimum(b[3:], dims)
    return int(np.prod(np.maximum(np.ceil(hi) - np.floor(lo), 0.0)))


def place(ctx, pool, case_id, level, geoms):
    """Place geometries as solid into one case of a pool.  `geoms` is a list of
    (GeometryDesc, triangles or None), each written in voxel units of the
    case's level-`level` grid; their cells (cell size 1; implicit shapes
    clipped to the grid) are made on the GPU by fl_geometry_process into one
    device buffer and handed to fl_pool_set_solid_cells without leaving the
    device (the mask is their union).  Returns the number of cells placed."""
    nz, ny, nx = pool.mask_shape(case_id, level)
    dims = np.array([nx, ny, nz], np.float64)
    items = []
    for d, tris in geoms:
        t = np.ascontiguousarray(tris if tris is not None else np.zeros((0, 9)), np.float32).reshape(-1, 9)
        items.append((d, t, _cell_bound(ctx, d, t, dims)))
    cap = max(1, sum(k for _, _, k in items))
    out = [DeviceArray(ctx, (cap,), np.int32) for _ in range(3)]
    box = (ctypes.c_float * 6)(0.0, 0.0, 0.0, float(nx), float(ny), float(nz))
    used = 0
    for d, t, k in items:
        n = ctypes.c_size_t()
        at = [ctypes.c_void_p(o.ptr.value + 4 * used) for o in out]
        ctx.call("fl_geometry_process", ctypes.byref(d), t.ctypes.data_as(ctypes.c_void_p), ctypes.c_size_t(len(t)),
                 ctypes.c_float(1.0), box, *at, None, None, ctypes.c_size_t(cap - used), ctypes.byref(n))
        used += n.value
    pool.set_solid_cells(case_id, level, out[0].ptr, out[1].ptr, out[2].ptr, used)
    return used
