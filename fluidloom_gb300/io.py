"""Pool output and restart: VTK XML PolyData snapshots of the site fields and
bit-exact snapshots of a pool's state.

`VTKWriter` follows the reference's writer (src/io/VTKWriter.cpp:19-95): one
`snapshot_<step:06d>.vtp` per call in the output directory, points at cell
centres with a `Level` array -- here every lattice site of every brick, in the
level-0 lattice units of its case, with `Density`, `Velocity` and `CaseId`
added (the reference leaves the field arrays as a TODO, VTKWriter.cpp:83-88).
Arrays are base64 binary (or ASCII, for small checks).

`save_snapshot` / `load_snapshot` keep the cases, bricks and current
populations; a pool restored from a snapshot continues bit for bit like the
pool it was taken from.
"""
import base64
import os

import numpy as np

from .lbm import LbmCase, Pool, pack_mask, unpack_mask


def _site_points(bricks):
    s = np.arange(512)
    lx, ly, lz = s & 7, (s >> 3) & 7, s >> 6
    scale = 1.0 / (1 << bricks["level"].astype(np.int64))[:, None]
    px = (bricks["x"][:, None].astype(np.float64) * 8 + lx + 0.5) * scale
    py = (bricks["y"][:, None].astype(np.float64) * 8 + ly + 0.5) * scale
    pz = (bricks["z"][:, None].astype(np.float64) * 8 + lz + 0.5) * scale
    return np.stack([px, py, pz], -1).reshape(-1, 3).astype(np.float32)


def _data_array(name, a, ncomp, vtype, ascii_):
    a = np.ascontiguousarray(a)
    head = '<DataArray type="%s" Name="%s"%s format="%s">' % (
        vtype, name, ' NumberOfComponents="%d"' % ncomp if ncomp > 1 else "", "ascii" if ascii_ else "binary")
    if ascii_:
        body = " ".join(str(v) for v in a.reshape(-1).tolist())
    else:
        raw = a.tobytes()
        body = base64.b64encode(np.uint64(len(raw)).tobytes() + raw).decode()
    return "        %s\n          %s\n        </DataArray>\n" % (head, body)


def write_vtp(path, pool, case=None, ascii=False, per="site"):
    """One VTK PolyData file of the pool's sites (per="site") or brick centres
    (per="brick", with the mean over the brick's fluid sites), optionally of one case."""
    b = pool.bricks()
    m = pool.macroscopic()
    keep = np.ones(len(b["x"]), bool) if case is None else b["case_id"] == case
    b = {k: v[keep] for k, v in b.items()}
    rho_s, vel_s = m["density"][keep], m["velocity"][keep]
    if per == "site":
        pts = _site_points(b)
        rho = rho_s.reshape(-1)
        vel = vel_s.reshape(-1, 3)
        level = np.repeat(b["level"].astype(np.int32), 512)
        cid = np.repeat(b["case_id"].astype(np.int32), 512)
    else:
        scale = 1.0 / (1 << b["level"].astype(np.int64))
        pts = np.stack([(b[a].astype(np.float64) * 8 + 4.0) * scale for a in ("x", "y", "z")], -1).astype(np.float32)
        fluid = np.maximum((rho_s != 0).sum(1), 1)
        rho = (rho_s.sum(1) / fluid).astype(np.float32)
        vel = (vel_s.sum(1) / fluid[:, None]).astype(np.float32)
        level = b["level"].astype(np.int32)
        cid = b["case_id"].astype(np.int32)
    n = len(pts)
    os.makedirs(os.path.dirname(os.path.abspath(path)), exist_ok=True)
    with open(path, "w") as fh:
        fh.write('<?xml version="1.0"?>\n')
        fh.write('<VTKFile type="PolyData" version="1.0" byte_order="LittleEndian" header_type="UInt64">\n')
        fh.write("  <PolyData>\n")
        fh.write('    <Piece NumberOfPoints="%d" NumberOfVerts="%d">\n' % (n, n))
        fh.write("      <Points>\n")
        fh.write(_data_array("Points", pts, 3, "Float32", ascii))
        fh.write("      </Points>\n      <Verts>\n")
        fh.write(_data_array("connectivity", np.arange(n, dtype=np.int64), 1, "Int64", ascii))
        fh.write(_data_array("offsets", np.arange(1, n + 1, dtype=np.int64), 1, "Int64", ascii))
        fh.write("      </Verts>\n      <PointData>\n")
        fh.write(_data_array("Level", level, 1, "Int32", ascii))
        fh.write(_data_array("CaseId", cid, 1, "Int32", ascii))
        fh.write(_data_array("Density", rho, 1, "Float32", ascii))
        fh.write(_data_array("Velocity", vel, 3, "Float32", ascii))
        fh.write("      </PointData>\n    </Piece>\n  </PolyData>\n</VTKFile>\n")
    return path


class VTKWriter:
    """VTKWriter(output_dir).write_snapshot(step, time, pool) -> output_dir/snapshot_<step>.vtp."""

    def __init__(self, output_dir, ascii=False, per="site"):
        self.output_dir = output_dir
        self.ascii = ascii
        self.per = per
        os.makedirs(output_dir, exist_ok=True)

    def write_snapshot(self, step, time, pool, case=None):
        del time  # the .vtp carries no time, as in the reference
        return write_vtp(os.path.join(self.output_dir, "snapshot_%06d.vtp" % step), pool, case, self.ascii, self.per)


def read_vtp_arrays(path):
    """The binary or ASCII DataArrays of a file written above, by name (for tests and tools)."""
    import re
    txt = open(path).read()
    out = {}
    for m in re.finditer(r'<DataArray type="(\w+)" Name="(\w+)"(?: NumberOfComponents="(\d+)")? format="(\w+)">'
                         r'\s*(.*?)\s*</DataArray>', txt, re.S):
        vtype, name, nc, fmt, body = m.groups()
        dt = {"Float32": np.float32, "Int32": np.int32, "Int64": np.int64}[vtype]
        if fmt == "ascii":
            a = np.array(body.split(), dtype=dt)
        else:
            raw = base64.b64decode(body)
            a = np.frombuffer(raw[8:8 + int(np.frombuffer(raw[:8], np.uint64)[0])], dt)
        out[name] = a.reshape(-1, int(nc)) if nc else a
    return out


def save_snapshot(pool, path):
    """Cases, bricks and current populations of a pool, as one .npz file."""
    b = pool.bricks()
    f = pool.populations()
    active = np.zeros(len(pool.cases), bool)
    active[np.unique(b["case_id"])] = True
    cases = np.frombuffer(b"".join(bytes(c) if c is not None else bytes(LbmCase()) for c in pool.cases), np.uint8)
    masks = {}
    for c in np.flatnonzero(active):
        lv, m = pool.solid_mask(int(c))
        if lv >= 0:
            masks["mask_level_%d" % c] = np.int32(lv)
            masks["mask_words_%d" % c] = pack_mask(m)
    np.savez(path, version=np.int32(1), cases=cases, active=active, f=f, **b, **masks)
    return path


def load_snapshot(ctx, path):
    """A new pool in the saved state (removed cases stay removed)."""
    z = np.load(path)
    if int(z["version"]) != 1:
        raise ValueError("unknown snapshot version %d" % int(z["version"]))
    raw = z["cases"].tobytes()
    size = ctypes_sizeof_case()
    cases = [LbmCase.from_buffer_copy(raw[i * size:(i + 1) * size]) for i in range(len(raw) // size)]
    pool = Pool(ctx, cases)
    gone = [i for i, a in enumerate(z["active"]) if not a]
    if gone:
        pool.remove_cases(gone)
    pool.load({k: z[k] for k in ("x", "y", "z", "level", "case_id")}, z["f"])
    for c in np.flatnonzero(z["active"]):
        if "mask_level_%d" % c in z.files:
            lv = int(z["mask_level_%d" % c])
            pool.set_solid_mask(int(c), lv, unpack_mask(z["mask_words_%d" % c], pool.mask_shape(int(c), lv)))
    return pool


def ctypes_sizeof_case():
    import ctypes
    return ctypes.sizeof(LbmCase)
