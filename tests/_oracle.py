"""Loader for the CPU oracle (oracle/_build/liboracle.so) — tests only."""
import ctypes
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

P = ctypes.c_void_p
_lib = None


def ptr(a):
    return a.ctypes.data_as(P) if a is not None else None


class LbmCase(ctypes.Structure):
    _fields_ = [("ext", ctypes.c_int32 * 3), ("bc", ctypes.c_int32 * 6), ("wall_u", ctypes.c_float * 3),
                ("inlet_u", ctypes.c_float * 3), ("tau0", ctypes.c_float), ("max_level", ctypes.c_int32),
                ("has_sphere", ctypes.c_int32), ("sphere_c", ctypes.c_float * 3), ("sphere_r", ctypes.c_float),
                ("refine_frac", ctypes.c_float), ("coarsen_frac", ctypes.c_float), ("band", ctypes.c_float),
                ("init_u", ctypes.c_float * 3)]


class Mesh(ctypes.Structure):
    _fields_ = [("x", P), ("y", P), ("z", P), ("level", P), ("state", P), ("flags", P), ("material", P),
                ("case_id", P), ("n", ctypes.c_size_t)]


class Domain(ctypes.Structure):
    _fields_ = [("depth", ctypes.c_int), ("anchor_level", ctypes.c_int), ("max_level", ctypes.c_int),
                ("ext", ctypes.c_int32 * 3), ("periodic", ctypes.c_int32 * 3)]


class BalanceStats(ctypes.Structure):
    _fields_ = [("converged", ctypes.c_int32), ("iterations", ctypes.c_uint32), ("violations", ctypes.c_uint32),
                ("marked", ctypes.c_uint32), ("per_iter_violations", ctypes.c_uint32 * 64),
                ("per_iter_marked", ctypes.c_uint32 * 64)]


class AdaptCfg(ctypes.Structure):
    _fields_ = [("max_level", ctypes.c_int), ("min_level", ctypes.c_int), ("balance_mode", ctypes.c_int),
                ("max_balance_iterations", ctypes.c_int), ("enforce_balance", ctypes.c_int),
                ("averaging_rule", ctypes.c_int)]


class AdaptStats(ctypes.Structure):
    _fields_ = [("num_split", ctypes.c_uint32), ("num_children", ctypes.c_uint32), ("num_groups", ctypes.c_uint32),
                ("num_merged", ctypes.c_uint32), ("num_survivors", ctypes.c_uint32), ("num_out", ctypes.c_uint32),
                ("balance", BalanceStats)]


def load():
    global _lib
    if _lib is None:
        from oracle.build import build
        path = build()
        L = ctypes.CDLL(path)
        L.or_hilbert_encode1.restype = ctypes.c_uint64
        L.or_hilbert_encode1.argtypes = [ctypes.c_int32] * 3 + [ctypes.c_uint8]
        L.or_hilbert_encode.argtypes = [P, P, P, ctypes.c_uint8, P, P, ctypes.c_size_t]
        L.or_hilbert_decode.argtypes = [P, ctypes.c_uint8, P, P, P, ctypes.c_size_t]
        L.or_morton8_encode.argtypes = [P, P, P, P, ctypes.c_size_t]
        L.or_cell_keys.argtypes = [P, P, P, P, P, ctypes.c_int, ctypes.c_int, P, ctypes.c_size_t]
        L.or_sort_pairs_u64_u32.argtypes = [P, P, ctypes.c_size_t]
        L.or_scan_exclusive_u32.restype = ctypes.c_uint32
        L.or_scan_exclusive_u32.argtypes = [P, P, ctypes.c_size_t]
        L.or_compact_and_permute.restype = ctypes.c_size_t
        L.or_compact_and_permute.argtypes = [P, P, ctypes.c_size_t, P]
        L.or_apply_permutation.argtypes = [P, P, ctypes.c_size_t, ctypes.c_size_t, P]
        L.or_hash_capacity.restype = ctypes.c_uint64
        L.or_hash_capacity.argtypes = [ctypes.c_size_t]
        L.or_hash_build.restype = ctypes.c_int
        L.or_hash_build.argtypes = [P, P, ctypes.c_size_t, ctypes.c_uint64, P, P]
        L.or_hash_query.argtypes = [P, P, ctypes.c_uint64, P, P, ctypes.c_size_t]
        L.or_neighbours.argtypes = [ctypes.POINTER(Mesh), ctypes.POINTER(Domain), ctypes.c_int, P]
        L.or_balance.restype = ctypes.c_int
        L.or_balance.argtypes = [ctypes.POINTER(Mesh), ctypes.POINTER(Domain), ctypes.c_int, ctypes.c_int,
                                 ctypes.c_int, ctypes.POINTER(BalanceStats)]
        L.or_adapt.restype = ctypes.c_size_t
        L.or_adapt.argtypes = [ctypes.POINTER(Mesh), ctypes.POINTER(Domain), ctypes.POINTER(AdaptCfg), P,
                               ctypes.c_uint32, ctypes.c_int] + [P] * 12 + [ctypes.POINTER(AdaptStats)]
        L.or_interp_trilinear.argtypes = [ctypes.POINTER(Mesh), ctypes.POINTER(Domain), P, ctypes.c_uint32,
                                          P, P, P, P, ctypes.c_size_t, P]
        L.or_restrict_groups.argtypes = [P, ctypes.c_uint32, P, ctypes.c_size_t, ctypes.c_int, P]
        L.or_blob_flags.argtypes = [P, P, P, P, ctypes.c_size_t, P, ctypes.c_int, ctypes.c_float, ctypes.c_float,
                                    ctypes.c_int, P]
        L.or_pool_new.restype = P
        L.or_pool_new.argtypes = [ctypes.POINTER(LbmCase), ctypes.c_int]
        L.or_pool_free.argtypes = [P]
        L.or_pool_steps.argtypes = [P, ctypes.c_int, ctypes.c_int]
        L.or_pool_regrid.argtypes = [P]
        L.or_pool_regrid_flags.argtypes = [P, P]
        L.or_pool_upload.argtypes = [P, P]
        L.or_pool_flags.argtypes = [P, P, P]
        L.or_pool_size.restype = ctypes.c_size_t
        L.or_pool_size.argtypes = [P]
        L.or_pool_bricks.argtypes = [P, P, P, P, P, P]
        L.or_pool_nbr.argtypes = [P, P]
        L.or_pool_populations.argtypes = [P, P]
        L.or_pool_conservation.argtypes = [P, P]
        L.or_pool_fluid_lups.restype = ctypes.c_uint64
        L.or_pool_fluid_lups.argtypes = [P]
        L.or_pool_set_mask.argtypes = [P, ctypes.c_int, ctypes.c_int, P, ctypes.c_size_t]
        L.or_pool_fp64_steps.argtypes = [P, ctypes.c_int, ctypes.c_int, P]
        _lib = L
    return _lib


# ---- numpy conveniences -------------------------------------------------
def hilbert_encode(x, y, z, level):
    L = load()
    x, y, z = (np.ascontiguousarray(a, np.int32) for a in (x, y, z))
    k = np.empty(len(x), np.uint64)
    L.or_hilbert_encode(ptr(x), ptr(y), ptr(z), level, ptr(k), None, len(x))
    return k


def hilbert_decode(k, level):
    L = load()
    k = np.ascontiguousarray(k, np.uint64)
    x, y, z = (np.empty(len(k), np.int32) for _ in range(3))
    L.or_hilbert_decode(ptr(k), level, ptr(x), ptr(y), ptr(z), len(k))
    return x, y, z


def morton8(x, y, z):
    L = load()
    x, y, z = (np.ascontiguousarray(a, np.int32) for a in (x, y, z))
    k = np.empty(len(x), np.uint64)
    L.or_morton8_encode(ptr(x), ptr(y), ptr(z), ptr(k), len(x))
    return k


def cell_keys(x, y, z, level, case_id, depth, anchor_level):
    L = load()
    x, y, z = (np.ascontiguousarray(a, np.int32) for a in (x, y, z))
    level = np.ascontiguousarray(level, np.uint8)
    cs = None if case_id is None else np.ascontiguousarray(case_id, np.uint16)
    k = np.empty(len(x), np.uint64)
    L.or_cell_keys(ptr(x), ptr(y), ptr(z), ptr(level), ptr(cs), depth, anchor_level, ptr(k), len(x))
    return k


# ---- mesh helpers ---------------------------------------------------------
def mesh_struct(cols):
    """ctypes or_mesh over numpy columns (kept alive by the returned tuple)."""
    keep = {k: np.ascontiguousarray(v) for k, v in cols.items()}
    m = Mesh()
    for k in ("x", "y", "z", "level", "state", "flags", "material"):
        setattr(m, k, keep[k].ctypes.data_as(P))
    m.case_id = keep["case_id"].ctypes.data_as(P) if "case_id" in keep else None
    m.n = len(keep["x"])
    return m, keep


def anchor_for(ext, depth=21):
    """Deepest anchor level that keeps ext << A within the depth-bit key space."""
    e = max(ext)
    return depth - int(np.ceil(np.log2(e))) if e > 1 else depth


def domain(depth=21, anchor=None, max_level=21, ext=(1, 1, 1), periodic=(0, 0, 0)):
    if anchor is None:
        anchor = anchor_for(ext, depth)
    max_level = min(max_level, anchor)
    d = Domain()
    d.depth, d.anchor_level, d.max_level = depth, anchor, max_level
    d.ext[:] = list(ext)
    d.periodic[:] = list(periodic)
    return d


def uniform_mesh(level, ext=(1, 1, 1)):
    n = [e << level for e in ext]
    g = np.stack(np.meshgrid(np.arange(n[0]), np.arange(n[1]), np.arange(n[2]), indexing="ij"), -1).reshape(-1, 3)
    N = len(g)
    return {"x": g[:, 0].astype(np.int32), "y": g[:, 1].astype(np.int32), "z": g[:, 2].astype(np.int32),
            "level": np.full(N, level, np.uint8), "state": np.zeros(N, np.uint8), "flags": np.zeros(N, np.int32),
            "material": np.zeros(N, np.uint32)}


def adapt(cols, cfg_kw, dom, fields=None, C=0):
    """Run the oracle regrid; returns (new columns, stats, new fields, src, kind, members)."""
    L = load()
    cols = {k: np.array(v) for k, v in cols.items()}
    m, keep = mesh_struct(cols)
    n = m.n
    cap = 8 * n + 8
    out = {"x": np.zeros(cap, np.int32), "y": np.zeros(cap, np.int32), "z": np.zeros(cap, np.int32),
           "level": np.zeros(cap, np.uint8), "state": np.zeros(cap, np.uint8), "flags": np.zeros(cap, np.int32),
           "material": np.zeros(cap, np.uint32), "case_id": np.zeros(cap, np.uint16)}
    src = np.zeros(cap, np.uint32)
    kind = np.zeros(cap, np.uint8)
    members = np.zeros(cap, np.uint32)
    of = np.zeros(cap * max(C, 1), np.float32)
    cfg = AdaptCfg(**cfg_kw)
    st = AdaptStats()
    f = np.ascontiguousarray(fields, np.float32) if fields is not None else None
    M = L.or_adapt(ctypes.byref(m), ctypes.byref(dom), ctypes.byref(cfg), ptr(f), C, 0,
                   ptr(out["x"]), ptr(out["y"]), ptr(out["z"]), ptr(out["level"]), ptr(out["state"]),
                   ptr(out["flags"]), ptr(out["material"]), ptr(out["case_id"]) if "case_id" in cols else None,
                   ptr(of) if C else None, ptr(src), ptr(kind), ptr(members), ctypes.byref(st))
    res = {k: v[:M] for k, v in out.items() if k != "case_id" or "case_id" in cols}
    # flags after balance (the oracle updates the input columns in place)
    return res, st, (of[:M * C].reshape(M, C) if C else None), src[:M], kind[:M], members[:st.num_groups * 8], keep


def balance(cols, dom, mode, max_level, iters=10):
    L = load()
    cols = {k: np.array(v) for k, v in cols.items()}
    m, keep = mesh_struct(cols)
    st = BalanceStats()
    L.or_balance(ctypes.byref(m), ctypes.byref(dom), mode, max_level, iters, ctypes.byref(st))
    return keep["flags"].copy(), st


def neighbours(cols, dom, subslots):
    L = load()
    m, keep = mesh_struct(cols)
    nbr = np.zeros(m.n * 26 * subslots, np.uint32)
    L.or_neighbours(ctypes.byref(m), ctypes.byref(dom), subslots, ptr(nbr))
    return nbr


def random_octree(seed, ext=(2, 2, 2), rounds=3, max_level=6, frac=0.3, balanced=True, start_level=2):
    """A random leaf set built by repeated oracle regrids with random refine flags,
    starting from a uniform mesh at start_level."""
    rng = np.random.default_rng(seed)
    cols = uniform_mesh(start_level, ext)
    dom = domain(ext=ext, max_level=max_level)
    for r in range(rounds):
        n = len(cols["x"])
        cols["flags"] = np.where(rng.random(n) < frac, 1, 0).astype(np.int32)
        cols, st, *_ = adapt(cols, dict(max_level=max_level, min_level=0, balance_mode=1 if balanced else 0,
                                        max_balance_iterations=10, enforce_balance=1 if balanced else 0,
                                        averaging_rule=0), dom)
        cols = {k: v.copy() for k, v in cols.items()}
    return cols


# ---- brick pool ------------------------------------------------------------
class OraclePool:
    def __init__(self, cases):
        L = load()
        arr = (LbmCase * len(cases))()
        for i, c in enumerate(cases):
            ctypes.memmove(ctypes.byref(arr[i]), ctypes.byref(c), ctypes.sizeof(LbmCase))
        self.ncases = len(cases)
        self.h = L.or_pool_new(arr, len(cases))

    def n(self):
        return load().or_pool_size(self.h)

    def step(self, k, threads=0):
        import os
        load().or_pool_steps(self.h, k, threads or (os.cpu_count() or 1))

    def regrid(self):
        load().or_pool_regrid(self.h)

    def regrid_flags(self, flags):
        fl = np.ascontiguousarray(flags, np.int32)
        load().or_pool_regrid_flags(self.h, ptr(fl))

    def upload(self, f):
        f = np.ascontiguousarray(f, np.float32)
        load().or_pool_upload(self.h, ptr(f))

    def bricks(self):
        n = self.n()
        x, y, z = (np.empty(n, np.int32) for _ in range(3))
        lv, cs = np.empty(n, np.uint8), np.empty(n, np.uint16)
        load().or_pool_bricks(self.h, ptr(x), ptr(y), ptr(z), ptr(lv), ptr(cs))
        return {"x": x, "y": y, "z": z, "level": lv, "case_id": cs}

    def populations(self):
        n = self.n()
        f = np.empty((19, n, 512), np.float32)
        load().or_pool_populations(self.h, ptr(f))
        return f

    def nbr(self):
        a = np.empty(self.n() * 26 * 4, np.uint32)
        load().or_pool_nbr(self.h, ptr(a))
        return a

    def flags(self):
        n = self.n()
        fl, wm = np.empty(n, np.int32), np.empty(n, np.float32)
        load().or_pool_flags(self.h, ptr(fl), ptr(wm))
        return fl, wm

    def conservation(self):
        out = np.empty((self.ncases, 4), np.float64)
        load().or_pool_conservation(self.h, ptr(out))
        return out

    def lups(self):
        return load().or_pool_fluid_lups(self.h)

    def fp64_steps(self, k, threads=0):
        """Populations after the next k steps run in FP64 from the current state (the pool is unchanged)."""
        import os
        out = np.empty((19, self.n(), 512), np.float64)
        load().or_pool_fp64_steps(self.h, k, threads or (os.cpu_count() or 1), ptr(out))
        return out

    def set_mask(self, case_id, level, words):
        """Solid-mask words (uint32, bit (z*Ny + y)*Nx + x) of one case; None removes them."""
        if words is None:
            load().or_pool_set_mask(self.h, case_id, 0, None, 0)
            return
        self._mask = getattr(self, "_mask", {})
        self._mask[case_id] = w = np.ascontiguousarray(words, np.uint32)
        load().or_pool_set_mask(self.h, case_id, level, ptr(w), w.size)

    def __del__(self):
        try:
            load().or_pool_free(self.h)
        except Exception:
            pass


def gaussian_blobs(seed, n=64, sigma=(0.02, 0.1)):
    """Seeded blob table {cx, cy, cz, 1/(2 sigma^2), amplitude} (the regrid microbenchmark's field)."""
    rng = np.random.default_rng(seed)
    c = rng.random((n, 3))
    s = rng.uniform(sigma[0], sigma[1], n)
    return np.concatenate([c, (1.0 / (2 * s * s))[:, None], np.ones((n, 1))], 1).astype(np.float32)


def blob_flags(cols, blobs, lo, hi, max_level):
    L = load()
    n = len(cols["x"])
    out = np.empty(n, np.int32)
    keep = [np.ascontiguousarray(cols[k]) for k in ("x", "y", "z", "level")]
    b = np.ascontiguousarray(blobs, np.float32)
    L.or_blob_flags(*[ptr(a) for a in keep], n, ptr(b), len(b), lo, hi, max_level, ptr(out))
    return out


# ---------------------------------------------------------------- geometry

def geometry_struct(d):
    """The oracle's or_geometry has the C layout of fl_geometry_desc."""
    return ctypes.byref(d)


def _geo_lib():
    L = load()
    if not getattr(L, "_geo_set", False):
        L.or_geometry_aabb.argtypes = [P, P]
        L.or_geometry_inside.argtypes = [P, P, P, P, ctypes.c_size_t, P]
        L.or_geometry_evaluate.argtypes = [P, P, P, P, ctypes.c_size_t, P]
        L.or_stl_voxelize.restype = ctypes.c_size_t
        L.or_stl_voxelize.argtypes = [P, ctypes.c_size_t, P, ctypes.c_float, P, P, P, ctypes.c_size_t]
        L.or_geometry_candidates.restype = ctypes.c_size_t
        L.or_geometry_candidates.argtypes = [P, ctypes.c_float, P, P, P, P, ctypes.c_size_t]
        L._geo_set = True
    return L


def geometry_aabb(d):
    b = np.zeros(6, np.float32)
    _geo_lib().or_geometry_aabb(ctypes.byref(d), ptr(b))
    return b


def geometry_inside(d, pts):
    pts = np.asarray(pts, np.float32).reshape(-1, 3)
    cols = [np.ascontiguousarray(pts[:, a]) for a in range(3)]
    out = np.zeros(len(pts), np.uint8)
    _geo_lib().or_geometry_inside(ctypes.byref(d), *[ptr(c) for c in cols], len(pts), ptr(out))
    return out.astype(bool)


def geometry_evaluate(d, cells):
    cells = np.asarray(cells, np.int32).reshape(-1, 3)
    cols = [np.ascontiguousarray(cells[:, a]) for a in range(3)]
    out = np.zeros(len(cells), np.uint8)
    _geo_lib().or_geometry_evaluate(ctypes.byref(d), *[ptr(c) for c in cols], len(cells), ptr(out))
    return out.astype(bool)


def _cells_out(fn, cap=1 << 22):
    x, y, z = (np.zeros(cap, np.int32) for _ in range(3))
    n = fn(ptr(x), ptr(y), ptr(z), cap)
    return np.stack([x[:n], y[:n], z[:n]], -1)


def stl_voxelize(tris, d, cell):
    t = np.ascontiguousarray(tris, np.float32).reshape(-1, 9)
    return _cells_out(lambda px, py, pz, cap: _geo_lib().or_stl_voxelize(ptr(t), len(t), ctypes.byref(d), cell,
                                                                          px, py, pz, cap))


def geometry_candidates(d, cell, dom):
    b = np.asarray(dom, np.float32)
    return _cells_out(lambda px, py, pz, cap: _geo_lib().or_geometry_candidates(ctypes.byref(d), cell, ptr(b),
                                                                                px, py, pz, cap))
