"""Python view of the brick-pool part of the C ABI (fl_lbm_case, fl_pool_*)."""
import ctypes

import numpy as np

from .amr import AdaptStats

P = ctypes.c_void_p
Q = 19


class LbmCase(ctypes.Structure):
    _fields_ = [("ext", ctypes.c_int32 * 3), ("bc", ctypes.c_int32 * 6), ("wall_u", ctypes.c_float * 3),
                ("inlet_u", ctypes.c_float * 3), ("tau0", ctypes.c_float), ("max_level", ctypes.c_int32),
                ("has_sphere", ctypes.c_int32), ("sphere_c", ctypes.c_float * 3), ("sphere_r", ctypes.c_float),
                ("refine_frac", ctypes.c_float), ("coarsen_frac", ctypes.c_float), ("band", ctypes.c_float),
                ("init_u", ctypes.c_float * 3)]


def pack_mask(mask):
    """Solid-mask words of a bool grid (Nz, Ny, Nx): bit (z*Ny + y)*Nx + x, 32 to a uint32."""
    b = np.packbits(np.ascontiguousarray(mask, bool).reshape(-1), bitorder="little")
    b = np.concatenate([b, np.zeros((-b.size) % 4, np.uint8)])
    return b.view("<u4").astype(np.uint32)


def unpack_mask(words, shape):
    """The bool grid of pack_mask's words."""
    n = int(np.prod(shape))
    bits = np.unpackbits(np.ascontiguousarray(words, "<u4").view(np.uint8), bitorder="little")[:n]
    return bits.astype(bool).reshape(shape)


class PoolInfo(ctypes.Structure):
    _fields_ = [("num_bricks", ctypes.c_size_t), ("capacity", ctypes.c_size_t), ("num_cases", ctypes.c_int32),
                ("max_level", ctypes.c_int32), ("bricks_per_level", ctypes.c_uint32 * 16),
                ("fluid_lups_per_step", ctypes.c_uint64), ("population_bytes", ctypes.c_uint64),
                ("fluid_sites_per_level", ctypes.c_uint64 * 16), ("num_active_cases", ctypes.c_int32),
                ("usable", ctypes.c_int32), ("general_bricks_per_level", ctypes.c_uint32 * 16),
                ("stencil_descriptors_per_level", ctypes.c_uint64 * 16)]


WALL, MOVING, INLET, OUTLET, PERIODIC = 1, 2, 3, 4, 0


def cavity(edge_sites=32, max_level=2, u_lid=0.05, tau=0.56):
    """Lid-driven cavity: walls, lid moving +x on the top z face."""
    c = LbmCase()
    e = edge_sites // 8
    c.ext[:] = [e, e, e]
    c.bc[:] = [WALL, WALL, WALL, WALL, WALL, MOVING]
    c.wall_u[:] = [u_lid, 0.0, 0.0]
    c.tau0 = tau
    c.max_level = max_level
    c.refine_frac, c.coarsen_frac = 0.5, 0.1
    return c


def sphere_channel(nx=128, ny=64, nz=64, max_level=3, radius=8.0, centre=(32.0, 32.0, 32.0), u_in=0.04,
                   tau=0.56, band=6.0):
    """Flow past a sphere: equilibrium inlet at x=0, zero-gradient outlet, periodic y/z."""
    c = LbmCase()
    c.ext[:] = [nx // 8, ny // 8, nz // 8]
    c.bc[:] = [INLET, OUTLET, PERIODIC, PERIODIC, PERIODIC, PERIODIC]
    c.inlet_u[:] = [u_in, 0.0, 0.0]
    c.init_u[:] = [u_in, 0.0, 0.0]
    c.tau0 = tau
    c.max_level = max_level
    c.has_sphere = 1
    c.sphere_c[:] = list(centre)
    c.sphere_r = radius
    c.band = band
    c.refine_frac, c.coarsen_frac = 0.5, 0.1
    return c


def periodic_box(nx=64, ny=64, nz=8, max_level=0, tau=0.8):
    """A box periodic on all six faces (no walls, no sphere): the Taylor-Green
    vortex case.  Sizes are in level-0 sites (multiples of 8)."""
    c = LbmCase()
    c.ext[:] = [nx // 8, ny // 8, nz // 8]
    c.bc[:] = [PERIODIC] * 6
    c.tau0 = tau
    c.max_level = max_level
    c.refine_frac, c.coarsen_frac = 2.0, -1.0  # no vorticity-driven regrid: refinement by explicit flags only
    return c


# D3Q19 velocities in the kernels' order: rest, +-x, +-y, +-z, then the twelve
# edge directions in opposite pairs; weights 1/3, 1/18, 1/36.
CX = (0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 1, -1, 1, -1, 0, 0, 0, 0)
CY = (0, 0, 0, 1, -1, 0, 0, 1, -1, -1, 1, 0, 0, 0, 0, 1, -1, 1, -1)
CZ = (0, 0, 0, 0, 0, 1, -1, 0, 0, 0, 0, 1, -1, -1, 1, 1, -1, -1, 1)
WQ = (1 / 3,) + (1 / 18,) * 6 + (1 / 36,) * 12


def site_centres(bricks):
    """Centre of every site, (n, 512, 3) in level-0 site units: site s = i + 8 j + 64 k of
    a level-l brick at native (x, y, z) sits at ((8 x + i + 1/2) / 2^l, ...)."""
    s = np.arange(512)
    ijk = np.stack([s & 7, (s >> 3) & 7, s >> 6], -1).astype(np.float64)
    b = np.stack([bricks["x"], bricks["y"], bricks["z"]], -1).astype(np.float64)[:, None, :]
    scale = (0.5 ** bricks["level"].astype(np.float64))[:, None, None]
    return (8.0 * b + ijk[None] + 0.5) * scale


def equilibrium(rho, u):
    """D3Q19 BGK equilibrium populations (19, ...) in FP32 of density rho (...) and
    velocity u (..., 3), evaluated in FP64."""
    rho = np.asarray(rho, np.float64)
    u = np.asarray(u, np.float64)
    usq = (u * u).sum(-1)
    out = np.empty((Q,) + rho.shape, np.float32)
    for q in range(Q):
        cu = CX[q] * u[..., 0] + CY[q] * u[..., 1] + CZ[q] * u[..., 2]
        out[q] = WQ[q] * rho * (1.0 + 3.0 * cu + 4.5 * cu * cu - 1.5 * usq)
    return out


def taylor_green(bricks, nx, ny, u0=0.01):
    """Populations (19, n, 512) of the z-invariant Taylor-Green vortex on an nx x ny periodic
    box: u = u0 sin(kx x) cos(ky y), v = -u0 cos(kx x) sin(ky y), w = 0, with its pressure
    p = rho0 u0^2 / 4 (cos 2 kx x + cos 2 ky y) as density 1 + 3 p (c_s^2 = 1/3)."""
    r = site_centres(bricks)
    kx, ky = 2 * np.pi / nx, 2 * np.pi / ny
    X, Y = kx * r[..., 0], ky * r[..., 1]
    u = np.stack([u0 * np.sin(X) * np.cos(Y), -u0 * np.cos(X) * np.sin(Y), np.zeros_like(X)], -1)
    rho = 1.0 + 3.0 * (u0 * u0 / 4.0) * (np.cos(2 * X) + np.cos(2 * Y))
    return equilibrium(rho, u)


def moments(f):
    """Density (n, 512) and velocity (n, 512, 3) of populations (19, n, 512), in FP64."""
    f = np.asarray(f, np.float64)
    rho = f.sum(0)
    j = np.stack([np.tensordot(np.asarray(c, np.float64), f, 1) for c in (CX, CY, CZ)], -1)
    return rho, j / rho[..., None]


class Pool:
    """A set of independent cases advanced together (fl_pool)."""

    def __init__(self, ctx, cases):
        self.ctx = ctx
        arr = (LbmCase * len(cases))(*cases)
        self.ncases = len(cases)
        self.cases = [LbmCase.from_buffer_copy(c) for c in cases]  # per case id, for snapshots
        h = ctypes.c_void_p()
        ctx.call("fl_pool_create", arr, len(cases), ctypes.byref(h))
        self.h = h

    def step(self, n=1):
        self.ctx.call("fl_pool_step", self.h, n)

    def regrid(self):
        st = AdaptStats()
        self.ctx.call("fl_pool_regrid", self.h, ctypes.byref(st))
        return st

    def info(self):
        i = PoolInfo()
        self.ctx.call("fl_pool_info_get", self.h, ctypes.byref(i))
        return i

    def set_options(self, graphs=1, grid_mult=0, streams=None, staging=None, step_sums=None):
        self.ctx.call("fl_pool_set_options", self.h, graphs, grid_mult)
        if step_sums is not None:
            self.ctx.call("fl_pool_set_step_sums", self.h, int(step_sums))
        if streams is not None:
            self.ctx.call("fl_pool_set_class_streams", self.h, streams)
        if staging is not None:
            self.ctx.call("fl_pool_set_staging", self.h, staging)

    def bricks(self):
        n = self.info().num_bricks
        x, y, z = (np.empty(n, np.int32) for _ in range(3))
        lv, cs = np.empty(n, np.uint8), np.empty(n, np.uint16)
        self.ctx.call("fl_pool_download", self.h, *[a.ctypes.data_as(P) for a in (x, y, z, lv, cs)], None)
        return {"x": x, "y": y, "z": z, "level": lv, "case_id": cs}

    def populations(self):
        n = self.info().num_bricks
        f = np.empty((Q, n, 512), np.float32)
        self.ctx.call("fl_pool_download", self.h, None, None, None, None, None, f.ctypes.data_as(P))
        return f

    def nbr(self):
        n = self.info().num_bricks
        a = np.empty(n * 26 * 4, np.uint32)
        self.ctx.call("fl_pool_nbr", self.h, a.ctypes.data_as(P))
        return a

    def flags(self):
        n = self.info().num_bricks
        fl, wm = np.empty(n, np.int32), np.empty(n, np.float32)
        self.ctx.call("fl_pool_flags", self.h, fl.ctypes.data_as(P), wm.ctypes.data_as(P))
        return fl, wm

    def conservation(self):
        out = np.empty((self.info().num_cases, 4), np.float64)
        self.ctx.call("fl_pool_conservation", self.h, out.ctypes.data_as(P))
        return out

    def profile_steps(self, n):
        """Per kernel (interior, general, all-solid): (kernel ms, launches, fluid sites updated)."""
        ms, la, st = (ctypes.c_double * 3)(), (ctypes.c_uint32 * 3)(), (ctypes.c_uint64 * 3)()
        self.ctx.call("fl_pool_profile_steps", self.h, n, ms, la, st)
        return [(ms[k], la[k], st[k]) for k in range(3)]

    def profile_levels(self, n):
        """Per level and kernel: (kernel ms, launches, fluid sites updated), arrays (16, 3)."""
        ms, la, st = (ctypes.c_double * 48)(), (ctypes.c_uint32 * 48)(), (ctypes.c_uint64 * 48)()
        self.ctx.call("fl_pool_profile_levels", self.h, n, ms, la, st)
        return (np.array(ms[:]).reshape(16, 3), np.array(la[:]).reshape(16, 3), np.array(st[:]).reshape(16, 3))

    def upload(self, f):
        f = np.ascontiguousarray(f, np.float32)
        self.ctx.call("fl_pool_upload", self.h, f.ctypes.data_as(P))

    def set_velocities(self, wall_u=None, inlet_u=None):
        w = None if wall_u is None else np.ascontiguousarray(wall_u, np.float32)
        i = None if inlet_u is None else np.ascontiguousarray(inlet_u, np.float32)
        self.ctx.call("fl_pool_set_velocities", self.h, w.ctypes.data_as(P) if w is not None else None,
                      i.ctypes.data_as(P) if i is not None else None)

    def mask_shape(self, case_id, level):
        """(Nz, Ny, Nx) of a case's solid-mask grid at `level` (N = ext * 8 << level)."""
        c = self.cases[case_id]
        return tuple((int(c.ext[a]) * 8) << level for a in (2, 1, 0))

    def set_solid_mask(self, case_id, level, mask):
        """Solid voxels of one case at `level` (bool (Nz, Ny, Nx)), OR-ed with its sphere; None removes them."""
        if mask is None:
            self.ctx.call("fl_pool_set_solid_mask", self.h, case_id, 0, None, ctypes.c_size_t(0))
            return
        mask = np.asarray(mask, bool)
        if mask.shape != self.mask_shape(case_id, level):
            raise ValueError("mask shape %s, want %s" % (mask.shape, self.mask_shape(case_id, level)))
        w = pack_mask(mask)
        self.ctx.call("fl_pool_set_solid_mask", self.h, case_id, level, w.ctypes.data_as(P), ctypes.c_size_t(w.size))

    def set_solid_cells(self, case_id, level, x, y, z, n):
        """Solid mask from n cells of the level-`level` grid given as device columns (pointers)."""
        cols = [v if isinstance(v, P) else P(v) for v in (x, y, z)]
        self.ctx.call("fl_pool_set_solid_cells", self.h, case_id, level, *cols, ctypes.c_size_t(n))

    def solid_mask(self, case_id):
        """(level, bool (Nz, Ny, Nx)) of the case's solid mask, or (-1, None)."""
        lv = ctypes.c_int32()
        self.ctx.call("fl_pool_get_solid_mask", self.h, case_id, ctypes.byref(lv), None, ctypes.c_size_t(0))
        if lv.value < 0:
            return -1, None
        shape = self.mask_shape(case_id, lv.value)
        w = np.empty((int(np.prod(shape)) + 31) // 32, np.uint32)
        self.ctx.call("fl_pool_get_solid_mask", self.h, case_id, ctypes.byref(lv), w.ctypes.data_as(P),
                      ctypes.c_size_t(w.size))
        return lv.value, unpack_mask(w, shape)

    def add_cases(self, cases):
        arr = (LbmCase * len(cases))(*cases)
        ids = (ctypes.c_int32 * len(cases))()
        self.ctx.call("fl_pool_add_cases", self.h, arr, len(cases), ids)
        self.ncases = self.info().num_cases
        for c, i in zip(cases, ids):
            while len(self.cases) <= i:
                self.cases.append(None)
            self.cases[i] = LbmCase.from_buffer_copy(c)
        return list(ids)

    def remove_cases(self, ids):
        a = (ctypes.c_int32 * len(ids))(*ids)
        self.ctx.call("fl_pool_remove_cases", self.h, a, len(ids))

    def regrid_flags(self, flags):
        """Regrid with one int32 flag per brick (pool order): > 0 split, -1 merge, 0 keep."""
        fl = np.ascontiguousarray(flags, np.int32)
        st = AdaptStats()
        self.ctx.call("fl_pool_regrid_flags", self.h, fl.ctypes.data_as(P), ctypes.byref(st))
        return st

    def regrid_cases(self, due_ids):
        n = self.info().num_cases
        due = np.zeros(n, np.uint8)
        due[list(due_ids)] = 1
        st = AdaptStats()
        self.ctx.call("fl_pool_regrid_cases", self.h, due.ctypes.data_as(P), ctypes.byref(st))
        return st

    def case_state(self, cid, with_f=True):
        nb = ctypes.c_size_t()
        self.ctx.call("fl_pool_download_case", self.h, cid, None, None, None, None, None, ctypes.byref(nb))
        n = nb.value
        x, y, z = (np.empty(n, np.int32) for _ in range(3))
        lv = np.empty(n, np.uint8)
        f = np.empty((Q, n, 512), np.float32) if with_f else None
        self.ctx.call("fl_pool_download_case", self.h, cid, *[a.ctypes.data_as(P) for a in (x, y, z, lv)],
                      f.ctypes.data_as(P) if with_f else None, ctypes.byref(nb))
        return {"x": x, "y": y, "z": z, "level": lv}, f

    def macroscopic(self):
        """Density and velocity of every site, shape (bricks, 512) each (0 inside the sphere)."""
        n = self.info().num_bricks
        out = [np.empty((n, 512), np.float32) for _ in range(4)]
        self.ctx.call("fl_pool_macroscopic", self.h, *[a.ctypes.data_as(P) for a in out])
        return {"density": out[0], "velocity": np.stack(out[1:], -1)}

    def load(self, bricks, f):
        """Replace bricks and populations by a saved state (see snapshot.save)."""
        cols = [np.ascontiguousarray(bricks[k], t) for k, t in
                (("x", np.int32), ("y", np.int32), ("z", np.int32), ("level", np.uint8), ("case_id", np.uint16))]
        f = np.ascontiguousarray(f, np.float32)
        self.ctx.call("fl_pool_load", self.h, ctypes.c_size_t(len(cols[0])), *[a.ctypes.data_as(P) for a in cols],
                      f.ctypes.data_as(P))

    def close(self):
        if self.h:
            self.ctx.call("fl_pool_destroy", self.h)
            self.h = None

    def __del__(self):
        try:
            if self.h and self.ctx.handle:
                self.ctx.lib.fl_pool_destroy(self.ctx.handle, self.h)
        except Exception:
            pass
