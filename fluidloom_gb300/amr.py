"""Python mirror of the AMR part of the C ABI: fl_mesh, fl_adapt_config and
friends as ctypes structures, and a host-side helper that moves a leaf set in
and out of device columns.  Field names follow the reference's
AdaptationConfig / BalanceResult (include/fluidloom/adaptation/AdaptationTypes.h)."""
import ctypes

import numpy as np

from .runtime import DeviceArray

P = ctypes.c_void_p


class FlMesh(ctypes.Structure):
    _fields_ = [("x", P), ("y", P), ("z", P), ("level", P), ("state", P), ("flags", P), ("material", P),
                ("case_id", P), ("num_cells", ctypes.c_size_t), ("capacity", ctypes.c_size_t)]


class AdaptConfig(ctypes.Structure):
    _fields_ = [("max_refinement_level", ctypes.c_uint8), ("min_refinement_level", ctypes.c_uint8),
                ("max_balance_iterations", ctypes.c_uint32), ("enforce_2_1_balance", ctypes.c_int32),
                ("balance_mode", ctypes.c_int32), ("averaging_rule", ctypes.c_int32),
                ("buffer_growth_factor", ctypes.c_double), ("key_depth", ctypes.c_int32),
                ("anchor_level", ctypes.c_int32), ("ext", ctypes.c_int32 * 3), ("periodic", ctypes.c_int32 * 3),
                ("input_balanced", ctypes.c_int32)]

    @classmethod
    def make(cls, max_level=8, min_level=0, balance_mode=0, enforce=True, iters=10, rule=0, depth=21, anchor=None,
             ext=(1, 1, 1), periodic=(0, 0, 0), growth=1.5, input_balanced=False):
        if anchor is None:  # deepest anchor level with ext << anchor inside the depth-bit key space
            e = max(ext)
            anchor = depth - (int(e - 1).bit_length() if e > 1 else 0)
        c = cls()
        c.max_refinement_level = max_level
        c.min_refinement_level = min_level
        c.max_balance_iterations = iters
        c.enforce_2_1_balance = int(enforce)
        c.balance_mode = balance_mode
        c.averaging_rule = rule
        c.buffer_growth_factor = growth
        c.key_depth = depth
        c.anchor_level = anchor
        c.ext[:] = list(ext)
        c.periodic[:] = list(periodic)
        c.input_balanced = int(input_balanced)
        return c


class BalanceResult(ctypes.Structure):
    _fields_ = [("converged", ctypes.c_int32), ("iterations", ctypes.c_uint32),
                ("total_violations_detected", ctypes.c_uint32), ("total_cells_marked_for_balance", ctypes.c_uint32)]


class AdaptStats(ctypes.Structure):
    _fields_ = [("num_split", ctypes.c_uint32), ("num_children", ctypes.c_uint32), ("num_groups", ctypes.c_uint32),
                ("num_merged", ctypes.c_uint32), ("num_survivors", ctypes.c_uint32),
                ("num_cells_out", ctypes.c_size_t), ("balance", BalanceResult)]


COLS = [("x", np.int32), ("y", np.int32), ("z", np.int32), ("level", np.uint8), ("state", np.uint8),
        ("flags", np.int32), ("material", np.uint32)]


class Mesh:
    """A device leaf set allocated with fl_mesh_alloc."""

    def __init__(self, ctx, cols, with_case=False, capacity=None):
        self.ctx = ctx
        n = len(cols["x"])
        self.m = FlMesh()
        cap = max(capacity or n, 1)
        ctx.call("fl_mesh_alloc", ctypes.c_size_t(cap), int(with_case or "case_id" in cols), ctypes.byref(self.m))
        self.upload(cols)

    def upload(self, cols):
        n = len(cols["x"])
        assert n <= self.m.capacity
        for name, dt in COLS + [("case_id", np.uint16)]:
            if name == "case_id" and not self.m.case_id:
                continue
            a = np.ascontiguousarray(cols.get(name, np.zeros(n, dt)), dt)
            if n:
                self.ctx.call("fl_memcpy_h2d", getattr(self.m, name), a.ctypes.data_as(P), ctypes.c_size_t(a.nbytes))
        self.m.num_cells = n

    def download(self):
        n = self.m.num_cells
        out = {}
        for name, dt in COLS + [("case_id", np.uint16)]:
            if name == "case_id" and not self.m.case_id:
                continue
            a = np.empty(n, dt)
            if n:
                self.ctx.call("fl_memcpy_d2h", a.ctypes.data_as(P), getattr(self.m, name), ctypes.c_size_t(a.nbytes))
            out[name] = a
        return out

    @property
    def n(self):
        return self.m.num_cells

    def free(self):
        if self.m.x:
            self.ctx.call("fl_mesh_free", ctypes.byref(self.m))

    def __del__(self):
        try:
            if self.m.x and self.ctx.handle:
                self.ctx.lib.fl_mesh_free(self.ctx.handle, ctypes.byref(self.m))
        except Exception:
            pass


__all__ = ["FlMesh", "AdaptConfig", "BalanceResult", "AdaptStats", "Mesh", "DeviceArray"]
