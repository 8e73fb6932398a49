"""Execution graph over the C ABI (fl_graph_*): nodes with read/write field sets
and AMR levels, hazard analysis, topological order, and the scheduler that runs
them on CUDA streams (optionally replaying captured CUDA graphs).

Mirrors the reference runtime (include/fluidloom/runtime/nodes/ExecutionNode.h,
src/runtime/dependency/HazardAnalyzer.cpp, DependencyGraphBuilder.cpp,
src/runtime/scheduler/TopologicalScheduler.cpp).
"""
import ctypes

from . import _capi
from .runtime import FluidLoomError

KERNEL, HALO_EXCHANGE, BARRIER, ADAPT_MESH, LBM_STEP, HOST = range(6)
RAW, WAW, WAR, LEVEL_BARRIER = range(4)
HAZARD_NAMES = {RAW: "RAW", WAW: "WAW", WAR: "WAR", LEVEL_BARRIER: "LEVEL_BARRIER"}

NODE_FN = ctypes.CFUNCTYPE(ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p)
HOST_FN = ctypes.CFUNCTYPE(None, ctypes.c_void_p)


class NodeDesc(ctypes.Structure):
    _fields_ = [("type", ctypes.c_int32), ("name", ctypes.c_char * 64), ("level", ctypes.c_int32),
                ("halo_depth", ctypes.c_int32), ("reads", ctypes.c_char_p), ("writes", ctypes.c_char_p),
                ("fn", NODE_FN), ("host_fn", HOST_FN), ("user", ctypes.c_void_p), ("pool", ctypes.c_void_p),
                ("nsteps", ctypes.c_int32)]


class Hazard(ctypes.Structure):
    _fields_ = [("src", ctypes.c_uint64), ("dst", ctypes.c_uint64), ("type", ctypes.c_int32),
                ("field", ctypes.c_char * 68)]


class Graph:
    """A dependency graph of execution nodes; `ctx` may be None for analysis only."""

    def __init__(self, ctx=None):
        self.ctx = ctx
        self.lib = _capi.lib()
        h = ctypes.c_void_p()
        self._check(self.lib.fl_graph_create(ctx.handle if ctx is not None else None, ctypes.byref(h)),
                    "fl_graph_create")
        self.h = h
        self._keep = []  # callbacks must outlive the graph

    def _check(self, st, what):
        if st != 0:
            msg = self.lib.fl_graph_last_error(self.h) if getattr(self, "h", None) else None
            msg = msg.decode() if msg else self.lib.fl_status_string(st).decode()
            raise FluidLoomError(st, "%s: %s" % (what, msg))
        return st

    def add(self, kind, name, reads=(), writes=(), level=-1, halo_depth=0, fn=None, host_fn=None, pool=None,
            nsteps=1):
        """Add a node; returns its id.  fn(stream) for KERNEL nodes enqueues work on the
        stream (the context's stream points at it meanwhile); host_fn() for HOST nodes."""
        d = NodeDesc()
        d.type = kind
        d.name = name.encode()[:63]
        d.level = level
        d.halo_depth = halo_depth
        d.reads = ",".join(reads).encode() if reads else None
        d.writes = ",".join(writes).encode() if writes else None
        if fn is not None:
            cb = NODE_FN(lambda ctx, stream, user: int(fn(stream) or 0))
            self._keep.append(cb)
            d.fn = cb
        if host_fn is not None:
            hb = HOST_FN(lambda user: host_fn())
            self._keep.append(hb)
            d.host_fn = hb
        d.pool = pool.h if pool is not None else None
        d.nsteps = nsteps
        nid = ctypes.c_int64()
        self._check(self.lib.fl_graph_add_node(self.h, ctypes.byref(d), ctypes.byref(nid)), "fl_graph_add_node")
        return nid.value

    def add_edge(self, a, b):
        self._check(self.lib.fl_graph_add_edge(self.h, a, b), "fl_graph_add_edge")

    def analyze(self):
        """HazardAnalyzer::analyzeNodes + enforceHazards; returns [(from, to, type, field)]."""
        n = ctypes.c_size_t()
        self._check(self.lib.fl_graph_analyze(self.h, None, 0, ctypes.byref(n)), "fl_graph_analyze")
        out = (Hazard * max(n.value, 1))()
        self._check(self.lib.fl_graph_hazards(self.h, out, n.value, ctypes.byref(n)), "fl_graph_hazards")
        return [(int(h.src), int(h.dst), int(h.type), h.field.decode()) for h in out[:n.value]]

    def build(self):
        self._check(self.lib.fl_graph_build(self.h), "fl_graph_build")

    def order(self):
        n = ctypes.c_size_t()
        self._check(self.lib.fl_graph_order(self.h, None, 0, ctypes.byref(n)), "fl_graph_order")
        ids = (ctypes.c_int64 * max(n.value, 1))()
        self._check(self.lib.fl_graph_order(self.h, ids, n.value, ctypes.byref(n)), "fl_graph_order")
        return list(ids[:n.value])

    def num_edges(self):
        n = ctypes.c_size_t()
        self._check(self.lib.fl_graph_num_edges(self.h, ctypes.byref(n)), "fl_graph_num_edges")
        return n.value

    def execute(self, cuda_graphs=True):
        self._check(self.lib.fl_graph_execute(self.h, 1 if cuda_graphs else 0), "fl_graph_execute")

    def set_profiling(self, on=True):
        self._check(self.lib.fl_graph_set_profiling(self.h, 1 if on else 0), "fl_graph_set_profiling")

    def stats(self, nid):
        c, t = ctypes.c_uint64(), ctypes.c_double()
        self._check(self.lib.fl_graph_node_stats(self.h, nid, ctypes.byref(c), ctypes.byref(t)), "fl_graph_node_stats")
        return c.value, t.value

    def dot(self):
        n = ctypes.c_size_t()
        self._check(self.lib.fl_graph_dot(self.h, None, 0, ctypes.byref(n)), "fl_graph_dot")
        buf = ctypes.create_string_buffer(n.value + 1)
        self._check(self.lib.fl_graph_dot(self.h, buf, n.value + 1, ctypes.byref(n)), "fl_graph_dot")
        return buf.value.decode()

    def close(self):
        if getattr(self, "h", None):
            self.lib.fl_graph_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
