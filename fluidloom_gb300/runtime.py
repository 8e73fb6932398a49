"""Context and device-buffer helpers over the C ABI (no torch dependency)."""
import ctypes

import numpy as np

from . import _capi


class FluidLoomError(RuntimeError):
    """Raised for a non-zero status (mirrors fluidloom::FluidLoomError)."""

    def __init__(self, status, message):
        super().__init__("[FluidLoomError] %s (status %d)" % (message, status))
        self.status = status


def check(ctx, status, what=""):
    if status != 0:
        L = _capi.lib()
        msg = L.fl_last_error(ctx.handle if ctx is not None else None)
        msg = msg.decode() if msg else L.fl_status_string(status).decode()
        raise FluidLoomError(status, "%s: %s" % (what, msg))
    return status


class Context:
    """Owns an fl_ctx (CUDA stream, scratch, status words) on one device."""

    def __init__(self, device=0):
        L = _capi.lib()
        h = ctypes.c_void_p()
        st = L.fl_ctx_create(device, ctypes.byref(h))
        if st != 0:
            raise FluidLoomError(st, L.fl_status_string(st).decode())
        self.handle = h
        self.lib = L

    def call(self, name, *args):
        st = getattr(self.lib, name)(self.handle, *args)
        check(self, st, name)
        return st

    def sync(self):
        self.call("fl_ctx_synchronize")

    def launch_count(self):
        """Kernels launched on behalf of this context so far (graph replays count their nodes)."""
        c = ctypes.c_uint64()
        self.call("fl_ctx_launch_count", ctypes.byref(c))
        return c.value

    def set_stream(self, stream_ptr):
        self.call("fl_ctx_set_stream", ctypes.c_void_p(stream_ptr))

    def close(self):
        if self.handle:
            self.lib.fl_ctx_destroy(self.handle)
            self.handle = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class DeviceArray:
    """A typed device buffer allocated through fl_device_alloc."""

    def __init__(self, ctx, shape, dtype):
        self.ctx = ctx
        self.shape = tuple(np.atleast_1d(shape)) if not isinstance(shape, tuple) else shape
        self.dtype = np.dtype(dtype)
        self.nbytes = int(np.prod(self.shape)) * self.dtype.itemsize
        p = ctypes.c_void_p()
        ctx.call("fl_device_alloc", ctypes.c_size_t(self.nbytes), ctypes.byref(p))
        self.ptr = p

    @classmethod
    def from_host(cls, ctx, a):
        a = np.ascontiguousarray(a)
        d = cls(ctx, a.shape, a.dtype)
        if a.nbytes:
            ctx.call("fl_memcpy_h2d", d.ptr, a.ctypes.data_as(ctypes.c_void_p), ctypes.c_size_t(a.nbytes))
        return d

    def to_host(self):
        out = np.empty(self.shape, self.dtype)
        if self.nbytes:
            self.ctx.call("fl_memcpy_d2h", out.ctypes.data_as(ctypes.c_void_p), self.ptr,
                          ctypes.c_size_t(self.nbytes))
        return out

    def zero(self):
        if self.nbytes:
            self.ctx.call("fl_memset_d", self.ptr, 0, ctypes.c_size_t(self.nbytes))
        return self

    def free(self):
        if self.ptr:
            self.ctx.call("fl_device_free", self.ptr)
            self.ptr = None

    def __del__(self):
        try:
            if self.ptr and self.ctx.handle:
                self.ctx.lib.fl_device_free(self.ctx.handle, self.ptr)
        except Exception:
            pass
