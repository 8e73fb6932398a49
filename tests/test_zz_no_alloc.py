"""The allocation-free scan, called through the C ABI.

It exists for callers that cannot allocate device memory (a thread capturing
a CUDA graph, FFI hosts that own every device allocation).  The test compares
it with the ordinary scan entry point on two calls in a row: the second call
must not see the first call's leftovers in the shared scratch array.  The file
is named so that pytest collects it last.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _scan_both(ctx, a):
    from fluidloom_gb300 import DeviceArray
    n = len(a)
    d_in = DeviceArray.from_host(ctx, a)
    d_ref, d_new = DeviceArray(ctx, (max(n, 1),), np.uint32), DeviceArray(ctx, (max(n, 1),), np.uint32)
    t_ref, t_new = DeviceArray(ctx, (1,), np.uint32), DeviceArray(ctx, (1,), np.uint32)
    ctx.call("fl_scan_exclusive_u32", d_in.ptr, d_ref.ptr, n, t_ref.ptr)
    ctx.sync()
    st = ctx.lib.fl_scan_exclusive_u32_noalloc(d_in.ptr, d_new.ptr, n, t_new.ptr, ctx.lib.fl_ctx_stream(ctx.handle))
    assert st == 0, st
    return d_ref.to_host()[:n], d_new.to_host()[:n], int(t_ref.to_host()[0]), int(t_new.to_host()[0])


def test_noalloc_scan_matches_scan_twice(ctx):
    rng = np.random.default_rng(2024)
    first = rng.integers(0, 1 << 20, 5_000_003).astype(np.uint32)   # many tiles
    second = rng.integers(0, 9, 70_001).astype(np.uint32)           # fewer tiles, stale words beyond
    for a in (first, second):
        ref, new, tr, tn = _scan_both(ctx, a)
        np.testing.assert_array_equal(new, ref)  # integer scan: exact
        assert tn == tr


def test_noalloc_scan_rejects_oversize(ctx):
    # 2^26 + 1 elements exceed the fixed scratch; rejected before any device access
    st = ctx.lib.fl_scan_exclusive_u32_noalloc(None, None, (1 << 26) + 1, None, None)
    assert st == -3  # FL_E_CAPACITY
