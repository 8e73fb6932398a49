"""The allocation-free scan, called through the C ABI.

It exists for callers that cannot allocate device memory: embedders that own
every device allocation through their own pool, hosts under a fixed memory
budget, FFI hosts that must not allocate on their hot path.  The tests compare
it with the ordinary scan entry point on two calls in a row (the second call
must not see the first call's leftovers in the shared scratch array), at the
largest size the fixed scratch holds, and with no elements.  The file is named
so that pytest collects it last.
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


def test_noalloc_scan_at_the_size_limit(ctx):
    """n == 2^26: the last tile's status word is the last one of the fixed array."""
    from fluidloom_gb300 import DeviceArray
    n = 1 << 26
    a = (np.arange(n, dtype=np.uint64) * 2654435761 % 4).astype(np.uint32)
    d_in = DeviceArray.from_host(ctx, a)
    d_out = DeviceArray(ctx, (n,), np.uint32)
    d_tot = DeviceArray(ctx, (1,), np.uint32)
    st = ctx.lib.fl_scan_exclusive_u32_noalloc(d_in.ptr, d_out.ptr, n, d_tot.ptr, ctx.lib.fl_ctx_stream(ctx.handle))
    assert st == 0, st
    ref = np.zeros(n, np.uint32)
    np.cumsum(a[:-1], dtype=np.uint32, out=ref[1:])
    np.testing.assert_array_equal(d_out.to_host(), ref)
    assert int(d_tot.to_host()[0]) == int((int(ref[-1]) + int(a[-1])) & 0xFFFFFFFF)


def test_noalloc_scan_empty_sets_total(ctx):
    """n == 0 touches nothing but the total, which becomes 0."""
    from fluidloom_gb300 import DeviceArray
    d_tot = DeviceArray.from_host(ctx, np.array([0xDEADBEEF], np.uint32))
    st = ctx.lib.fl_scan_exclusive_u32_noalloc(None, None, 0, d_tot.ptr, ctx.lib.fl_ctx_stream(ctx.handle))
    assert st == 0, st
    ctx.sync()
    assert int(d_tot.to_host()[0]) == 0
