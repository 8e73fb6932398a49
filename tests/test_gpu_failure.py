"""Failure detection without a GPU fault: a bounded device wait that nothing
releases runs out, the call reports FL_E_DEVICE_TIMEOUT, and the context keeps
working; host-side bad inputs are rejected before any launch."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_lookback_wait_runs_out_and_context_survives(ctx):
    st = ctx.lib.fl_lookback_timeout_probe(ctx.handle, 2000)
    assert st == -6  # FL_E_DEVICE_TIMEOUT
    from fluidloom_gb300 import DeviceArray
    a = np.arange(100000, dtype=np.uint32)
    d, o = DeviceArray.from_host(ctx, a), DeviceArray(ctx, (100000,), np.uint32)
    ctx.call("fl_scan_exclusive_u32", d.ptr, o.ptr, 100000, None)
    np.testing.assert_array_equal(o.to_host(), np.concatenate([[0], np.cumsum(a[:-1])]).astype(np.uint32))


def test_invalid_inputs_rejected(ctx):
    L = ctx.lib
    assert L.fl_sort_pairs_u64_u32(ctx.handle, None, None, 10, 0, 64) == -1
    assert L.fl_sort_pairs_u64_u32(ctx.handle, None, None, 10, 8, 4) == -1
    assert L.fl_lookback_timeout_probe(ctx.handle, 0) == -1
