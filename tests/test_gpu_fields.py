"""The pool's populations through the field API (fl_pool_populations_field): a
19-component field of the context's structure-of-arrays manager, as the
reference allocates populations (SOAFieldManager.cpp:17-131) and binds them to
kernel nodes (KernelNode.cpp:27-29).  Its component pointers read the pool's
current populations, writes through them reach the pool, and the pool keeps
stepping exactly as the oracle after the view was taken (the parity copy that
gathers level 0 into one buffer changes nothing)."""
import ctypes

import numpy as np
import pytest

from fluidloom_gb300.lbm import Pool, cavity
from tests import _oracle as O

pytestmark = pytest.mark.gpu


def _component(ctx, h, q, n):
    p = ctypes.c_void_p()
    ctx.call("fl_soa_device_ptr", ctypes.c_uint64(h), q, ctypes.byref(p))
    out = np.empty(n * 512, np.float32)
    ctx.call("fl_memcpy_d2h", out.ctypes.data_as(ctypes.c_void_p), p, ctypes.c_size_t(out.nbytes))
    return out.reshape(n, 512), p


@pytest.mark.parametrize("steps", [2, 3])
def test_populations_field_view(ctx, steps):
    case = cavity(16, 1, u_lid=0.05)
    gp, op = Pool(ctx, [case]), O.OraclePool([case])
    gp.step(steps)
    op.step(steps)
    h = ctypes.c_uint64()
    ctx.call("fl_pool_populations_field", gp.h, b"populations", ctypes.byref(h))
    n = gp.info().num_bricks
    cells, pitch, ver = ctypes.c_size_t(), ctypes.c_size_t(), ctypes.c_uint64()
    ctx.call("fl_soa_info", h, ctypes.byref(cells), ctypes.byref(pitch), ctypes.byref(ver))
    assert cells.value == n * 512 and pitch.value == gp.info().capacity * 512 * 4
    f = gp.populations()
    for q in range(19):
        comp, _ = _component(ctx, h.value, q, n)
        np.testing.assert_array_equal(comp, f[q])
    np.testing.assert_array_equal(f, op.populations())
    # the pool steps on as before the view
    gp.step(2)
    op.step(2)
    np.testing.assert_array_equal(gp.populations(), op.populations())
    # a write through the field reaches the pool
    ctx.call("fl_pool_populations_field", gp.h, b"populations", ctypes.byref(h))
    _, p5 = _component(ctx, h.value, 5, n)
    v = np.array([0.125], np.float32)
    ctx.call("fl_memcpy_h2d", p5, v.ctypes.data_as(ctypes.c_void_p), ctypes.c_size_t(4))
    assert gp.populations()[5, 0, 0] == np.float32(0.125)
    gp.close()
