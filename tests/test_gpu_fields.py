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


def test_step_sums_stop_after_field_export(ctx):
    """With step sums on, a conservation read after a step uses the step's own sums.  Once
    the populations are exported as a writable field the pool cannot see writes through it,
    so it recomputes the sums from the stored state: a write through the field shows up in
    the next conservation read, which equals that of a pool uploaded with the same state."""
    from fluidloom_gb300.lbm import Pool
    from tests.test_gpu_lbm import cases_small
    gp = Pool(ctx, [cases_small()[1]])
    gp.set_options(step_sums=True)
    gp.step(3)
    before = gp.conservation()
    h = ctypes.c_uint64()
    ctx.call("fl_pool_populations_field", gp.h, b"populations", ctypes.byref(h))
    n = gp.info().num_bricks
    _, p0 = _component(ctx, h.value, 0, n)
    f0 = np.empty(1, np.float32)
    ctx.call("fl_memcpy_d2h", f0.ctypes.data_as(ctypes.c_void_p), p0, ctypes.c_size_t(4))
    v = np.array([f0[0] + 0.5], np.float32)  # add mass at the first site of the first brick
    ctx.call("fl_memcpy_h2d", p0, v.ctypes.data_as(ctypes.c_void_p), ctypes.c_size_t(4))
    after = gp.conservation()
    assert after[0, 0] != before[0, 0]
    ref = Pool(ctx, [cases_small()[1]])
    ref.upload(gp.populations())
    np.testing.assert_array_equal(after, ref.conservation())
    gp.step(1)
    ref.step(1)
    np.testing.assert_array_equal(gp.conservation(), ref.conservation())
    ref.close()
    gp.close()

