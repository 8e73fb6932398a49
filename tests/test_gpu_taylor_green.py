"""The Taylor-Green vortex on the GPU (the physics check of the collide-stream;
the analytic solution and the case set-up are in test_oracle_taylor_green.py):
the GPU pool equals the oracle bit for bit on the periodic box, on one level and
with a refined central patch, and meets the same decay-rate, shape and mass
bounds on its own."""
import numpy as np
import pytest

from fluidloom_gb300.lbm import Pool
from tests import _oracle as O
from tests.test_oracle_taylor_green import CASES, mode_amplitude, taylor_green_pool

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("case", sorted(CASES))
def test_taylor_green_gpu_equals_oracle(ctx, case):
    patch = CASES[case][0]
    gp = taylor_green_pool(lambda cs: Pool(ctx, cs), 64, patch)
    op = taylor_green_pool(O.OraclePool, 64, patch)
    for k in ("x", "y", "z", "level"):
        np.testing.assert_array_equal(gp.bricks()[k], op.bricks()[k])
    gp.step(10)
    op.step(10)
    g, o = gp.populations(), op.populations()
    # FP32 populations within 1e-5 relative of the FP32 oracle (observed: equal)
    np.testing.assert_allclose(g, o, rtol=1e-5, atol=0)
    assert np.array_equal(g, o)
    np.testing.assert_allclose(gp.conservation(), op.conservation(), rtol=1e-12, atol=1e-12)
    gp.close()


@pytest.mark.parametrize("case", sorted(CASES))
def test_taylor_green_decay_on_the_gpu(ctx, case):
    patch, rate_tol, resid_tol = CASES[case]
    nx, tau, steps = 64, 0.8, 400
    gp = taylor_green_pool(lambda cs: Pool(ctx, cs), nx, patch, tau)
    a0, _ = mode_amplitude(gp.bricks(), gp.populations(), nx, nx)
    m0 = gp.conservation()[0]
    gp.step(steps)
    a1, resid = mode_amplitude(gp.bricks(), gp.populations(), nx, nx)
    m1 = gp.conservation()[0]
    exact = (tau - 0.5) / 3.0 * 2 * (2 * np.pi / nx) ** 2
    rate = -np.log(a1 / a0) / steps
    assert abs(rate / exact - 1) < rate_tol, (rate, exact)
    assert resid < resid_tol
    assert abs(m1[0] - m0[0]) / m0[0] < steps * 2.0 ** -23
    gp.close()
