"""An independent physics check of the collide-stream: the Taylor-Green vortex.

The reference holds the analytic solution in
tests/validation/analytical/TaylorGreenSolution.h:25-47.  tests/golden/
taylor_green_ref.npz records what that header computes (compiled in place by
oracle/Makefile.ref; tests/golden/make_taylor_green.py), and `analytic` below
is checked against it.  On the plane z = 0 its field is the 2-D vortex
u = sin x cos y, v = -cos x sin y, an exact Navier-Stokes solution that decays
as exp(-2 nu t) (wavenumbers 1 on [0, 2 pi]).  The header's 3-D field
(a cos z factor on u and v) is not a Navier-Stokes solution; in the Stokes
limit it decays as exp(-3 nu t), not the header's exp(-2 nu t):
test_three_d_field_decays_faster_than_the_header_states shows it.

On the lattice: a box of N x N x 8 sites, periodic on every face, started at
the vortex's equilibrium (with its pressure), nu = (tau - 1/2) / 3; the mode's
amplitude must decay at nu (kx^2 + ky^2) per level-0 step and the field keep
its shape, on one level and with a refined central patch (coarse/fine coupling
and the tau rescaling of each level), and the FP64 mass sum must stay constant
to FP32 round-off.  Here the oracle runs it; the GPU tests run the same cases
and equal the oracle bit for bit."""
import os

import numpy as np
import pytest

from fluidloom_gb300 import lbm
from tests import _oracle as O

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "taylor_green_ref.npz")


def analytic(x, y, z, t, re):
    """TaylorGreenSolution::computeVelocity and ::computeKineticEnergy
    (TaylorGreenSolution.h:25-47): nu = 1/Re, velocity decay exp(-2 nu t),
    energy decay exp(-4 nu t)."""
    nu = 1.0 / re
    d = np.exp(-2.0 * nu * t)
    u = np.sin(x) * np.cos(y) * np.cos(z) * d
    v = -np.cos(x) * np.sin(y) * np.cos(z) * d
    return np.stack([u, v, np.zeros_like(u)], -1), np.exp(-4.0 * nu * t)


def test_analytic_restatement_matches_reference_header():
    g = np.load(GOLDEN)
    uvw, e = analytic(g["xyz"][:, 0], g["xyz"][:, 1], g["xyz"][:, 2], g["t"], g["re"])
    np.testing.assert_allclose(uvw, g["uvw"], rtol=0, atol=1e-15)
    np.testing.assert_allclose(e, g["energy"], rtol=1e-15)


def mode_amplitude(bricks, f, nx, ny):
    """Projection of the velocity on the vortex's shape (volume weighted) and the
    relative L2 residual of what the projection leaves."""
    rho, u = lbm.moments(f)
    r = lbm.site_centres(bricks)
    X, Y = 2 * np.pi / nx * r[..., 0], 2 * np.pi / ny * r[..., 1]
    # the analytic solution of the header on the plane z = 0, at t = 0 (shape only)
    shape, _ = analytic(X, Y, np.zeros_like(X), 0.0, 1.0)
    vol = (0.125 ** bricks["level"].astype(np.float64))[:, None]
    a = ((u * shape).sum(-1) * vol).sum() / ((shape * shape).sum(-1) * vol).sum()
    resid = np.sqrt((((u - a * shape) ** 2).sum(-1) * vol).sum() / ((a * a * (shape * shape).sum(-1)) * vol).sum())
    return a, resid


def patch_flags(bricks, nx):
    """Refine the central half of the box in x and y (all of z)."""
    e = nx // 8
    return ((bricks["x"] >= e // 4) & (bricks["x"] < 3 * e // 4) & (bricks["y"] >= e // 4) &
            (bricks["y"] < 3 * e // 4)).astype(np.int32)


def taylor_green_pool(make, nx, patch, tau=0.8, u0=0.01):
    """A pool (oracle or GPU, from make(cases)) holding the vortex, refined in the
    centre when patch is set."""
    pool = make([lbm.periodic_box(nx, nx, 8, max_level=1 if patch else 0, tau=tau)])
    if patch:
        pool.regrid_flags(patch_flags(pool.bricks(), nx))
    pool.upload(lbm.taylor_green(pool.bricks(), nx, nx, u0))
    return pool


# decay-rate tolerance (relative) and residual bound per case, from the
# lattice's discretisation error at 64 sites per wavelength
CASES = {"one_level": (False, 0.01, 1e-3), "refined_patch": (True, 0.025, 0.05)}


@pytest.mark.parametrize("case", sorted(CASES))
def test_taylor_green_decay_on_the_oracle(case):
    patch, rate_tol, resid_tol = CASES[case]
    nx, tau, steps = 64, 0.8, 200
    pool = taylor_green_pool(O.OraclePool, nx, patch, tau)
    b = pool.bricks()
    assert (np.bincount(b["level"]) > 0).sum() == (2 if patch else 1)
    a0, _ = mode_amplitude(b, pool.populations(), nx, nx)
    m0 = pool.conservation()[0]
    pool.step(steps)
    a1, resid = mode_amplitude(pool.bricks(), pool.populations(), nx, nx)
    m1 = pool.conservation()[0]
    nu = (tau - 0.5) / 3.0
    exact = nu * 2 * (2 * np.pi / nx) ** 2
    rate = -np.log(a1 / a0) / steps
    assert abs(rate / exact - 1) < rate_tol, (rate, exact)
    assert resid < resid_tol
    # mass: the FP64 sum of the FP32 populations drifts by FP32 round-off only
    assert abs(m1[0] - m0[0]) / m0[0] < steps * 2.0 ** -23


def test_three_d_field_decays_faster_than_the_header_states():
    """The header's 3-D field u = sin x cos y cos z, v = -cos x sin y cos z
    carries |k|^2 = 3: at small amplitude (Stokes flow) it decays as
    exp(-3 nu t), while TaylorGreenSolution.h:30 states exp(-2 nu t)."""
    n, tau, u0, steps = 32, 0.8, 1e-4, 100
    pool = O.OraclePool([lbm.periodic_box(n, n, n, 0, tau)])
    b = pool.bricks()
    r = lbm.site_centres(b) * (2 * np.pi / n)
    uvw, _ = analytic(r[..., 0], r[..., 1], r[..., 2], 0.0, 1.0)
    pool.upload(lbm.equilibrium(np.ones(r.shape[:-1]), u0 * uvw))
    pool.step(steps)
    _, u = lbm.moments(pool.populations())
    a = (u * uvw).sum() / (uvw * uvw).sum() / u0
    nu_k2 = (tau - 0.5) / 3.0 * (2 * np.pi / n) ** 2
    rate = -np.log(a) / steps / nu_k2
    assert abs(rate - 3.0) < 0.05 and abs(rate - 2.0) > 0.9
