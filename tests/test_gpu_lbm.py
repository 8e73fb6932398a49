"""GPU brick pool (D3Q19 collide-stream, regrid, flags, conservation) vs the
CPU oracle.  Tolerance for FP32 populations: 1e-5 relative (the kernels are
built without FMA contraction, so the expected difference is zero)."""
import numpy as np
import pytest

from tests import _oracle as O

pytestmark = pytest.mark.gpu
RTOL = 1e-5


def cases_small():
    from fluidloom_gb300 import lbm
    cav = lbm.cavity(16, 1)
    sph = lbm.sphere_channel(64, 32, 32, 2, radius=4.0, centre=(16.0, 16.0, 16.0), u_in=0.04, band=3.0)
    return cav, sph


def assert_pool_equal(gp, op, check_f=True):
    gb, ob = gp.bricks(), op.bricks()
    for k in ("x", "y", "z", "level", "case_id"):
        np.testing.assert_array_equal(gb[k], ob[k], err_msg=k)
    np.testing.assert_array_equal(gp.nbr(), op.nbr())
    if check_f:
        gf, of = gp.populations(), op.populations()
        np.testing.assert_allclose(gf, of, rtol=RTOL, atol=0)
        return float(np.abs(gf - of).max())
    return 0.0


@pytest.mark.parametrize("staging", [0, 2])
@pytest.mark.parametrize("which", [0, 1])
def test_pool_steps_and_regrid_vs_oracle(ctx, which, staging):
    from fluidloom_gb300.lbm import Pool
    c = cases_small()[which]
    gp, op = Pool(ctx, [c]), O.OraclePool([c])
    gp.set_options(staging=staging)
    assert gp.info().fluid_lups_per_step == op.lups()
    assert_pool_equal(gp, op)
    for rnd in range(2):
        gp.step(3)
        op.step(3)
        assert_pool_equal(gp, op)
        np.testing.assert_allclose(gp.conservation(), op.conservation(), rtol=1e-12, atol=1e-9)
        gfl, gwm = gp.flags()
        ofl, owm = op.flags()
        np.testing.assert_array_equal(gfl, ofl)
        np.testing.assert_array_equal(gwm, owm)
        gp.regrid()
        op.regrid()
        assert_pool_equal(gp, op)


def test_graphs_match_direct_launches(ctx):
    from fluidloom_gb300.lbm import Pool
    c = cases_small()[1]
    a, b = Pool(ctx, [c]), Pool(ctx, [c])
    a.set_options(graphs=1)
    b.set_options(graphs=0)
    a.step(5)
    b.step(5)
    np.testing.assert_array_equal(a.populations(), b.populations())


@pytest.mark.parametrize("graphs", [0, 1])
def test_concurrent_class_streams_match_one_stream(ctx, graphs):
    """General bricks on a second stream (fork/join, inside graphs or not) give the
    same populations as the three classes in order on one stream, across a regrid."""
    from fluidloom_gb300.lbm import Pool
    c = cases_small()[1]
    a, b = Pool(ctx, [c]), Pool(ctx, [c])
    a.set_options(graphs=graphs, streams=2)
    b.set_options(graphs=0, streams=1)
    for p in (a, b):
        p.step(4)
        p.regrid()
        p.step(3)
    np.testing.assert_array_equal(a.populations(), b.populations())


@pytest.mark.parametrize("staging", [1, 2])
@pytest.mark.parametrize("graphs", [0, 1])
def test_bulk_staged_kernels_match_register_kernels(ctx, staging, graphs):
    """The collide kernels with each brick's planes (and, in mode 2, the general bricks'
    quad masks and descriptor values) bulk-copied into shared memory give the register
    kernels' populations bit for bit, both cases in one pool, across a regrid."""
    from fluidloom_gb300.lbm import Pool
    cs = list(cases_small())
    a, b = Pool(ctx, cs), Pool(ctx, cs)
    a.set_options(graphs=graphs, staging=staging)
    b.set_options(graphs=graphs, staging=0)
    for p in (a, b):
        p.step(4)
        p.regrid()
        p.step(3)
    np.testing.assert_array_equal(a.populations(), b.populations())
    a.set_options(graphs=graphs, staging=0)  # and back: the pool keeps stepping in either mode
    for p in (a, b):
        p.step(2)
    np.testing.assert_array_equal(a.populations(), b.populations())


def test_graphs_after_upload_match_direct_launches(ctx):
    """After an upload the captured steps stay valid: the first steps replay graphs that also
    rewrite the all-solid bricks (the uploaded state is perturbed everywhere, inside the sphere
    too), then the plain ones, and every step equals uncaptured launches bit for bit."""
    from fluidloom_gb300.lbm import Pool
    c = cases_small()[1]
    a, b = Pool(ctx, [c]), Pool(ctx, [c])
    a.set_options(graphs=1)
    b.set_options(graphs=0)
    a.step(3)
    b.step(3)
    f = a.populations()
    f = (f * (1.0 + 1e-3 * np.random.default_rng(7).standard_normal(f.shape))).astype(np.float32)
    for rnd in range(2):
        a.upload(f)
        b.upload(f)
        for k in range(5):
            a.step(1)
            b.step(1)
            np.testing.assert_array_equal(a.populations(), b.populations())


@pytest.mark.parametrize("staging", [0, 1, 2])
def test_fused_conservation_sums_equal_recomputed(ctx, staging):
    """Each level's last sub-step writes its bricks' conservation sums from the values it
    stores; they equal k_brick_sums' recomputation from the stored state bit for bit (both
    cases in one pool: walls, a moving lid, the sphere's solid sites, three levels), after
    steps and after a regrid, in every staging mode."""
    from fluidloom_gb300.lbm import Pool
    p = Pool(ctx, list(cases_small()))
    p.set_options(staging=staging, step_sums=True)
    for rnd in range(2):
        p.step(3)
        fused = p.conservation()           # from the step's own sums
        p.upload(p.populations())          # the same state, marked replaced: sums recomputed
        again = p.conservation()
        np.testing.assert_array_equal(fused, again)
        p.regrid()
    p.close()


def test_conservation_async_equals_sync(ctx):
    """fl_pool_conservation_async queues the sums and their copy into pinned host memory
    without waiting; after a synchronise they equal the synchronous call's, step by step."""
    import ctypes
    from fluidloom_gb300.lbm import Pool
    p = Pool(ctx, [cases_small()[1]])
    p.set_options(step_sums=True)  # the sums of each step from the step itself
    cp = ctypes.c_void_p()
    ctx.call("fl_host_alloc_pinned", ctypes.c_size_t(3 * 32), ctypes.byref(cp))
    got = np.ctypeslib.as_array(ctypes.cast(cp, ctypes.POINTER(ctypes.c_double)), shape=(3, 4))
    got[:] = np.nan
    want = []
    q = Pool(ctx, [cases_small()[1]])
    for k in range(3):
        p.step(1)
        ctx.call("fl_pool_conservation_async", p.h, ctypes.c_void_p(cp.value + 32 * k))
        q.step(1)
        want.append(q.conservation()[0])
    ctx.sync()
    np.testing.assert_array_equal(got, np.array(want))
    ctx.call("fl_host_free_pinned", cp)
    p.close()
    q.close()


def test_batch_equals_solo(ctx):
    """Two cases in one pool reproduce their solo runs bit for bit."""
    from fluidloom_gb300.lbm import Pool
    cav, sph = cases_small()
    both = Pool(ctx, [cav, sph])
    s0, s1 = Pool(ctx, [cav]), Pool(ctx, [sph])
    for p in (both, s0, s1):
        p.step(4)
        p.regrid()
        p.step(2)
    bb, bf = both.bricks(), both.populations()
    for cs, solo in ((0, s0), (1, s1)):
        m = bb["case_id"] == cs
        sb = solo.bricks()
        for k in ("x", "y", "z", "level"):
            np.testing.assert_array_equal(bb[k][m], sb[k])
        np.testing.assert_array_equal(bf[:, m, :], solo.populations())
        np.testing.assert_array_equal(both.conservation()[cs], solo.conservation()[0])


def test_mass_conserved_closed_cavity(ctx):
    from fluidloom_gb300 import lbm
    from fluidloom_gb300.lbm import Pool
    p = Pool(ctx, [lbm.cavity(16, 0)])
    m0 = p.conservation()[0, 0]
    p.step(20)
    m1 = p.conservation()[0, 0]
    # single level, walls: bounce-back conserves mass up to FP32 round-off
    assert abs(m1 - m0) / m0 < 1e-5


def test_settled_solid_bricks_skip_equals_always_writing(ctx):
    """All-solid bricks are written only for two sub-steps per level after a change of the
    bricks or populations; a pool stepped that way equals one whose steps always write them
    (captured by the execution graph), after an upload that puts other values into solid
    sites and across a regrid."""
    from fluidloom_gb300 import graph as G
    from fluidloom_gb300.lbm import Pool
    c = cases_small()[1]
    a, b = Pool(ctx, [c]), Pool(ctx, [c])
    f = a.populations()
    f[:, :, :] += np.float32(0.25) * np.random.default_rng(5).random(f.shape, np.float32)
    a.upload(f)
    b.upload(f)
    g = G.Graph(ctx)
    g.add(G.LBM_STEP, "b", reads=["f"], writes=["f"], pool=b, nsteps=5)
    g.analyze()
    g.build()
    for _ in range(2):
        a.step(5)
        g.execute(cuda_graphs=True)
        ctx.sync()
        np.testing.assert_array_equal(a.populations(), b.populations())
        a.regrid()
        b.regrid()


def test_gpu_populations_against_fp64(ctx):
    """The GPU's FP32 populations within 1e-5 relative of an FP64 run of the same steps."""
    from fluidloom_gb300.lbm import Pool
    c = cases_small()[1]
    gp, op = Pool(ctx, [c]), O.OraclePool([c])
    ref = op.fp64_steps(6)
    gp.step(6)
    f = gp.populations().astype(np.float64)
    assert float(np.max(np.abs(f - ref) / np.maximum(np.abs(ref), 1e-30))) < 1e-5
