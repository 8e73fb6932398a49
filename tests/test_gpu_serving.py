"""Cases merged into / removed from a running pool and per-case regrids: every
case keeps reproducing its solo run bit for bit (the serving pattern's
correctness condition)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _cases():
    from fluidloom_gb300 import lbm
    a = lbm.cavity(16, 1, u_lid=0.06, tau=0.6)
    b = lbm.sphere_channel(32, 16, 16, 2, radius=2.0, centre=(8.0, 8.0, 8.0), u_in=0.04, band=2.0)
    c = lbm.cavity(24, 2, u_lid=0.03, tau=0.55)
    return a, b, c


def _state(pool, cid):
    g, f = pool.case_state(cid)
    return g, f


def _same(p1, c1, p2, c2):
    g1, f1 = _state(p1, c1)
    g2, f2 = _state(p2, c2)
    for k in ("x", "y", "z", "level"):
        np.testing.assert_array_equal(g1[k], g2[k])
    np.testing.assert_array_equal(f1, f2)


def test_add_remove_and_per_case_regrid_match_solo(ctx):
    from fluidloom_gb300.lbm import Pool
    a, b, c = _cases()
    mix = Pool(ctx, [a])
    sa, sb, sc = Pool(ctx, [a]), Pool(ctx, [b]), Pool(ctx, [c])
    # A runs 3 steps, then B and C join
    mix.step(3)
    sa.step(3)
    ids = mix.add_cases([b, c])
    assert sorted(ids) == [1, 2]
    ib, ic = ids
    _same(mix, 0, sa, 0)
    _same(mix, ib, sb, 0)
    _same(mix, ic, sc, 0)
    # 4 more steps; A regrids alone (B, C not due)
    mix.step(4)
    for p in (sa, sb, sc):
        p.step(4)
    mix.regrid_cases([0])
    sa.regrid()
    _same(mix, 0, sa, 0)
    _same(mix, ib, sb, 0)
    _same(mix, ic, sc, 0)
    # A finishes and leaves; B and C continue, B regrids
    mix.remove_cases([0])
    mix.step(2)
    sb.step(2)
    sc.step(2)
    mix.regrid_cases([ib])
    sb.regrid()
    _same(mix, ib, sb, 0)
    _same(mix, ic, sc, 0)
    # a new case reuses the freed id
    ids2 = mix.add_cases([a])
    assert ids2 == [0]
    sa2 = Pool(ctx, [a])
    mix.step(2)
    sa2.step(2)
    sb.step(2)
    _same(mix, 0, sa2, 0)
    _same(mix, ib, sb, 0)
    info = mix.info()
    assert info.num_active_cases == 3


def test_pool_emptied_and_refilled(ctx):
    """Every case leaves (a pool of no bricks: empty level lists, case ranges and
    descriptor tables), the pool steps and regrids empty, then a new case joins
    and runs as it does alone."""
    from fluidloom_gb300.lbm import Pool
    a, b, c = _cases()
    mix = Pool(ctx, [a, b])
    mix.step(2)
    mix.remove_cases([0, 1])
    info = mix.info()
    assert info.num_bricks == 0 and info.fluid_lups_per_step == 0 and info.num_active_cases == 0
    mix.step(2)
    mix.regrid()
    ids = mix.add_cases([c])
    solo = Pool(ctx, [c])
    for p in (mix, solo):
        p.step(3)
        p.regrid()
        p.step(1)
    _same(mix, ids[0], solo, 0)
    assert mix.info().fluid_lups_per_step == solo.info().fluid_lups_per_step


def test_served_loop_matches_solo_runs(ctx):
    """The serving loop (admission at regrid boundaries, shared regrids, removal at
    completion) leaves every job with the state of its solo run."""
    from fluidloom_gb300 import lbm, serving
    a, b, c = _cases()
    jobs = [serving.Job(0, 0.0, a, 45), serving.Job(1, 0.0, b, 30), serving.Job(2, 0.002, c, 61)]
    lups, makespan, steps_run = serving.run_served(ctx, jobs, budget_bytes=1e12, check_ids={0, 1, 2})
    assert lups > 0 and makespan > 0 and steps_run >= 61
    for j in jobs:
        assert j.end is not None and j.end >= j.start >= j.arrival
        _, _, solo = serving.run_solo(ctx, j)
        g1, f1 = j.result
        g2, f2 = solo
        for k in ("x", "y", "z", "level"):
            np.testing.assert_array_equal(g1[k], g2[k])
        np.testing.assert_array_equal(f1, f2)


def test_admission_defers_and_refuses_under_a_small_budget(ctx):
    """A budget of 100 level-0 bricks' worth of populations: the first 32^3 cavity
    (64 bricks) is admitted, the second would bring the resident bricks to 128, so
    it is taken out again and admitted once the first has finished (deferred, not
    lost), and the small third job waits behind it in arrival order; a job whose
    level-0 bricks alone exceed the budget is refused.  Every admitted job still
    ends in its solo state."""
    from fluidloom_gb300 import lbm, serving
    mid1 = lbm.cavity(32, 1, u_lid=0.04, tau=0.6)
    mid2 = lbm.cavity(32, 1, u_lid=0.03, tau=0.58)
    a = _cases()[0]
    big = lbm.sphere_channel(128, 64, 64, 1, radius=8.0, centre=(32.0, 32.0, 32.0), u_in=0.04, band=6.0)
    jobs = [serving.Job(0, 0.0, mid1, 25), serving.Job(1, 0.0, mid2, 25), serving.Job(2, 0.0, a, 25),
            serving.Job(3, 0.0, big, 25)]
    budget = 100 * serving.BRICK_BYTES
    assert jobs[3].start_bytes() > budget and all(j.start_bytes() <= budget for j in jobs[:3])
    lups, makespan, steps_run = serving.run_served(ctx, jobs, budget_bytes=budget, check_ids={0, 1, 2})
    assert jobs[3].refused and jobs[3].cid is None
    assert run_deferrals() > 0
    assert jobs[1].start >= jobs[0].end  # the second waited for the first
    for j in jobs[:3]:
        assert j.end is not None and j.refused is None
        _, _, solo = serving.run_solo(ctx, j)
        g1, f1 = j.result
        g2, f2 = solo
        for k in ("x", "y", "z", "level"):
            np.testing.assert_array_equal(g1[k], g2[k])
        np.testing.assert_array_equal(f1, f2)


def run_deferrals():
    from fluidloom_gb300 import serving
    return serving.run_served.deferrals


def test_cancelled_job_leaves_the_others_unchanged(ctx):
    """A job cancelled after 12 of its steps leaves the pool at that step boundary; the
    jobs that stay still end in their solo states."""
    from fluidloom_gb300 import serving
    a, b, c = _cases()
    jobs = [serving.Job(0, 0.0, a, 45), serving.Job(1, 0.0, b, 40), serving.Job(2, 0.0, c, 33)]
    cancel = lambda j, now: "cancelled by the test" if j.jid == 1 and j.done >= 12 else None
    serving.run_served(ctx, jobs, budget_bytes=1e12, check_ids={0, 2}, cancel=cancel)
    assert jobs[1].cancelled == "cancelled by the test" and jobs[1].done == 12
    for j in (jobs[0], jobs[2]):
        assert j.cancelled is None and j.done == j.steps
        _, _, solo = serving.run_solo(ctx, j)
        g1, f1 = j.result
        g2, f2 = solo
        for k in ("x", "y", "z", "level"):
            np.testing.assert_array_equal(g1[k], g2[k])
        np.testing.assert_array_equal(f1, f2)
