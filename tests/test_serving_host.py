"""Host logic of the serving loop (no GPU): run_served against a fake pool that keeps
per-case bricks and step counts, so admission order, deferral, refusal, regrid
scheduling and completion are checked without a device."""
import types

import pytest

from fluidloom_gb300 import serving
from fluidloom_gb300.lbm import cavity


class FakeServePool:
    """Cases hold their level-0 bricks (x2 once they have stepped: a refined mesh); the
    reserved buffers are the resident bricks' bytes rounded up to a 64-brick capacity."""
    log = []

    def __init__(self, ctx, cases):
        self.cases, self.steps, self.next = {}, {}, 0
        FakeServePool.log.append(("create",))
        self.add_cases(cases)

    def _bricks(self, cid):
        e = self.cases[cid].ext
        return int(e[0] * e[1] * e[2]) * (2 if self.steps[cid] else 1)

    def add_cases(self, cases):
        ids = []
        for c in cases:
            self.cases[self.next], self.steps[self.next] = c, 0
            ids.append(self.next)
            FakeServePool.log.append(("add", self.next))
            self.next += 1
        return ids

    def remove_cases(self, ids):
        for i in ids:
            del self.cases[i], self.steps[i]
            FakeServePool.log.append(("remove", i))

    def info(self):
        n = sum(self._bricks(c) for c in self.cases)
        return types.SimpleNamespace(num_bricks=n, fluid_lups_per_step=n * 512,
                                     population_bytes=-(-n // 64) * 64 * serving.BRICK_BYTES)

    def step(self, k):
        for c in self.steps:
            self.steps[c] += k

    def regrid(self):
        FakeServePool.log.append(("regrid", tuple(sorted(self.cases))))

    def regrid_cases(self, ids):
        FakeServePool.log.append(("regrid", tuple(sorted(ids))))

    def case_state(self, cid):
        return ("state", cid, self.steps[cid])

    def close(self):
        FakeServePool.log.append(("close",))


class FakeCtx:
    def sync(self):
        pass


@pytest.fixture
def fake_pool(monkeypatch):
    FakeServePool.log = []
    monkeypatch.setattr(serving, "Pool", FakeServePool)
    return FakeServePool


def _jobs(specs):
    return [serving.Job(i, 0.0, cavity(edge, 1), steps) for i, (edge, steps) in enumerate(specs)]


def test_jobs_run_to_completion_in_arrival_order(fake_pool):
    jobs = _jobs([(16, 40), (16, 25), (32, 60)])
    lups, makespan, steps_run = serving.run_served(FakeCtx(), jobs, budget_bytes=10 ** 12, check_ids=(0, 2))
    assert all(j.done == j.steps and j.end is not None and j.refused is None for j in jobs)
    adds = [e[1] for e in fake_pool.log if e[0] == "add"]
    assert adds == [0, 1, 2]  # everything fits: admitted together, in arrival order
    assert steps_run == 60 and lups > 0
    assert jobs[0].result == ("state", 0, 40) and jobs[2].result == ("state", 2, 60)
    assert jobs[1].result is None  # not a checked job
    # each job regrids every 20 of its own steps, never at its last one: all three at step 20
    # (one pool regrid), job 2 alone at 40 (job 0 ends there), none at 60
    regrids = [e[1] for e in fake_pool.log if e[0] == "regrid"]
    assert regrids == [(0, 1, 2), (2,)]


def test_resident_cap_defers_then_admits(fake_pool):
    # 2x2x2 level-0 bricks per 16^3 cavity, twice that once stepped: 8 -> 16 bricks each; a cap
    # of 12 bricks holds one job, not two
    jobs = _jobs([(16, 20), (16, 20), (16, 20)])
    serving.run_served(FakeCtx(), jobs, budget_bytes=10 ** 12, resident_bytes=12 * serving.BRICK_BYTES)
    assert all(j.done == j.steps for j in jobs)
    # job 1 is added next to job 0 and taken out again (over the cap), then admitted once job 0 ends
    assert serving.run_served.deferrals >= 1
    assert jobs[0].end <= jobs[1].start <= jobs[1].end <= jobs[2].start


def test_job_above_the_budget_is_refused(fake_pool):
    jobs = _jobs([(16, 20), (64, 20)])
    budget = jobs[1].start_bytes() - 1
    serving.run_served(FakeCtx(), jobs, budget_bytes=budget)
    assert jobs[0].refused is None and jobs[0].done == 20
    assert jobs[1].refused and "budget" in jobs[1].refused and jobs[1].done == 0
    assert ("add", 1) not in fake_pool.log


def test_trace_of_the_served_timeline(fake_pool, tmp_path):
    import json
    jobs = _jobs([(16, 20), (16, 20), (64, 20)])
    serving.run_served(FakeCtx(), jobs, budget_bytes=jobs[2].start_bytes() - 1,
                       resident_bytes=12 * serving.BRICK_BYTES)
    path = tmp_path / "t.json"
    serving.write_trace(jobs, str(path))
    ev = json.load(open(path))
    for j in jobs[:2]:
        mine = [e for e in ev if e["tid"] == j.jid]
        queued, resident = mine
        assert queued["ph"] == resident["ph"] == "X" and queued["cat"] == "queue"
        assert queued["ts"] + queued["dur"] == resident["ts"]  # admitted when the queue span ends
        assert resident["args"]["steps"] == 20 and resident["dur"] >= 0
    assert sum(e["args"]["deferred"] for e in ev if e["cat"] == "resident") >= 1
    refused = [e for e in ev if e["tid"] == 2]
    assert len(refused) == 1 and refused[0]["ph"] == "i" and "budget" in refused[0]["args"]["reason"]


def test_cancelled_jobs_leave_at_a_step_boundary(fake_pool):
    # job 1 is cancelled after 10 of its steps (resident), job 2 while it waits in the queue
    jobs = _jobs([(16, 40), (16, 40), (16, 40)])

    def cancel(j, now):
        if j.jid == 1 and j.done >= 10:
            return "client cancelled"
        if j.jid == 2 and jobs[0].done >= 5 and j.start is None:
            return "client cancelled"
        return None

    serving.run_served(FakeCtx(), jobs, budget_bytes=10 ** 12, resident_bytes=20 * serving.BRICK_BYTES,
                       cancel=cancel)
    assert jobs[0].done == 40 and jobs[0].cancelled is None
    assert jobs[1].cancelled == "client cancelled" and jobs[1].done == 10 and jobs[1].end is not None
    assert ("remove", jobs[1].cid) in fake_pool.log  # its case left the pool
    assert jobs[2].cancelled and jobs[2].start is None and jobs[2].done == 0
    assert jobs[2].deferred >= 1 and jobs[2].cid is None  # tried once (over the cap), never resident
    ev = serving.trace_events(jobs)
    assert [e["name"] for e in ev if e["ph"] == "i"] == ["job 1 cancelled", "job 2 cancelled"]


def test_deadline_cancels(fake_pool):
    jobs = [serving.Job(0, 0.0, cavity(16, 1), 30), serving.Job(1, 0.0, cavity(16, 1), 30, deadline=0.0)]
    serving.run_served(FakeCtx(), jobs, budget_bytes=10 ** 12)
    assert jobs[0].done == 30 and jobs[0].cancelled is None
    assert jobs[1].cancelled.startswith("deadline") and jobs[1].done < 30
