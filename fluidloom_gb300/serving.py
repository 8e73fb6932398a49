"""Serving: a request loop that admits AMR-LBM jobs as they arrive, merges them
into the running pool at level-0 step boundaries (continuous batching), keeps
every case resident on the device until it finishes, and reports aggregate
MLUPS with p50/p99 time-to-completion against plain sequential GPU runs of the
same jobs (one job at a time, arrival order).

  python -m fluidloom_gb300.serving [--rate 50] [--duration 60] [--steps 200 2000] [--budget-gb 150] [--trace t.json]

Jobs (synthetic, seeded): Poisson arrivals; 70 % lid-driven cavities, 30 %
sphere-in-channel; base size log-uniform between 16^3 and 128x64x64 sites;
1-3 refinement levels; steps uniform in the given range; regrid every 20
steps.  Jobs are admitted at pool steps that are multiples of the regrid
interval, so every resident job's regrids fall on the same pool steps and one
regrid of the due cases serves them all (each job still regrids every 20 of
its own steps, exactly as when it runs alone).  Admission is gated by each
job's population footprint against the HBM budget.  A job's result is its
final state; for --check jobs it is compared bit for bit with the same job run
alone.
"""
import argparse
import collections
import json
import time

import numpy as np

from . import Context
from .lbm import Pool, cavity, sphere_channel

BRICK_BYTES = 3 * 19 * 512 * 4  # three population buffers per brick


class Job:
    __slots__ = ("jid", "arrival", "case", "steps", "regrid_every", "done", "cid", "start", "end", "result",
                 "refused", "deferred", "deadline", "cancelled")

    def __init__(self, jid, arrival, case, steps, regrid_every=20, deadline=None):
        self.jid, self.arrival, self.case, self.steps, self.regrid_every = jid, arrival, case, steps, regrid_every
        self.deadline = deadline  # seconds from arrival to completion; past it the job is cancelled
        self.cancelled = None  # the reason, when the job was cancelled before it finished
        self.done = 0
        self.cid = None
        self.start = self.end = None
        self.result = None
        self.refused = None  # the reason, when admission refused the job for good
        self.deferred = 0  # times it was added and taken out again over the budget

    def start_bytes(self):
        """Population bytes of the job's level-0 bricks: the least it holds from its first step,
        so a job whose bound exceeds the whole budget can never run."""
        e = self.case.ext
        return int(e[0] * e[1] * e[2]) * BRICK_BYTES


def make_jobs(rate, duration, steps_range, seed=5):
    rng = np.random.default_rng(seed)
    t, jobs = 0.0, []
    while True:
        t += rng.exponential(1.0 / rate)
        if t >= duration:
            break
        lv = int(rng.integers(1, 4))
        steps = int(rng.integers(steps_range[0], steps_range[1] + 1))  # regrid interval 20 for every job
        if rng.random() < 0.7:
            edge = int(np.exp(rng.uniform(np.log(16), np.log(64))))
            edge = int(min(64, max(16, 8 * round(edge / 8))))
            case = cavity(edge, lv, u_lid=float(rng.uniform(0.02, 0.08)), tau=float(rng.uniform(0.52, 0.8)))
        else:
            s = float(np.exp(rng.uniform(0.0, np.log(4.0))))  # channel scale 1..4 -> 32x16x16 .. 128x64x64
            nx = int(min(128, max(32, 32 * round(s))))
            ny = nz = nx // 2
            case = sphere_channel(nx, ny, nz, lv, radius=nx / 16.0, centre=(nx / 4.0, ny / 2.0, nz / 2.0),
                                  u_in=0.04, tau=0.56, band=nx / 21.0)
        jobs.append(Job(len(jobs), t, case, steps))
    return jobs


def used_bytes(pool):
    """Population bytes the pool's resident bricks hold (three buffers per brick)."""
    return 0 if pool is None else int(pool.info().num_bricks) * BRICK_BYTES


def reserved_bytes(pool):
    """The pool's device footprint as the library reports it: its three population buffers
    at their current capacity (fl_pool_info population_bytes)."""
    return 0 if pool is None else int(pool.info().population_bytes)


def _cancel_reason(j, now, cancel):
    if cancel is not None:
        why = cancel(j, now)
        if why:
            return str(why)
    if j.deadline is not None and now - j.arrival > j.deadline:
        return "deadline of %.3f s passed" % j.deadline
    return None


def run_served(ctx, jobs, budget_bytes, check_ids=(), regrid_every=20, resident_bytes=None, admit_every=None,
               cancel=None):
    """Continuous batching; returns the LUPs done, the makespan and the pool steps run.

    Jobs are admitted in arrival order at pool steps that are multiples of
    admit_every (default: the regrid interval, so that resident jobs share their
    regrids), gated by measured bytes: a queued job is added, and if the bricks
    then resident hold more than min(budget_bytes, resident_bytes), or the pool's
    reserved buffers exceed budget_bytes, it is taken out again and waits
    (deferred) -- it keeps the footprint it was measured at, so it is only tried
    again once that fits.  A job whose level-0 bricks alone exceed the whole
    budget (start_bytes) is refused.  resident_bytes is the throughput knob:
    enough resident bricks to keep HBM busy, and no more, so queued jobs start in
    order instead of all sharing the GPU.

    Cancellation, at step boundaries (no kernel of the pool in flight): a queued or
    resident job is cancelled when cancel(job, now) returns a reason, or when its
    deadline (seconds from arrival) has passed; a resident job's case leaves the pool
    like a finished one, and the other jobs go on unaffected."""
    cap = budget_bytes if resident_bytes is None else min(budget_bytes, resident_bytes)
    admit_every = admit_every or regrid_every
    pending = collections.deque(sorted(jobs, key=lambda j: j.arrival))
    queue, active = collections.deque(), {}
    need = {}  # job id -> bytes its bricks took when it was last added
    pool = None
    lups = 0
    steps_run = 0
    phase = 0  # pool steps since the last admission boundary (restarts whenever the pool empties)
    deferrals = 0
    t0 = time.perf_counter()
    while pending or queue or active:
        now = time.perf_counter() - t0
        while pending and pending[0].arrival <= now:
            j = pending.popleft()
            if j.start_bytes() > budget_bytes:
                j.refused = "level-0 footprint %.3f GB above the %.3f GB budget" % (j.start_bytes() / 1e9,
                                                                                   budget_bytes / 1e9)
                j.start = j.end = now
                continue
            queue.append(j)
        for j in [j for j in queue if _cancel_reason(j, now, cancel)]:
            queue.remove(j)
            j.cancelled, j.end = _cancel_reason(j, now, cancel), now
        gone = [cid for cid, j in active.items() if _cancel_reason(j, now, cancel)]
        if gone:
            for cid in gone:
                j = active.pop(cid)
                j.cancelled, j.end = _cancel_reason(j, now, cancel), now
            pool.remove_cases(gone)
        if not active:
            phase = 0
        if phase % admit_every == 0 and queue:
            used = used_bytes(pool)
            while queue:
                j = queue[0]
                if active and j.jid in need and used + need[j.jid] > cap:
                    break  # known not to fit until jobs finish
                if pool is None:
                    pool = Pool(ctx, [j.case])
                    cid = 0
                else:
                    cid = pool.add_cases([j.case])[0]
                now_used = used_bytes(pool)
                need[j.jid] = now_used - used
                if active and (now_used > cap or reserved_bytes(pool) > budget_bytes):
                    pool.remove_cases([cid])  # over the budget: back to the queue until jobs finish
                    deferrals += 1
                    j.deferred += 1
                    break
                used = now_used
                queue.popleft()
                j.cid, j.start = cid, time.perf_counter() - t0
                active[cid] = j
        if not active:
            if pending:
                time.sleep(max(0.0, min(0.05, pending[0].arrival - (time.perf_counter() - t0))))
            continue
        lups += pool.info().fluid_lups_per_step
        pool.step(1)
        steps_run += 1
        phase += 1
        due = []
        for cid, j in active.items():
            j.done += 1
            if j.regrid_every and j.done % j.regrid_every == 0 and j.done < j.steps:
                due.append(cid)
        if due:
            if len(due) == len(active):
                pool.regrid()
            else:
                pool.regrid_cases(due)
        fin = [cid for cid, j in active.items() if j.done >= j.steps]
        if fin:
            ctx.sync()
            now = time.perf_counter() - t0
            for cid in fin:
                j = active.pop(cid)
                j.end = now
                if j.jid in check_ids:
                    j.result = pool.case_state(cid)
            pool.remove_cases(fin)
    ctx.sync()
    makespan = time.perf_counter() - t0
    if pool is not None:
        pool.close()
    run_served.deferrals = deferrals
    return lups, makespan, steps_run


def trace_events(jobs):
    """The served timeline as Chrome trace events, in the reference profiler's event format
    (src/profiling/Profiler.cpp:53-96: name, cat, ph, ts and dur in microseconds, pid, tid):
    per job, on a track of its own, a "queued" span from arrival to admission and a
    "resident" span from admission to completion (its steps, case slot and deferrals as
    args); a refused job is an instant event at its arrival with the reason, a cancelled
    one an instant event when it was cancelled."""
    ev = []
    for j in sorted(jobs, key=lambda j: j.jid):
        base = {"pid": 0, "tid": int(j.jid)}
        if j.refused:
            ev.append(dict(base, name="job %d refused" % j.jid, cat="admission", ph="i", s="t",
                           ts=int(round(j.arrival * 1e6)), args={"reason": j.refused}))
            continue
        if j.end is None:
            continue
        a, en = int(round(j.arrival * 1e6)), int(round(j.end * 1e6))
        st = en if j.start is None else int(round(j.start * 1e6))  # a job cancelled in the queue
        ev.append(dict(base, name="job %d queued" % j.jid, cat="queue", ph="X", ts=a, dur=max(0, st - a)))
        if j.start is not None:
            ev.append(dict(base, name="job %d" % j.jid, cat="resident", ph="X", ts=st, dur=max(0, en - st),
                           args={"steps": int(j.steps), "steps_done": int(j.done), "case_slot": j.cid,
                                 "deferred": int(j.deferred)}))
        if j.cancelled:
            ev.append(dict(base, name="job %d cancelled" % j.jid, cat="admission", ph="i", s="t", ts=en,
                           args={"reason": j.cancelled}))
    return ev


def write_trace(jobs, path):
    """trace_events(jobs) as a JSON array (chrome://tracing, Perfetto)."""
    with open(path, "w") as f:
        json.dump(trace_events(jobs), f)


def run_solo(ctx, job):
    """The same job alone on the GPU; returns (seconds, LUPs, final state)."""
    p = Pool(ctx, [job.case])
    ctx.sync()
    t0 = time.perf_counter()
    lups = 0
    for s in range(1, job.steps + 1):
        lups += p.info().fluid_lups_per_step
        p.step(1)
        if job.regrid_every and s % job.regrid_every == 0 and s < job.steps:
            p.regrid()
    ctx.sync()
    dt = time.perf_counter() - t0
    state = p.case_state(0)
    p.close()
    return dt, lups, state


def percentile(v, q):
    return float(np.percentile(np.asarray(v), q)) if len(v) else None


def benchmark(ctx, rate=50.0, duration=60.0, steps_range=(200, 2000), budget_gb=150.0, resident_gb=6.0, check=8,
              seed=5, trace=None):
    """Serve the arrival stream, then run the same jobs one at a time in arrival order;
    returns throughput and p50/p99 time to completion of both, and the checked jobs whose
    served result differs from their solo run.  trace: a path for the served timeline
    (write_trace)."""
    jobs = make_jobs(rate, duration, list(steps_range), seed)
    check_ids = set(range(min(check, len(jobs))))
    lups, makespan, steps_run = run_served(ctx, jobs, budget_gb * 1e9, check_ids, resident_bytes=resident_gb * 1e9)
    if trace:
        write_trace(jobs, trace)
    refused = [j for j in jobs if j.refused]
    jobs = [j for j in jobs if not j.refused and not j.cancelled]
    lat = [j.end - j.arrival for j in jobs]
    # plain sequential: each job alone, one after another in arrival order
    end_prev, lat_plain, solo_s, solo_lups, mismatched = 0.0, [], 0.0, 0, []
    for j in sorted(jobs, key=lambda j: j.arrival):
        dt, lu, state = run_solo(ctx, j)
        solo_s += dt
        solo_lups += lu
        start = max(j.arrival, end_prev)
        end_prev = start + dt
        lat_plain.append(end_prev - j.arrival)
        if j.jid in check_ids:
            g1, f1 = j.result
            g2, f2 = state
            same = all(np.array_equal(g1[k], g2[k]) for k in ("x", "y", "z", "level")) and np.array_equal(f1, f2)
            if not same:
                mismatched.append(j.jid)
    return {"jobs": len(jobs), "rate_per_s": rate, "duration_s": duration, "steps_range": list(steps_range),
            "admission": "arrival order, resident bricks' bytes <= %.1f GB, reserved buffers <= the %.0f GB budget"
                         % (resident_gb, budget_gb),
            "served_makespan_s": round(makespan, 3), "served_mlups": round(lups / makespan / 1e6, 1),
            "served_p50_s": percentile(lat, 50), "served_p99_s": percentile(lat, 99),
            "plain_mlups": round(solo_lups / solo_s / 1e6, 1), "plain_makespan_s": round(end_prev, 3),
            "plain_p50_s": percentile(lat_plain, 50), "plain_p99_s": percentile(lat_plain, 99),
            "pool_steps": steps_run, "checked": sorted(check_ids), "mismatched": mismatched,
            "refused": len(refused), "deferrals": run_served.deferrals}


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--rate", type=float, default=50.0)
    ap.add_argument("--duration", type=float, default=60.0)
    ap.add_argument("--steps", type=int, nargs=2, default=[200, 2000])
    ap.add_argument("--budget-gb", type=float, default=150.0)
    ap.add_argument("--resident-gb", type=float, default=6.0,
                    help="admission stops while the resident population footprint exceeds this")
    ap.add_argument("--check", type=int, default=8, help="jobs whose result is compared with their solo run")
    ap.add_argument("--seed", type=int, default=5)
    ap.add_argument("--trace", default=None, help="write the served timeline as a Chrome trace JSON file")
    args = ap.parse_args(argv)
    ctx = Context(0)
    res = benchmark(ctx, args.rate, args.duration, args.steps, args.budget_gb, args.resident_gb, args.check,
                    args.seed, trace=args.trace)
    print(json.dumps(res))
    return res


if __name__ == "__main__":
    main()
