"""bench.py — AMR lattice-Boltzmann throughput on one GB300 (flow past a sphere).

Workload (the headline configuration): D3Q19 BGK, FP32 SoA populations in
8^3-site bricks, base grid 128x64x64 sites (16x8x8 level-0 bricks), 3
refinement levels, sphere of radius 8 base sites at (32,32,32) with half-way
bounce-back, equilibrium inlet u=0.04 at x=0, zero-gradient outlet, periodic
y/z, tau_0 = 0.56; bricks within 6 base sites of the sphere surface refined to
level 3 (balanced 2:1 over faces, edges and corners); regrid every 25 steps
from vorticity (refine > 0.5 max, coarsen < 0.1 max) plus the band.  A step is
one level-0 time step (level l sub-cycled 2^l times).  Synthetic, seeded
inputs: the reference publishes no dataset or benchmark numbers.

value = fluid lattice updates per second over all ranks (MLUPS), populations
resident in HBM.  e2e = the same through the public C ABI from pinned host
memory: the full population state uploaded at the start and downloaded at the
end of the timed region, per-step inlet/wall velocities host->device and the
per-step FP64 mass/momentum read back.  Also reported: regrid ms per cycle on
this workload and the 16.7M-leaf regrid microbenchmark (flags, 2:1 balance,
split/merge, 63-bit key sort, compaction, neighbour rebuild).

  python bench.py [--gpus N --steps K --warmup W] [--impl reference]
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

BYTES_PER_LUP = 152  # 19 FP32 reads + 19 FP32 writes per fluid site update
REGRID_EVERY = 25
METRIC = "AMR-LBM MLUPS (D3Q19, flow past a sphere)"
UNIT = "MLUPS"


RUN_STEPS = 1000  # the configuration's run length
# Vorticity thresholds of the sphere case, as fractions of the case's maximum |vorticity|: the
# configuration names "a threshold" and "about 20 M leaf cells at peak"; over its 1000 steps
# the peak fluid sites are 8.5 M at 0.5 (only the band refines), 11.7 M at 0.1, 14.9 M at
# 0.07, 18.2 M at 0.05 and 24.3 M at 0.03, so 0.04 (coarsen below 0.015) gives about 20 M.
SPHERE_REFINE_FRAC, SPHERE_COARSEN_FRAC = 0.04, 0.015


def sphere_case(scale=1):
    from fluidloom_gb300 import lbm
    c = lbm.sphere_channel(128 // scale, 64 // scale, 64 // scale, 3, radius=8.0 / scale,
                           centre=(32.0 / scale,) * 3, u_in=0.04, tau=0.56, band=6.0 / scale)
    c.refine_frac, c.coarsen_frac = SPHERE_REFINE_FRAC, SPHERE_COARSEN_FRAC
    return c


def workload_config(extra=None):
    c = {"workload": "flow past a sphere, D3Q19 BGK FP32, 128x64x64 base, 3 levels, r=8, u=0.04, tau0=0.56",
         "base_grid": [128, 64, 64], "levels": 3, "brick": "8^3 sites", "regrid_every": REGRID_EVERY,
         "refine": "6-cell band around the sphere, plus bricks with |vorticity| > %g of the case's maximum "
                   "(coarsen below %g)" % (SPHERE_REFINE_FRAC, SPHERE_COARSEN_FRAC),
         "l2": "inputs larger than L2 (populations > 129 MB), no flush", "graphs": True}
    if extra:
        c.update(extra)
    return c


# ---------------------------------------------------------------- clocks
class ClockSampler:
    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.path = None

    def start(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + q,
                                          "--format=csv,noheader,nounits", "-lms", "50"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
            return
        # the sampler is up once it has written its first sample (at most 3 s)
        t0 = time.time()
        while time.time() - t0 < 3.0 and self.proc.poll() is None:
            if os.path.getsize(self.path) > 0:
                break
            time.sleep(0.01)

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(5)
        except Exception:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            p = [x.strip() for x in line.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                mx.append(float(p[2]))
            except ValueError:
                continue
            for nm, v in zip(names, p[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        os.unlink(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peak():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        return float(json.load(open(p))["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def ncu_traffic():
    """DRAM bytes per fluid site update of the collide-stream, from the committed ncu summary
    (dram__bytes_read.sum + dram__bytes_write.sum of one level-3 sub-step / its fluid sites)."""
    p = os.path.join(ROOT, "profiles", "collide_stream_sphere_ncu.md")
    if not os.path.exists(p):
        return None
    for line in open(p):
        if line.startswith("dram_bytes_per_fluid_site:"):
            try:
                return float(line.split(":", 1)[1])
            except ValueError:
                return None
    return None


# ---------------------------------------------------------------- GPU arm
def timer(ctx):
    import ctypes
    ctx.call("fl_ctx_timer_start")

    def stop():
        ms = ctypes.c_float()
        ctx.call("fl_ctx_timer_stop", ctypes.byref(ms))
        return ms.value
    return stop


def blob_table(seed, n=64):
    """Seeded Gaussian blobs over the unit cube: {cx, cy, cz, 1/(2 sigma^2), amplitude},
    centres uniform, sigma uniform in [0.02, 0.1] of the domain."""
    rng = np.random.default_rng(seed)
    c = rng.random((n, 3))
    s = rng.uniform(0.02, 0.1, n)
    return np.ascontiguousarray(np.concatenate([c, (1 / (2 * s * s))[:, None], np.ones((n, 1))], 1), np.float32)


def microbench_mesh(L=8):
    """The regrid microbenchmark's synthetic octree: a uniform level-L mesh (8^L leaves)
    regridded once by thresholding blob field 1 (refine above 0.7 to level L+1, coarsen
    below 0.4) -- about 0.98 x 8^L leaves over three levels -- then the benchmark's
    regrid by an independent blob field 2 (same thresholds, up to level L+2), whose
    refinement crosses the first regrid's level boundaries so FULL26 balance iterates."""
    n1 = 1 << L
    idx = np.arange(n1 ** 3, dtype=np.int64)
    N = len(idx)
    start = {"x": (idx % n1).astype(np.int32), "y": ((idx // n1) % n1).astype(np.int32),
             "z": (idx // (n1 * n1)).astype(np.int32), "level": np.full(N, L, np.uint8),
             "state": np.zeros(N, np.uint8), "flags": np.zeros(N, np.int32), "material": np.zeros(N, np.uint32)}
    return {"start": start, "regrids": [(blob_table(1), 0.4, 0.7, L + 1), (blob_table(2), 0.4, 0.7, L + 2)]}


def regrid_microbench(ctx, L=8):
    """The regrid of the microbenchmark octree (microbench_mesh; the first regrid untimed):
    blob flags, FULL26 balance to a fixed point, split/merge, key-order rebuild, the
    neighbour table; then a 63-bit key sort of the result alone and the primitives."""
    import ctypes
    from fluidloom_gb300 import DeviceArray
    from fluidloom_gb300.amr import AdaptConfig, AdaptStats, Mesh
    mb = microbench_mesh(L)
    m = Mesh(ctx, mb["start"], capacity=1 << (3 * L))
    out = {}
    st = None
    for r, (blobs, lo, hi, ml) in enumerate(mb["regrids"]):
        # the second regrid's input is the first's output: stated balanced when its balance converged
        cfg = AdaptConfig.make(max_level=ml, min_level=0, balance_mode=1,
                               input_balanced=st is not None and st.balance.converged == 1)
        leaves_in = m.n
        stop = timer(ctx)
        ctx.call("fl_flags_from_blobs", ctypes.byref(m.m), blobs.ctypes.data_as(ctypes.c_void_p), len(blobs),
                 ctypes.c_float(lo), ctypes.c_float(hi), ml)
        flags_ms = stop()
        st = AdaptStats()
        fp = ctypes.c_void_p(0)
        stop = timer(ctx)
        ctx.call("fl_adapt", ctypes.byref(m.m), ctypes.byref(cfg), ctypes.byref(fp), 0, ctypes.byref(st))
        adapt_ms = stop()
    out["flags_ms"], out["adapt_ms"] = flags_ms, adapt_ms
    n = m.n
    nbr = DeviceArray(ctx, (n * 26,), np.uint32)
    stop = timer(ctx)
    ctx.call("fl_neighbour_rebuild", ctypes.byref(m.m), ctypes.byref(cfg), 1, nbr.ptr)
    out["neighbour_ms"] = stop()
    nbr.free()
    # the leaves' 63-bit keys: the 21-level Hilbert key of each leaf's anchor (unique per leaf),
    # with uint32 leaf ids, shuffled so the sort has work to do
    keys = DeviceArray(ctx, (n,), np.uint64)
    ctx.call("fl_cell_keys", m.m.x, m.m.y, m.m.z, m.m.level, None, 21, 21, keys.ptr, n)
    perm = np.random.default_rng(5).permutation(n).astype(np.uint32)
    hk = keys.to_host()[perm]
    keys.free()
    # the sort's shape (digit width, tile threads) tuned on copies of these keys (each shape's
    # first call untimed, so the library's scratch already has its size), then the timed sort
    from fluidloom_gb300.batching import autotune_sort
    shape, shape_ms = autotune_sort(ctx, hk, perm, 0, 63)
    out["sort_shape"] = {"digit_bits": shape[0], "tile_threads": shape[1], "passes": -(-63 // shape[0]),
                         "tuned_ms": {"%dx%d" % s: round(t, 4) for s, t in shape_ms.items()}}
    keys = DeviceArray.from_host(ctx, hk)
    ids = DeviceArray.from_host(ctx, perm)
    del hk
    ctx.sync()
    stop = timer(ctx)
    ctx.call("fl_sort_pairs_u64_u32", keys.ptr, ids.ptr, n, 0, 63)
    out["sort_ms"] = stop()
    out["primitives"] = primitives_on(ctx, m, keys, ids, n, out)
    lv = np.bincount(m.download()["level"], minlength=L + 3)[L - 2:].tolist()
    out.update({"octree": "uniform level %d (%d leaves), regridded once by blob field 1; timed: the regrid by "
                          "blob field 2 (refine > 0.7 to level %d, coarsen < 0.4)" % (L, 8 ** L, L + 2),
                "leaves_in": int(leaves_in), "leaves_out": int(n), "levels_out_from_%d" % (L - 2): lv,
                "split": st.num_split, "merged_groups": st.num_groups,
                "balance_iterations": st.balance.iterations, "balance_marked": st.balance.total_cells_marked_for_balance,
                "sorted_keys_per_s": n / (out["sort_ms"] * 1e-3),
                "regrid_ms": out["flags_ms"] + out["adapt_ms"] + out["neighbour_ms"]})
    m.free()
    return out


def primitives_on(ctx, m, keys, ids, n, out):
    """The regrid's primitives alone on the n-leaf result mesh, each against the algorithmic
    bytes of its unit: encode 24 B per key (12 B coordinates in, 8 B key + 4 B id out); radix
    sort 8 + 24 B per key and pass (ceil(63 / d) passes of the tuned d-bit digits); scan 8 B per
    element; hash build 24 B per key + 12 B per slot cleared; hash query 12 B per query + one
    32-byte sector per probe; neighbour rebuild 104 B of table written + 23 B read per leaf
    (coordinates, level, locator key, directory share); halo pack / unpack of a 19-component field 4 + 2 x 76 B per cell
    (a random cell order); restriction 32 + 9 x 76 B per sibling group.  Times are
    CUDA-event times of one call each, after one untimed call of the same (so no call is
    timed while the library's scratch grows)."""
    import ctypes
    from fluidloom_gb300 import DeviceArray
    peak, _ = measured_peak()
    res = {}

    def put(name, ms, nbytes, units, unit_name):
        res[name] = {"ms": round(ms, 4), "gbs": round(nbytes / (ms * 1e-3) / 1e9, 1),
                     "frac_of_measured": round(nbytes / (ms * 1e-3) / 1e9 / peak, 3),
                     unit_name + "_per_s": round(units / (ms * 1e-3), 1)}

    N = ctypes.c_size_t(n)
    ek = DeviceArray(ctx, (n,), np.uint64)
    ei = DeviceArray(ctx, (n,), np.uint32)
    ctx.call("fl_hilbert_encode", m.m.x, m.m.y, m.m.z, 21, ek.ptr, ei.ptr, N)
    stop = timer(ctx)
    ctx.call("fl_hilbert_encode", m.m.x, m.m.y, m.m.z, 21, ek.ptr, ei.ptr, N)
    put("hilbert_encode", stop(), 24.0 * n, n, "keys")
    ek.free()
    ei.free()
    put("radix_sort", out["sort_ms"], (8.0 + 24.0 * out["sort_shape"]["passes"]) * n, n, "keys")
    a = DeviceArray(ctx, (n,), np.uint32).zero()
    b = DeviceArray(ctx, (n,), np.uint32)
    tot = DeviceArray(ctx, (1,), np.uint32)
    ctx.call("fl_scan_exclusive_u32", a.ptr, b.ptr, N, tot.ptr)
    stop = timer(ctx)
    ctx.call("fl_scan_exclusive_u32", a.ptr, b.ptr, N, tot.ptr)
    put("scan", stop(), 8.0 * n, n, "elements")
    ctx.lib.fl_hash_compute_capacity.restype = ctypes.c_uint64
    cap = int(ctx.lib.fl_hash_compute_capacity(N))
    tk = DeviceArray(ctx, (cap,), np.uint64)
    tv = DeviceArray(ctx, (cap,), np.uint32)
    ctx.call("fl_hash_build", tk.ptr, tv.ptr, ctypes.c_uint64(cap), keys.ptr, None, N)
    stop = timer(ctx)
    ctx.call("fl_hash_build", tk.ptr, tv.ptr, ctypes.c_uint64(cap), keys.ptr, None, N)
    put("hash_build", stop(), 24.0 * n + 12.0 * cap, n, "keys")
    ctx.call("fl_hash_query", tk.ptr, tv.ptr, ctypes.c_uint64(cap), keys.ptr, b.ptr, N)
    stop = timer(ctx)
    ctx.call("fl_hash_query", tk.ptr, tv.ptr, ctypes.c_uint64(cap), keys.ptr, b.ptr, N)
    put("hash_query", stop(), (12.0 + 32.0) * n, n, "queries")
    # algorithmic bytes: the 26-entry row written (104 B) and per leaf its coordinates and level
    # (13 B), its locator key (8 B) and its share of the bucket directory (2 B) read
    put("neighbour_rebuild", out["neighbour_ms"], (104.0 + 13.0 + 8.0 + 2.0) * n, 26 * n, "probes")
    for d in (a, tot, tk, tv):
        d.free()
    # ghost fill primitives over a 19-component field (populations-like): gather by index,
    # scatter back, and restriction of n/8 sibling groups (members in key order)
    C = 19
    fld = DeviceArray(ctx, (n * C,), np.float32).zero()
    pk = DeviceArray(ctx, (n * C,), np.float32)
    idx = DeviceArray.from_host(ctx, np.random.default_rng(3).permutation(n).astype(np.uint32))
    ctx.call("fl_pack_halo", fld.ptr, C, idx.ptr, N, pk.ptr)
    stop = timer(ctx)
    ctx.call("fl_pack_halo", fld.ptr, C, idx.ptr, N, pk.ptr)
    put("pack_halo", stop(), (4.0 + 2 * 4.0 * C) * n, n, "cells")
    ctx.call("fl_unpack_halo", pk.ptr, C, idx.ptr, N, fld.ptr)
    stop = timer(ctx)
    ctx.call("fl_unpack_halo", pk.ptr, C, idx.ptr, N, fld.ptr)
    put("unpack_halo", stop(), (4.0 + 2 * 4.0 * C) * n, n, "cells")
    g = n // 8
    mem = DeviceArray.from_host(ctx, np.arange(g * 8, dtype=np.uint32))
    ctx.call("fl_restrict_groups", fld.ptr, C, mem.ptr, ctypes.c_size_t(g), 0, pk.ptr)
    stop = timer(ctx)
    ctx.call("fl_restrict_groups", fld.ptr, C, mem.ptr, ctypes.c_size_t(g), 0, pk.ptr)
    put("restrict_groups", stop(), (32.0 + 9 * 4.0 * C) * g, g, "groups")
    for d in (b, fld, pk, idx, mem):
        d.free()
    return res


def fp64_error(ctx, steps=(1, 10)):
    """The GPU's FP32 populations against an FP64 run of the same steps (the oracle's
    arithmetic in double, same mesh) on the half-resolution sphere case: max relative
    difference over all sites and populations after each step count."""
    from fluidloom_gb300.lbm import Pool
    from tests import _oracle as O
    case = sphere_case(scale=2)
    op = O.OraclePool([case])
    out = {"case": "sphere at half resolution per axis (64x32x32 base, 3 levels, r=4)"}
    for k in steps:
        ref = op.fp64_steps(k)
        gp = Pool(ctx, [case])
        gp.step(k)
        f = gp.populations().astype(np.float64)
        gp.close()
        out["max_rel_after_%d_steps" % k] = float(np.max(np.abs(f - ref) / np.maximum(np.abs(ref), 1e-30)))
    return out


def full_run(ctx, steps=1000):
    """The sphere case as its configuration runs it: 1000 level-0 steps with a vorticity
    regrid every 25, from a fresh pool; wall time from the first step to the last
    (synchronised), every regrid included, and the mesh as the flow develops."""
    from fluidloom_gb300.lbm import Pool
    pool = Pool(ctx, [sphere_case()])
    ctx.sync()
    lups, peak_sites, trace = 0, 0, []
    t0 = time.perf_counter()
    for s in range(1, steps + 1):
        inf = pool.info()
        lups += inf.fluid_lups_per_step
        peak_sites = max(peak_sites, sum(int(inf.fluid_sites_per_level[l]) for l in range(4)))
        pool.step(1)
        if s % REGRID_EVERY == 0:
            pool.regrid()
        if s % 250 == 0:
            inf = pool.info()
            trace.append({"step": s, "bricks": int(inf.num_bricks),
                          "fluid_sites": sum(int(inf.fluid_sites_per_level[l]) for l in range(4))})
    ctx.sync()
    dt = time.perf_counter() - t0
    pool.close()
    return {"steps": steps, "regrids": steps // REGRID_EVERY, "wall_s": round(dt, 3),
            "mlups": round(lups / dt / 1e6, 1), "peak_fluid_sites": peak_sites, "mesh": trace}


def config1_run(ctx, cpu=True):
    """Configuration 1 as it is specified: the lid-driven cavity, 32^3 sites, max level 2,
    lid 0.05 in +x on the top z face, tau 0.56, 200 steps with a vorticity regrid every 20, from
    a fresh pool.  GPU: wall time from the first step to the last (synchronised), regrids
    included, and each regrid's CUDA-event time; CPU: the oracle (OpenMP over all host
    threads) on the same 200 steps and regrids."""
    from fluidloom_gb300.lbm import Pool, cavity
    case = cavity(32, 2, u_lid=0.05, tau=0.56)
    pool = Pool(ctx, [case])
    ctx.sync()
    lups, regrid_ms = 0, []
    t0 = time.perf_counter()
    for _ in range(10):  # 20 steps (one call: the mesh is fixed between regrids), then a regrid
        lups += 20 * pool.info().fluid_lups_per_step
        pool.step(20)
        stop = timer(ctx)
        pool.regrid()
        regrid_ms.append(stop())
    ctx.sync()
    dt = time.perf_counter() - t0
    inf = pool.info()
    out = {"workload": "lid-driven cavity 32^3, max level 2, lid 0.05, tau 0.56, 200 steps, regrid every 20",
           "gpu_mlups": round(lups / dt / 1e6, 1), "gpu_wall_s": round(dt, 4),
           "regrid_ms_per_cycle_median": round(float(np.median(regrid_ms)), 3),
           "regrid_ms_per_cycle_max": round(float(max(regrid_ms)), 3), "fluid_lups": int(lups),
           "final_bricks_per_level": [int(inf.bricks_per_level[l]) for l in range(3)]}
    pool.close()
    if cpu:
        from tests import _oracle as O
        threads = os.cpu_count() or 1
        op = O.OraclePool([case])
        cl = 0
        t0 = time.perf_counter()
        for _ in range(10):
            cl += 20 * op.lups()
            op.step(20, threads)
            op.regrid()
        out["cpu_mlups"] = round(cl / (time.perf_counter() - t0) / 1e6, 2)
        out["cpu"] = "oracle port, %d host threads, the same 200 steps and regrids" % threads
    return out


def cpu_sample(steps, threads=None):
    """The oracle (CPU port) on the workload itself (128x64x64 base, 3 levels, r=8): `steps` level-0 steps."""
    from tests import _oracle as O
    case = sphere_case()
    p = O.OraclePool([case])
    lups = p.lups()
    threads = threads or os.cpu_count() or 1
    t0 = time.perf_counter()
    p.step(steps, threads)
    dt = time.perf_counter() - t0
    return lups * steps / dt / 1e6, threads, lups


def run_gpu(args):
    import ctypes
    from fluidloom_gb300 import build as fbuild
    fbuild.build()
    import fluidloom_gb300 as fl
    from fluidloom_gb300.lbm import Pool
    from fluidloom_gb300.replicas import Replicas
    rep = Replicas()
    ws, rank, local = rep.world, rep.rank, rep.local
    ctx = fl.Context(local)
    pool = Pool(ctx, [sphere_case(args.scale)])
    if args.staging:
        pool.set_options(staging=args.staging)
    info0 = pool.info()
    # spin-up: the flow develops (and the vorticity regrids refine its wake) before anything is timed
    step_no = 0
    if args.spinup is None:  # the timed steps are the last of the configuration's 1000-step run
        args.spinup = max(0, RUN_STEPS - args.steps - args.warmup)
    for _ in range(args.spinup + args.warmup):
        pool.step(1)
        step_no += 1
        if step_no % REGRID_EVERY == 0:
            pool.regrid()
    ctx.sync()
    info = pool.info()
    bricks0 = info.num_bricks
    lups0 = info.fluid_lups_per_step
    rep.barrier()
    if args.profile_region:  # a profiler started with --profile-from-start off records from here on
        import torch
        torch.cuda.synchronize()
        torch.cuda.profiler.start()
    clocks = ClockSampler(local)
    clocks.start()
    total_lups = 0
    regrids = 0
    regrid_ms = []
    launches0 = ctx.launch_count()
    stop = timer(ctx)
    for k in range(args.steps):
        step_no += 1
        inf = pool.info()
        total_lups += inf.fluid_lups_per_step
        pool.step(1)
        if step_no % REGRID_EVERY == 0:
            pool.regrid()
            regrids += 1
    ms = stop()
    launches = ctx.launch_count() - launches0
    clk = clocks.stop()
    rep.barrier()
    ms_max = rep.max(ms)
    lups_all = rep.sum(float(total_lups))
    value = lups_all / (ms_max * 1e-3) / 1e6
    # regrid ms per cycle on this workload (one more regrid, timed alone)
    stop = timer(ctx)
    st = pool.regrid()
    regrid_ms.append(stop())
    # roofline: per-launch CUDA events around every collide-stream launch
    prof = pool.profile_steps(max(2, min(args.steps, 6)))
    kms = sum(p[0] for p in prof)
    nla = sum(p[1] for p in prof)
    sites = sum(p[2] for p in prof)
    peak, peak_kind = measured_peak()
    achieved = BYTES_PER_LUP * sites / (kms * 1e-3) / 1e9
    tr = ncu_traffic()
    per_kernel = {}
    for name, (m, la, st_) in zip(("k_collide_fast", "k_interface + k_collide_general", "k_collide_solid"), prof):
        if la:
            per_kernel[name] = {"launches": la, "avg_launch_ms": round(m / la, 4), "fluid_sites": int(st_),
                                "achieved_gbs": round(BYTES_PER_LUP * st_ / (m * 1e-3) / 1e9, 1),
                                "time_share": round(m / kms, 3)}
    nprof = max(2, min(args.steps, 6))
    lms, lla, lst = pool.profile_levels(nprof)
    per_level = []
    for l in range(16):
        for kk, name in enumerate(("interior", "general", "all-solid")):
            if lla[l, kk]:
                per_level.append({"level": l, "kernel": name, "ms_per_step": round(lms[l, kk] / nprof, 4),
                                  "launches_per_step": int(lla[l, kk]) // nprof,
                                  "achieved_gbs": round(BYTES_PER_LUP * lst[l, kk] / (lms[l, kk] * 1e-3) / 1e9, 1)})
    roofline = {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                "frac": round(achieved / peak, 4), "traffic": (round(tr * sites / nla) if tr else None),
                "traffic_source": ("not measured in this run: DRAM bytes per fluid site update from the committed "
                                   "ncu capture (profiles/collide_stream_sphere_ncu.md, dram__bytes_read.sum + "
                                   "dram__bytes_write.sum of one level-3 sub-step / its fluid sites) x the fluid "
                                   "sites per profiled launch" if tr else None),
                "kernel": "collide-stream (k_collide_fast + k_interface + k_collide_general + k_collide_solid)",
                "peak_source": peak_kind + " (MEASURED_PEAKS.json hbm_gbs)",
                "algorithmic_bytes_per_launch": round(BYTES_PER_LUP * sites / nla), "launches_profiled": nla,
                "avg_launch_ms": round(kms / nla, 4), "per_kernel": per_kernel, "per_level": per_level,
                # the timed steps themselves (dependency graph, regrids included): algorithmic
                # collide-stream bytes over the timed region
                "timed_region_achieved": round(value * 1e6 * BYTES_PER_LUP / 1e9, 1),
                "timed_region_frac": round(value * 1e6 * BYTES_PER_LUP / 1e9 / peak, 4)}
    if args.profile_region:
        import torch
        torch.cuda.synchronize()
        torch.cuda.profiler.stop()
    # e2e through the C ABI with pinned host buffers
    inf = pool.info()
    n = inf.num_bricks
    fbytes = 19 * n * 512 * 4
    hp = ctypes.c_void_p()
    ctx.call("fl_host_alloc_pinned", ctypes.c_size_t(fbytes), ctypes.byref(hp))
    hf = np.ctypeslib.as_array(ctypes.cast(hp, ctypes.POINTER(ctypes.c_float)), shape=(19, n, 512))
    ctx.call("fl_pool_download", pool.h, None, None, None, None, None, hp)
    vp = ctypes.c_void_p()
    ctx.call("fl_host_alloc_pinned", ctypes.c_size_t(64), ctypes.byref(vp))
    vel = np.ctypeslib.as_array(ctypes.cast(vp, ctypes.POINTER(ctypes.c_float)), shape=(2, 3))
    vel[:] = 0.0
    vel[1, 0] = 0.04
    # each step's conservation sums (mass, momentum; FP64) land in pinned host memory, one row per
    # step, copied asynchronously so the steps stay queued back to back
    cp = ctypes.c_void_p()
    ctx.call("fl_host_alloc_pinned", ctypes.c_size_t(max(args.steps, 1) * 32), ctypes.byref(cp))
    cons = np.ctypeslib.as_array(ctypes.cast(cp, ctypes.POINTER(ctypes.c_double)), shape=(max(args.steps, 1), 4))
    cons[:] = np.nan
    e2e_lups = 0
    # the caller reads the conservation sums every step: the steps write them as they go
    ctx.call("fl_pool_set_step_sums", pool.h, 1)
    # the steps after an upload replay graphs that also rewrite the all-solid bricks, the
    # steps after those the plain ones: capture all four (two level-0 parities each) first
    ctx.call("fl_pool_upload", pool.h, hp)
    pool.step(4)
    ctx.sync()
    rep.barrier()
    t0 = time.perf_counter()
    stop = timer(ctx)
    ctx.call("fl_pool_upload", pool.h, hp)
    ctx.sync()
    t_up = time.perf_counter()
    for k in range(args.steps):
        ctx.call("fl_pool_set_velocities", pool.h, vp, ctypes.c_void_p(vp.value + 12))
        e2e_lups += inf.fluid_lups_per_step
        pool.step(1)
        ctx.call("fl_pool_conservation_async", pool.h, ctypes.c_void_p(cp.value + 32 * k))
    ctx.sync()
    t_steps = time.perf_counter()
    ctx.call("fl_pool_download", pool.h, None, None, None, None, None, hp)
    e2e_ms = stop()
    e2e_wall = time.perf_counter() - t0
    e2e_phases = {"upload_ms": round((t_up - t0) * 1e3, 2), "steps_ms": round((t_steps - t_up) * 1e3, 2),
                  "download_ms": round((time.perf_counter() - t_steps) * 1e3, 2)}
    e2e_ms = max(e2e_ms, e2e_wall * 1e3)
    e2e_ms = rep.max(e2e_ms)
    e2e_value = rep.sum(float(e2e_lups)) / (e2e_ms * 1e-3) / 1e6
    h2d = (fbytes + args.steps * 24) / args.steps
    d2h = (fbytes + args.steps * 32) / args.steps
    # every step's sums arrived and are physical (mass positive and finite)
    if not (np.isfinite(cons[:args.steps]).all() and (cons[:args.steps, 0] > 0).all()):
        raise RuntimeError("e2e: a step's conservation read is missing or not finite")
    ctx.call("fl_host_free_pinned", hp)
    ctx.call("fl_host_free_pinned", vp)
    ctx.call("fl_host_free_pinned", cp)
    pool.close()
    full = None
    if rank == 0 and not args.no_full_run:
        full = full_run(ctx)
    cfg1 = None
    if rank == 0 and not args.no_config1:
        cfg1 = config1_run(ctx, cpu=not args.no_cpu)
    micro = None
    if rank == 0 and not args.no_microbench:
        micro = regrid_microbench(ctx)
    batch = None
    if rank == 0 and not args.no_batching:
        from fluidloom_gb300 import batching
        batch = batching.benchmark(ctx, batching.cavity_batch(256), 500, 20)
    serve = None
    if rank == 0 and not args.no_serving:
        from fluidloom_gb300 import serving
        serve = serving.benchmark(ctx, rate=50.0, duration=args.serving_seconds, steps_range=(200, 2000),
                                  budget_gb=150.0, check=8)
    cpu = None
    fp64 = None
    if rank == 0 and not args.no_cpu:
        v, th, sl = cpu_sample(2)
        cpu = {"value": round(v, 2), "unit": UNIT, "cores": th, "kind": "port",
               "sample": "CPU oracle (OpenMP, all host threads) on the same case (128x64x64 base, 3 levels, r=8; "
                         "%d fluid updates per step on its initial mesh), 2 level-0 steps" % sl}
        fp64 = fp64_error(ctx)
    if rank == 0:
        line = {"metric": METRIC, "value": round(value, 1), "unit": UNIT, "n_gpus": ws, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": round(ms_max / args.steps, 4), "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
                "config": workload_config({"timed_from_step": args.spinup + args.warmup + 1,
                                           "scale": args.scale, "staging": args.staging,
                                           "bricks": int(bricks0), "fluid_lups_per_step": int(lups0),
                                           "bricks_per_level": [int(info.bricks_per_level[l]) for l in range(4)],
                                           "fluid_sites_per_level": [int(info.fluid_sites_per_level[l]) for l in range(4)],
                                           "general_bricks_per_level": [int(info.general_bricks_per_level[l])
                                                                        for l in range(4)],
                                           "stencil_descriptors_per_level": [
                                               int(info.stencil_descriptors_per_level[l]) for l in range(4)],
                                           "initial_mesh": {"bricks": int(info0.num_bricks),
                                                            "fluid_lups_per_step": int(info0.fluid_lups_per_step)},
                                           "parallelism": "replicas" if ws > 1 else "single"}),
                "e2e": {"value": round(e2e_value, 1), "unit": UNIT, "h2d_bytes_per_step": int(h2d),
                        "d2h_bytes_per_step": int(d2h), "phases_wall": e2e_phases},
                "roofline": roofline, "cpu_baseline": cpu, "clocks": clk, "gpu_launches": int(launches),
                "regrid_ms_per_cycle": round(statistics.mean(regrid_ms), 3), "regrids_in_timed_region": regrids,
                "config1_cavity": cfg1, "config2_full_run": full, "regrid_microbench": micro, "batching": batch, "serving": serve,
                "fp32_vs_fp64": fp64}
        print(json.dumps(line))
    rep.close()


def run_reference(args):
    """The reference arm: the CPU implementation of the path (the oracle port; the reference's
    own OpenCL kernels cannot run on this host and it has no lattice-Boltzmann code) on the
    same workload as the GPU arm -- the full 128x64x64, 3-level sphere, a regrid every 25
    steps -- over all host threads.  K timed steps after W warm-up steps, at most 40 timed
    (about 1.2 s each on 16 host cores) so the run stays within minutes."""
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    from tests import _oracle as O
    p = O.OraclePool([sphere_case()])
    threads = os.cpu_count() or 1
    step_no = 0
    for _ in range(args.warmup):
        p.step(1, threads)
        step_no += 1
        if step_no % REGRID_EVERY == 0:
            p.regrid()
    k = min(args.steps, 40)
    lups = 0
    regrids = 0
    t0 = time.perf_counter()
    for _ in range(k):
        lups += p.lups()
        p.step(1, threads)
        step_no += 1
        if step_no % REGRID_EVERY == 0:
            p.regrid()
            regrids += 1
    dt = time.perf_counter() - t0
    value = lups / dt / 1e6
    sample = ("CPU restatement of the path (oracle/, OpenMP over all host threads; the reference has no "
              "lattice-Boltzmann code and its OpenCL kernels cannot run on this host) on the same workload: "
              "%d timed level-0 steps (of the %d asked) after %d warm-up steps, %d regrid(s) inside"
              % (k, args.steps, args.warmup, regrids))
    line = {"metric": METRIC, "value": round(value, 2), "unit": UNIT, "n_gpus": ws, "steps": k,
            "warmup": args.warmup, "ms_per_step": round(dt * 1e3 / k, 3), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic", "impl": "reference",
            "config": workload_config({"same_config": True}),
            "cpu_baseline": {"value": round(value, 2), "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": sample},
            "e2e": {"value": round(value, 2), "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gpu", choices=["gpu", "reference"])
    ap.add_argument("--no-microbench", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--spinup", type=int, default=None,
                    help="untimed level-0 steps (with regrids) before the warm-up; default: so that the timed "
                         "steps end at step 1000, the end of the configuration's run, where its mesh peaks")
    ap.add_argument("--no-full-run", action="store_true")
    ap.add_argument("--no-config1", action="store_true", help="skip the 32^3 cavity run of configuration 1")
    ap.add_argument("--scale", type=int, default=1, choices=[1, 2],
                    help="2 runs the sphere at half resolution per axis (profiling captures only; the "
                         "reported workload is scale 1)")
    ap.add_argument("--staging", type=int, default=0, choices=[0, 1, 2],
                    help="collide kernels' reads of a brick's own populations: 0 registers, 1 bulk copies into "
                         "shared memory, 2 also the general bricks' descriptor values (fl_pool_set_staging)")
    ap.add_argument("--profile-region", action="store_true",
                    help="bracket the timed steps, the regrid and the per-kernel profile passes with "
                         "cudaProfilerStart/Stop (for ncu --profile-from-start off)")
    ap.add_argument("--no-batching", action="store_true")
    ap.add_argument("--no-serving", action="store_true")
    ap.add_argument("--serving-seconds", type=float, default=2.0,
                    help="length of the Poisson arrival stream of the serving figure (the configuration's is 60 s)")
    ap.add_argument("--microbench-only", action="store_true",
                    help="run only the 2^24-leaf regrid microbench (one warm-up pass, one timed) and print it")
    ap.add_argument("--microbench-level", type=int, default=8,
                    help="level of the microbench's uniform start mesh (8: 2^24 leaves; 7 makes a small case)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.microbench_only:
        from fluidloom_gb300 import Context
        ctx = Context(0)
        regrid_microbench(ctx, L=args.microbench_level)
        print(json.dumps({"regrid_microbench": regrid_microbench(ctx, L=args.microbench_level)}))
        return
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
