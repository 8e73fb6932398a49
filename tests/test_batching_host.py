"""Host logic of the autotuners (no GPU): a fake context stands in for the C ABI and
reports scripted CUDA-event times, and the tests check what each tuner tries, what it
keeps and what it leaves set."""
import ctypes

import numpy as np

from fluidloom_gb300 import batching


class FakeCtx:
    """Records the calls autotune_sort makes; fl_ctx_timer_stop returns the time scripted
    for the sort shape currently set."""

    def __init__(self, ms_by_shape):
        self.ms = ms_by_shape
        self.shape = (8, 256)
        self.calls = []
        self.live = set()
        self.next_ptr = 0x1000

    def call(self, name, *args):
        self.calls.append(name)
        if name == "fl_device_alloc":
            ctypes.cast(args[1], ctypes.POINTER(ctypes.c_void_p))[0] = self.next_ptr
            self.live.add(self.next_ptr)
            self.next_ptr += 0x1000
        elif name == "fl_device_free":
            self.live.discard(args[0].value if isinstance(args[0], ctypes.c_void_p) else args[0])
        elif name == "fl_sort_set_config":
            self.shape = (args[0], args[1])
        elif name == "fl_ctx_timer_stop":
            ctypes.cast(args[0], ctypes.POINTER(ctypes.c_float))[0] = self.ms[self.shape]
        return 0


def test_autotune_sort_times_every_shape_and_keeps_the_fastest():
    ms = {(8, 256): 1.17, (8, 512): 1.22, (9, 256): 1.56, (9, 512): 1.15}
    ctx = FakeCtx(ms)
    keys = np.arange(1000, dtype=np.uint64)[::-1].copy()
    ids = np.arange(1000, dtype=np.uint32)
    choice, times = batching.autotune_sort(ctx, keys, ids, 0, 63, reps=3)
    assert choice == (9, 512) and ctx.shape == (9, 512)
    assert set(times) == set(batching.SORT_SHAPES)
    assert all(abs(times[s] - ms[s]) < 1e-6 for s in times)  # the c_float round trip
    # per shape: one untimed and three timed sorts, each on a fresh copy of the input
    assert ctx.calls.count("fl_sort_pairs_u64_u32") == 4 * len(batching.SORT_SHAPES)
    assert ctx.calls.count("fl_memcpy_h2d") == 2 + 2 * 4 * len(batching.SORT_SHAPES)
    assert not ctx.live  # its two device buffers are freed


def test_autotune_sort_default_shape_when_fastest():
    ms = {(8, 256): 1.0, (8, 512): 1.2, (9, 256): 1.5, (9, 512): 1.1}
    ctx = FakeCtx(ms)
    choice, _ = batching.autotune_sort(ctx, np.zeros(10, np.uint64), np.zeros(10, np.uint32), reps=1)
    assert choice == (8, 256) and ctx.shape == (8, 256)


class FakePool:
    """A pool whose graph-replayed steps take the time scripted for its current options."""

    def __init__(self, ms_of):
        self.ms_of = ms_of
        self.opts = None
        self.tried = []
        outer = self

        class Ctx:
            def call(self, name, *args):
                if name == "fl_ctx_timer_stop":
                    ctypes.cast(args[0], ctypes.POINTER(ctypes.c_float))[0] = outer.ms_of(*outer.opts)
                return 0

        self.ctx = Ctx()

    def set_options(self, graphs=1, grid_mult=0, streams=None, staging=None, step_sums=None):
        self.opts = (grid_mult, streams, staging)
        self.tried.append(self.opts)

    def step(self, n):
        pass


def test_autotune_pool_options():
    # fastest: 4 CTAs per SM on two streams with register loads; staging is tried only there
    def ms_of(g, st, sg):
        return abs(g - 4) + (0.5 if st == 1 else 0.0) + 0.3 * sg + 1.0

    pool = FakePool(ms_of)
    best = batching.autotune(pool, candidates=(2, 3, 4, 6, 8), streams=(1, 2), staging=(0, 1, 2), steps=4)
    assert best == (4, 2, 0)
    assert pool.opts == (4, 2, 0)  # left set on the pool
    grid = [(g, st, 0) for st in (1, 2) for g in (2, 3, 4, 6, 8)]
    assert pool.tried[:len(grid)] == grid
    assert pool.tried[len(grid):len(grid) + 2] == [(4, 2, 1), (4, 2, 2)]


def test_autotune_pool_picks_staging_when_faster():
    pool = FakePool(lambda g, st, sg: {0: 2.0, 1: 1.5, 2: 1.7}[sg] + 0.01 * g + (0.1 if st == 2 else 0))
    best = batching.autotune(pool, candidates=(2, 4), streams=(1, 2), staging=(0, 1, 2))
    assert best == (2, 1, 1) and pool.opts == (2, 1, 1)


def test_autotune_cache_skips_tuned_workloads(tmp_path):
    cache = str(tmp_path / "tune.json")
    first = FakePool(lambda g, st, sg: abs(g - 4) + (0.5 if st == 1 else 0.0) + 0.3 * sg + 1.0)
    assert batching.autotune(first, candidates=(2, 4, 8), cache=cache, key="wl") == (4, 2, 0)
    # the same workload again, on a GPU that would now prefer 8 CTAs per SM: the recorded
    # choice is set without timing anything
    second = FakePool(lambda g, st, sg: abs(g - 8) + 1.0)
    assert batching.autotune(second, candidates=(2, 4, 8), cache=cache, key="wl") == (4, 2, 0)
    assert second.tried == [(4, 2, 0)]
    # another workload is tuned and recorded beside it
    third = FakePool(lambda g, st, sg: abs(g - 8) + 1.0)
    assert batching.autotune(third, candidates=(2, 4, 8), staging=(0,), cache=cache, key="other")[0] == 8
    import json
    assert set(json.load(open(cache))["pool"]) == {"wl", "other"}


def test_autotune_sort_cache(tmp_path):
    cache = str(tmp_path / "tune.json")
    keys, ids = np.arange(5000, dtype=np.uint64), np.arange(5000, dtype=np.uint32)
    ctx = FakeCtx({(8, 256): 1.0, (8, 512): 1.2, (9, 256): 1.5, (9, 512): 0.9})
    assert batching.autotune_sort(ctx, keys, ids, 0, 63, cache=cache)[0] == (9, 512)
    ctx2 = FakeCtx({(8, 256): 0.5, (8, 512): 1.2, (9, 256): 1.5, (9, 512): 0.9})
    choice, times = batching.autotune_sort(ctx2, keys, ids, 0, 63, cache=cache)
    assert choice == (9, 512) and times == {} and ctx2.shape == (9, 512)
    assert "fl_sort_pairs_u64_u32" not in ctx2.calls


def test_pool_signature():
    import types
    from fluidloom_gb300.lbm import PoolInfo
    inf = PoolInfo()
    inf.num_cases, inf.max_level = 3, 2
    for l, n in enumerate((48, 100, 224)):
        inf.bricks_per_level[l] = n
    pool = types.SimpleNamespace(info=lambda: inf)
    assert batching.pool_signature(pool) == "cases=3 bricks=48,100,224"
