"""GPU scan / sort / compaction / hash / neighbour kernels vs the oracle."""
import ctypes

import numpy as np
import pytest

from tests import _oracle as O

pytestmark = pytest.mark.gpu


def D(ctx, a):
    from fluidloom_gb300 import DeviceArray
    return DeviceArray.from_host(ctx, a)


def E(ctx, shape, dt):
    from fluidloom_gb300 import DeviceArray
    return DeviceArray(ctx, shape, dt)


@pytest.mark.parametrize("n", [0, 1, 7, 4095, 4096, 4097, 65536, 65537, 1_000_003, 16_777_216])
def test_scan(ctx, n):
    rng = np.random.default_rng(n)
    a = rng.integers(0, 1000, n).astype(np.uint32)
    da = D(ctx, a)
    do = E(ctx, (max(n, 1),), np.uint32)
    tot = E(ctx, (1,), np.uint32)
    ctx.call("fl_scan_exclusive_u32", da.ptr, do.ptr, n, tot.ptr)
    want = np.empty(n, np.uint32)
    t = O.load().or_scan_exclusive_u32(O.ptr(a), O.ptr(want), n)
    if n:
        np.testing.assert_array_equal(do.to_host()[:n], want)
    assert int(tot.to_host()[0]) == t


def test_scan_in_place_wraps(ctx):
    a = np.full(300_000, 0xFFFFFFF0, np.uint32)
    da = D(ctx, a)
    ctx.call("fl_scan_exclusive_u32", da.ptr, da.ptr, len(a), None)
    want = np.empty_like(a)
    O.load().or_scan_exclusive_u32(O.ptr(a), O.ptr(want), len(a))
    np.testing.assert_array_equal(da.to_host(), want)


def test_scan_unaligned_pointers(ctx):
    """Input and output not 16-byte aligned: the per-item path of every tile."""
    n = 100_003
    a = np.random.default_rng(5).integers(0, 1000, n + 1).astype(np.uint32)
    da = D(ctx, a)
    do = E(ctx, (n + 2,), np.uint32)
    tot = E(ctx, (1,), np.uint32)
    ctx.call("fl_scan_exclusive_u32", ctypes.c_void_p(da.ptr.value + 4), ctypes.c_void_p(do.ptr.value + 8), n,
             tot.ptr)
    src = np.ascontiguousarray(a[1:])
    want = np.empty(n, np.uint32)
    t = O.load().or_scan_exclusive_u32(O.ptr(src), O.ptr(want), n)
    np.testing.assert_array_equal(do.to_host()[2:], want)
    assert int(tot.to_host()[0]) == t


def _sort(ctx, k, v, b0=0, b1=64):
    dk, dv = D(ctx, k), D(ctx, v)
    ctx.call("fl_sort_pairs_u64_u32", dk.ptr, dv.ptr, len(k), b0, b1)
    return dk.to_host(), dv.to_host()


@pytest.mark.parametrize("n", [0, 1, 2, 3071, 3072, 3073, 100_000, 1_048_577])
def test_sort_random_u64(ctx, n):
    rng = np.random.default_rng(n + 1)
    k = rng.integers(0, 2**63, n, dtype=np.uint64) * 2 + rng.integers(0, 2, n).astype(np.uint64)
    v = np.arange(n, dtype=np.uint32)
    gk, gv = _sort(ctx, k, v)
    wk, wv = k.copy(), v.copy()
    O.load().or_sort_pairs_u64_u32(O.ptr(wk), O.ptr(wv), n)
    np.testing.assert_array_equal(gk, wk)
    np.testing.assert_array_equal(gv, wv)


def test_sort_stable_with_ties(ctx):
    rng = np.random.default_rng(7)
    n = 500_000
    k = rng.integers(0, 50, n).astype(np.uint64) << np.uint64(40)
    v = rng.integers(0, 2**32, n, dtype=np.uint64).astype(np.uint32)
    gk, gv = _sort(ctx, k, v)
    wk, wv = k.copy(), v.copy()
    O.load().or_sort_pairs_u64_u32(O.ptr(wk), O.ptr(wv), n)
    np.testing.assert_array_equal(gk, wk)
    np.testing.assert_array_equal(gv, wv)
    ak, av = _sort(ctx, np.full(10000, 5, np.uint64), np.arange(10000, dtype=np.uint32))
    np.testing.assert_array_equal(av, np.arange(10000, dtype=np.uint32))


def test_sort_bit_range(ctx):
    rng = np.random.default_rng(3)
    n = 200_000
    k = rng.integers(0, 2**63, n, dtype=np.uint64)
    v = np.arange(n, dtype=np.uint32)
    gk, gv = _sort(ctx, k, v, 0, 63)
    order = np.argsort(k & np.uint64((1 << 63) - 1), kind="stable")
    np.testing.assert_array_equal(gv, v[order])


def test_sort_hilbert_keys_16m_sorted_and_permutation(ctx):
    """Full-size property check (16.7M 63-bit keys): ascending and a permutation of the input."""
    from fluidloom_gb300 import DeviceArray
    n = 1 << 24
    rng = np.random.default_rng(11)
    x, y, z = (rng.integers(0, 1 << 21, n).astype(np.int32) for _ in range(3))
    d = [DeviceArray.from_host(ctx, a) for a in (x, y, z)]
    dk, di = E(ctx, (n,), np.uint64), E(ctx, (n,), np.uint32)
    ctx.call("fl_hilbert_encode", d[0].ptr, d[1].ptr, d[2].ptr, 21, dk.ptr, di.ptr, n)
    k0 = dk.to_host()
    ctx.call("fl_sort_pairs_u64_u32", dk.ptr, di.ptr, n, 0, 63)
    k, i = dk.to_host(), di.to_host()
    assert (k[1:] >= k[:-1]).all()
    np.testing.assert_array_equal(k0[i], k)
    assert np.bincount(i, minlength=n).max() == 1


SORT_SHAPES = [(8, 256), (8, 512), (9, 256), (9, 512)]


@pytest.fixture
def sort_shape(ctx, request):
    """Set the context's radix sort shape for one test; the default shape afterwards."""
    ctx.call("fl_sort_set_config", *request.param)
    yield request.param
    ctx.call("fl_sort_set_config", 8, 256)


@pytest.mark.parametrize("sort_shape", SORT_SHAPES, indirect=True)
@pytest.mark.parametrize("n,b0,b1", [(0, 0, 64), (1, 0, 64), (6143, 0, 64), (6144, 0, 63), (6145, 5, 29),
                                      (300_001, 0, 64), (300_001, 0, 63), (70_000, 0, 3), (70_000, 55, 64)])
def test_sort_shapes_equal_stable_sort(ctx, sort_shape, n, b0, b1):
    """Every sort shape (digit width x tile threads) gives the stable order of the key bits
    [b0, b1): ragged tiles, one-digit and odd-width ranges, the top bits."""
    rng = np.random.default_rng(n + b0 + 7 * b1)
    k = rng.integers(0, 2**63, n, dtype=np.uint64) * 2 + rng.integers(0, 2, n).astype(np.uint64)
    v = np.arange(n, dtype=np.uint32)
    gk, gv = _sort(ctx, k, v, b0, b1)
    mask = np.uint64(((1 << (b1 - b0)) - 1) << b0) if b1 - b0 < 64 else np.uint64(0xFFFFFFFFFFFFFFFF)
    order = np.argsort(k & mask, kind="stable")
    np.testing.assert_array_equal(gv, v[order])
    np.testing.assert_array_equal(gk, k[order])


@pytest.mark.parametrize("sort_shape", SORT_SHAPES[1:], indirect=True)
def test_sort_shapes_ties_and_full_size(ctx, sort_shape):
    """Ties keep input order in every shape; 2^24 Hilbert keys equal the oracle's stable sort."""
    rng = np.random.default_rng(19)
    n = 400_000
    k = rng.integers(0, 700, n).astype(np.uint64) << np.uint64(30)
    v = rng.integers(0, 2**32, n, dtype=np.uint64).astype(np.uint32)
    gk, gv = _sort(ctx, k, v)
    wk, wv = k.copy(), v.copy()
    O.load().or_sort_pairs_u64_u32(O.ptr(wk), O.ptr(wv), n)
    np.testing.assert_array_equal(gk, wk)
    np.testing.assert_array_equal(gv, wv)
    from fluidloom_gb300 import DeviceArray
    n = 1 << 24
    x, y, z = (rng.integers(0, 1 << 21, n).astype(np.int32) for _ in range(3))
    d = [DeviceArray.from_host(ctx, a) for a in (x, y, z)]
    dk, di = E(ctx, (n,), np.uint64), E(ctx, (n,), np.uint32)
    ctx.call("fl_hilbert_encode", d[0].ptr, d[1].ptr, d[2].ptr, 21, dk.ptr, di.ptr, n)
    wk, wv = dk.to_host(), di.to_host()
    ctx.call("fl_sort_pairs_u64_u32", dk.ptr, di.ptr, n, 0, 63)
    O.load().or_sort_pairs_u64_u32(O.ptr(wk), O.ptr(wv), n)
    np.testing.assert_array_equal(dk.to_host(), wk)
    np.testing.assert_array_equal(di.to_host(), wv)


def test_sort_shape_validation(ctx):
    from fluidloom_gb300.runtime import FluidLoomError
    for bad in [(7, 256), (10, 512), (9, 384), (8, 384), (8, 0)]:
        with pytest.raises(FluidLoomError):
            ctx.call("fl_sort_set_config", *bad)
    b, t = ctypes.c_int(), ctypes.c_int()
    ctx.call("fl_sort_get_config", ctypes.byref(b), ctypes.byref(t))
    assert (b.value, t.value) == (8, 256)


@pytest.mark.parametrize("sort_shape", SORT_SHAPES[1:], indirect=True)
def test_sort_shapes_inside_compaction(ctx, sort_shape):
    """The compaction's sort runs in the context's shape: same survivors, order and permutation."""
    rng = np.random.default_rng(23)
    n = 250_000
    keys = rng.integers(0, 2**62, n, dtype=np.uint64)
    keys[rng.integers(0, n, 1000)] = np.uint64(0xFFFFFFFFFFFFFFFF)
    state = rng.integers(0, 2, n).astype(np.uint32)
    dk, ds = D(ctx, keys), D(ctx, state)
    perm, sk, si = E(ctx, (n,), np.uint32), E(ctx, (n,), np.uint64), E(ctx, (n,), np.uint32)
    nv = ctypes.c_size_t()
    ctx.call("fl_compact_and_permute", dk.ptr, ds.ptr, n, perm.ptr, sk.ptr, si.ptr, ctypes.byref(nv))
    keep = np.nonzero((state != 0) & (keys != np.uint64(0xFFFFFFFFFFFFFFFF)))[0]
    order = keep[np.argsort(keys[keep], kind="stable")]
    m = nv.value
    assert m == len(order)
    np.testing.assert_array_equal(sk.to_host()[:m], keys[order])
    np.testing.assert_array_equal(si.to_host()[:m], order.astype(np.uint32))
    want = np.full(n, 0xFFFFFFFF, np.uint32)
    want[order] = np.arange(m, dtype=np.uint32)
    np.testing.assert_array_equal(perm.to_host(), want)


def test_compact_and_permute(ctx):
    # test_hash_table.cpp:54-116 cases plus a random one
    cases = [(np.arange(10, dtype=np.uint64) * 100, (np.arange(10) % 2).astype(np.uint32)),
             (np.array([100, 50, 200, 25], np.uint64), np.ones(4, np.uint32)),
             (np.array([100, 200, 300], np.uint64), np.zeros(3, np.uint32))]
    rng = np.random.default_rng(0)
    k = rng.integers(0, 2**40, 300_000, dtype=np.uint64)
    k[::17] = np.uint64(0xFFFFFFFFFFFFFFFF)
    cases.append((k, rng.integers(0, 2, len(k)).astype(np.uint32)))
    for keys, state in cases:
        n = len(keys)
        dk, ds = D(ctx, keys), D(ctx, state)
        perm, sk, si = E(ctx, (n,), np.uint32), E(ctx, (n,), np.uint64), E(ctx, (n,), np.uint32)
        nv = ctypes.c_size_t()
        ctx.call("fl_compact_and_permute", dk.ptr, ds.ptr, n, perm.ptr, sk.ptr, si.ptr, ctypes.byref(nv))
        want = np.empty(n, np.uint32)
        m = O.load().or_compact_and_permute(O.ptr(keys), O.ptr(state), n, O.ptr(want))
        assert nv.value == m
        np.testing.assert_array_equal(perm.to_host(), want)


def test_apply_permutation(ctx):
    rng = np.random.default_rng(1)
    n = 100_000
    perm = rng.permutation(n).astype(np.uint32)
    perm[::5] = 0xFFFFFFFF
    for dt in (np.uint8, np.float32, np.float64):
        src = rng.random(n).astype(dt) if dt != np.uint8 else rng.integers(0, 255, n).astype(np.uint8)
        ds, dd = D(ctx, src), D(ctx, np.zeros(n, dt))
        dp = D(ctx, perm)  # keep every device buffer referenced until the call returns
        ctx.call("fl_apply_permutation", ds.ptr, dd.ptr, np.dtype(dt).itemsize, n, dp.ptr)
        want = np.zeros(n, dt)
        O.load().or_apply_permutation(O.ptr(src), O.ptr(want), np.dtype(dt).itemsize, n, O.ptr(perm))
        np.testing.assert_array_equal(dd.to_host(), want)


@pytest.mark.parametrize("n", [0, 5, 10000, 2_000_000])
def test_hash_build_query(ctx, n):
    L = ctx.lib
    cap = L.fl_hash_compute_capacity(n)
    assert cap == O.load().or_hash_capacity(n)
    assert cap & (cap - 1) == 0 and cap >= n / 0.6
    rng = np.random.default_rng(n)
    keys = rng.integers(0, 2**63, n, dtype=np.uint64)
    if n > 10:
        keys[5] = keys[3]  # duplicate: the last occurrence wins
    vals = rng.integers(0, 2**31, n).astype(np.uint32)
    tk, tv = E(ctx, (cap,), np.uint64), E(ctx, (cap,), np.uint32)
    dk = D(ctx, keys) if n else None  # keep every device buffer referenced until the call returns
    dv = D(ctx, vals) if n else None
    ctx.call("fl_hash_build", tk.ptr, tv.ptr, ctypes.c_uint64(cap), dk.ptr if n else None, dv.ptr if n else None, n)
    q = np.concatenate([keys, rng.integers(0, 2**63, 1000, dtype=np.uint64),
                        np.array([0xFFFFFFFFFFFFFFFF], np.uint64)])
    out = E(ctx, (len(q),), np.uint32)
    dq = D(ctx, q)
    ctx.call("fl_hash_query", tk.ptr, tv.ptr, ctypes.c_uint64(cap), dq.ptr, out.ptr, len(q))
    otk, otv = np.empty(cap, np.uint64), np.empty(cap, np.uint32)
    L2 = O.load()
    assert L2.or_hash_build(O.ptr(keys), O.ptr(vals), n, cap, O.ptr(otk), O.ptr(otv)) == 0
    want = np.empty(len(q), np.uint32)
    L2.or_hash_query(O.ptr(otk), O.ptr(otv), cap, O.ptr(q), O.ptr(want), len(q))
    np.testing.assert_array_equal(out.to_host(), want)


def test_hash_constants(ctx):
    # test_hash_table.cpp:30-51
    assert ctx.lib.fl_hash_compute_capacity(10) == 1 << 20
    assert ctx.lib.fl_hash_compute_capacity(10**8) == 1 << 28
