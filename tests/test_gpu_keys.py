"""GPU key kernels through the C ABI vs the reference's known answers and the oracle."""
import ctypes
import os

import numpy as np
import pytest

from tests import _oracle as O

pytestmark = pytest.mark.gpu
GOLD = np.load(os.path.join(os.path.dirname(__file__), "golden", "hilbert_ref.npz"))


def _encode(ctx, x, y, z, level, with_ids=False):
    from fluidloom_gb300 import DeviceArray
    dx, dy, dz = (DeviceArray.from_host(ctx, np.ascontiguousarray(a, np.int32)) for a in (x, y, z))
    dk = DeviceArray(ctx, (len(x),), np.uint64)
    di = DeviceArray(ctx, (len(x),), np.uint32) if with_ids else None
    ctx.call("fl_hilbert_encode", dx.ptr, dy.ptr, dz.ptr, level, dk.ptr, di.ptr if di else None, len(x))
    return (dk.to_host(), di.to_host()) if with_ids else dk.to_host()


def test_encode_matches_reference_kats(ctx):
    for sec in ["corners_l1", "roundtrip_l1_8", "canonical", "parent_child", "l21_random", "all_levels"]:
        xyz, lv, key = GOLD[sec + "_xyz"], GOLD[sec + "_level"], GOLD[sec + "_key"]
        for level in np.unique(lv):
            m = lv == level
            got = _encode(ctx, xyz[m, 0], xyz[m, 1], xyz[m, 2], int(level))
            np.testing.assert_array_equal(got, key[m], err_msg=sec)


@pytest.mark.parametrize("level", list(range(0, 22)))
def test_encode_random_vs_oracle(ctx, level):
    rng = np.random.default_rng(level)
    n = 300_001
    x, y, z = (rng.integers(-2**31, 2**31, n, dtype=np.int64).astype(np.int32) for _ in range(3))
    got, ids = _encode(ctx, x, y, z, level, with_ids=True)
    np.testing.assert_array_equal(got, O.hilbert_encode(x, y, z, level))
    np.testing.assert_array_equal(ids, np.arange(n, dtype=np.uint32))


@pytest.mark.parametrize("level", [1, 2, 3, 5, 8, 13, 20, 21])
def test_decode_roundtrip(ctx, level):
    from fluidloom_gb300 import DeviceArray
    rng = np.random.default_rng(100 + level)
    n = 200_003
    x, y, z = (rng.integers(0, 1 << level, n).astype(np.int32) for _ in range(3))
    k = O.hilbert_encode(x, y, z, level)
    dk = DeviceArray.from_host(ctx, k)
    ox, oy, oz = (DeviceArray(ctx, (n,), np.int32) for _ in range(3))
    ctx.call("fl_hilbert_decode", dk.ptr, level, ox.ptr, oy.ptr, oz.ptr, n)
    np.testing.assert_array_equal(ox.to_host(), x)
    np.testing.assert_array_equal(oy.to_host(), y)
    np.testing.assert_array_equal(oz.to_host(), z)


def test_morton8(ctx):
    from fluidloom_gb300 import DeviceArray
    xyz, key = GOLD["morton8_xyz"], GOLD["morton8_key"]
    rng = np.random.default_rng(3)
    extra = rng.integers(-2**31, 2**31, (100000, 3), dtype=np.int64).astype(np.int32)
    allxyz = np.concatenate([xyz, extra])
    d = [DeviceArray.from_host(ctx, np.ascontiguousarray(allxyz[:, i])) for i in range(3)]
    dk = DeviceArray(ctx, (len(allxyz),), np.uint64)
    ctx.call("fl_morton8_encode", d[0].ptr, d[1].ptr, d[2].ptr, dk.ptr, len(allxyz))
    got = dk.to_host()
    np.testing.assert_array_equal(got[:len(xyz)], key)
    np.testing.assert_array_equal(got, O.morton8(allxyz[:, 0], allxyz[:, 1], allxyz[:, 2]))


def test_cell_keys_with_case(ctx):
    from fluidloom_gb300 import DeviceArray
    rng = np.random.default_rng(9)
    n = 100000
    lv = rng.integers(0, 9, n).astype(np.uint8)
    x, y, z = (rng.integers(0, 16 << lv.astype(np.int64)).astype(np.int32) for _ in range(3))
    cs = rng.integers(0, 4096, n).astype(np.uint16)
    want = O.cell_keys(x, y, z, lv, cs, 17, 13)
    d = [DeviceArray.from_host(ctx, a) for a in (x, y, z, lv, cs)]
    dk = DeviceArray(ctx, (n,), np.uint64)
    ctx.call("fl_cell_keys", d[0].ptr, d[1].ptr, d[2].ptr, d[3].ptr, d[4].ptr, 17, 13, dk.ptr, n)
    np.testing.assert_array_equal(dk.to_host(), want)


def test_empty_and_invalid(ctx):
    ctx.call("fl_hilbert_encode", None, None, None, 8, None, None, 0)  # n = 0 is a no-op
    from fluidloom_gb300 import FluidLoomError
    with pytest.raises(FluidLoomError):
        ctx.call("fl_hilbert_encode", None, None, None, 8, None, None, 5)
