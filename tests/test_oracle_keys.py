"""Oracle key codecs vs the reference's own codec (golden vectors and, where the
reference tree is present, the codec compiled in place)."""
import ctypes
import os

import numpy as np
import pytest

from tests import _oracle as O

GOLD = np.load(os.path.join(os.path.dirname(__file__), "golden", "hilbert_ref.npz"))
REF_SO = os.path.join(os.path.dirname(os.path.dirname(__file__)), "oracle", "_ref", "libfl_ref_codec.so")


def _enc_levels(xyz, levels):
    out = np.empty(len(levels), np.uint64)
    for lv in np.unique(levels):
        m = levels == lv
        out[m] = O.hilbert_encode(xyz[m, 0], xyz[m, 1], xyz[m, 2], int(lv))
    return out


@pytest.mark.parametrize("section", ["corners_l1", "roundtrip_l1_8", "canonical", "parent_child",
                                     "l21_random", "all_levels"])
def test_oracle_encode_matches_reference_kat(section):
    xyz, lv, key = GOLD[section + "_xyz"], GOLD[section + "_level"], GOLD[section + "_key"]
    np.testing.assert_array_equal(_enc_levels(xyz, lv), key)


def test_known_sequence_level1():
    # test_hilbert_codec.cpp:33-58: (0,0,0) -> 0 and the 8 corners take keys 0..7
    assert O.hilbert_encode([0], [0], [0], 1)[0] == 0
    assert sorted(GOLD["corners_l1_key"].tolist()) == list(range(8))


def test_roundtrip_all_levels():
    # test_hilbert_codec.cpp:72-92: decode(encode(c)) == c for levels 1..8
    xyz, lv, key = GOLD["roundtrip_l1_8_xyz"], GOLD["roundtrip_l1_8_level"], GOLD["roundtrip_l1_8_key"]
    for level in range(1, 9):
        m = lv == level
        x, y, z = O.hilbert_decode(key[m], level)
        np.testing.assert_array_equal(np.stack([x, y, z], 1), xyz[m])


def test_roundtrip_21():
    xyz, key = GOLD["l21_random_xyz"], GOLD["l21_random_key"]
    x, y, z = O.hilbert_decode(key, 21)
    np.testing.assert_array_equal(np.stack([x, y, z], 1), xyz)
    assert int(key.max()) < (1 << 63)


def test_parent_is_shift():
    # test_hilbert_codec.cpp:108-125: getParent(child key) == parent key (key >> 3)
    k = GOLD["parent_child_key"]
    assert all(int(c) >> 3 == int(k[0]) for c in k[1:])


def test_morton8_matches_reference():
    xyz, key = GOLD["morton8_xyz"], GOLD["morton8_key"]
    np.testing.assert_array_equal(O.morton8(xyz[:, 0], xyz[:, 1], xyz[:, 2]), key)


@pytest.mark.skipif(not os.path.exists(REF_SO), reason="reference codec not built here")
def test_oracle_exhaustive_vs_reference_build():
    ref = ctypes.CDLL(REF_SO)
    P = ctypes.c_void_p
    for L in range(0, 6):
        n = 1 << L
        g = np.stack(np.meshgrid(*[np.arange(n, dtype=np.int32)] * 3, indexing="ij"), -1).reshape(-1, 3)
        x, y, z = (np.ascontiguousarray(g[:, i]) for i in range(3))
        want = np.empty(len(x), np.uint64)
        ref.ref_hilbert_encode(O.ptr(x), O.ptr(y), O.ptr(z), ctypes.c_uint8(L), O.ptr(want), ctypes.c_size_t(len(x)))
        np.testing.assert_array_equal(O.hilbert_encode(x, y, z, L), want)
        if L >= 1:
            assert sorted(want.tolist()) == list(range(n ** 3))  # bijection
    rng = np.random.default_rng(5)
    x, y, z = (rng.integers(-2**31, 2**31, 200000, dtype=np.int64).astype(np.int32) for _ in range(3))
    want = np.empty(len(x), np.uint64)
    ref.ref_morton8_encode(O.ptr(x), O.ptr(y), O.ptr(z), O.ptr(want), ctypes.c_size_t(len(x)))
    np.testing.assert_array_equal(O.morton8(x, y, z), want)
    for lv in (8, 13, 21):
        want = np.empty(len(x), np.uint64)
        ref.ref_hilbert_encode(O.ptr(x), O.ptr(y), O.ptr(z), ctypes.c_uint8(lv), O.ptr(want), ctypes.c_size_t(len(x)))
        np.testing.assert_array_equal(O.hilbert_encode(x, y, z, lv), want)


def test_cell_keys_definition():
    rng = np.random.default_rng(1)
    lv = rng.integers(0, 9, 1000).astype(np.uint8)
    x, y, z = (np.array([rng.integers(0, 1 << int(l)) for l in lv], np.int32) for _ in range(3))
    k = O.cell_keys(x, y, z, lv, None, 21, 21)
    sh = (21 - lv.astype(np.int64))
    want = O.hilbert_encode((x.astype(np.int64) << sh).astype(np.int32), (y.astype(np.int64) << sh).astype(np.int32),
                            (z.astype(np.int64) << sh).astype(np.int32), 21)
    np.testing.assert_array_equal(k, want)
