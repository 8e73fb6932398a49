"""Field descriptors, registry (host) and SOA manager (device) — the reference's
tests/unit/fields/test_field_manager.cpp cases."""
import ctypes

import pytest

from fluidloom_gb300 import _capi


class FieldDesc(ctypes.Structure):
    _fields_ = [("name", ctypes.c_char * 72), ("type", ctypes.c_int32), ("num_components", ctypes.c_uint16),
                ("halo_depth", ctypes.c_uint8), ("avg_rule", ctypes.c_uint8), ("solid_scheme", ctypes.c_uint8),
                ("reserved", ctypes.c_uint8 * 7), ("id", ctypes.c_uint64)]


def make(name, t=0, c=1, halo=0):
    d = FieldDesc()
    st = _capi.lib().fl_field_make(name, t, c, halo, 0, 0, ctypes.byref(d))
    return st, d


def fnv(s):
    h = 14695981039346656037
    for b in s.encode():
        h ^= b
        h = (h * 1099511628211) & 0xFFFFFFFFFFFFFFFF
    return h


def test_descriptor_construction_and_validation():
    st, d = make(b"density")
    assert st == 0 and d.num_components == 1 and d.halo_depth == 0 and d.id == fnv("density")
    st, d = make(b"velocity", c=3, halo=1)
    assert st == 0 and d.num_components == 3 and d.halo_depth == 1
    assert make(b"")[0] != 0                      # InvalidNameEmpty
    assert make(b"x" * 65)[0] != 0                # InvalidNameTooLong
    assert make(b"f", c=0)[0] != 0                # InvalidComponentsZero
    assert make(b"f", c=33)[0] != 0               # InvalidComponentsTooMany
    assert make(b"f", halo=3)[0] != 0             # InvalidHaloDepth
    L = _capi.lib()
    for t, c, want in ((0, 1, 4), (1, 1, 8), (0, 3, 12), (4, 1, 1)):   # BytesPerCell
        st, d = make(b"b", t=t, c=c)
        assert L.fl_field_bytes_per_cell(ctypes.byref(d)) == want
    assert make(b"a1")[1].id != make(b"a2")[1].id and make(b"a1")[1].id == make(b"a1")[1].id  # UniqueIDs


def test_registry():
    L = _capi.lib()
    L.fl_field_registry_clear()
    st, d = make(b"test_field_1", c=2)
    assert L.fl_field_register(ctypes.byref(d)) == 0
    assert L.fl_field_register(ctypes.byref(d)) != 0   # duplicate name
    out = FieldDesc()
    assert L.fl_field_lookup_name(b"test_field_1", ctypes.byref(out)) == 0 and out.num_components == 2
    assert L.fl_field_lookup_id(ctypes.c_uint64(d.id), ctypes.byref(out)) == 0 and out.name == b"test_field_1"
    assert L.fl_field_lookup_name(b"missing", ctypes.byref(out)) != 0
    assert L.fl_field_registry_count() == 1
    L.fl_field_registry_clear()
    assert L.fl_field_registry_count() == 0


@pytest.mark.gpu
def test_soa_manager(ctx):
    import numpy as np
    L = ctx.lib
    st, d = make(b"populations", t=0, c=19)
    h = ctypes.c_uint64()
    ctx.call("fl_soa_allocate", ctypes.byref(d), ctypes.c_size_t(1000), ctypes.byref(h))
    ptrs = []
    for c in range(19):
        p = ctypes.c_void_p()
        ctx.call("fl_soa_device_ptr", h, c, ctypes.byref(p))
        ptrs.append(p.value)
    pitch = ctypes.c_size_t()
    ctx.call("fl_soa_info", h, None, ctypes.byref(pitch), None)
    assert pitch.value % 128 == 0 and pitch.value >= 4000
    assert all(b - a == pitch.value for a, b in zip(ptrs, ptrs[1:]))   # component-major, no overlap
    a = np.arange(1000, dtype=np.float32)
    ctx.call("fl_memcpy_h2d", ctypes.c_void_p(ptrs[5]), a.ctypes.data_as(ctypes.c_void_p), ctypes.c_size_t(4000))
    ctx.call("fl_soa_resize", h, ctypes.c_size_t(3000))
    p = ctypes.c_void_p()
    ctx.call("fl_soa_device_ptr", h, 5, ctypes.byref(p))
    b = np.empty(1000, np.float32)
    ctx.call("fl_memcpy_d2h", b.ctypes.data_as(ctypes.c_void_p), p, ctypes.c_size_t(4000))
    np.testing.assert_array_equal(a, b)  # resize keeps the data
    ver = ctypes.c_uint64()
    ctx.call("fl_soa_info", h, None, None, ctypes.byref(ver))
    assert ver.value == 2
    assert L.fl_soa_device_ptr(ctx.handle, h, 19, ctypes.byref(p)) != 0   # component out of range
    ctx.call("fl_soa_deallocate", h)
