"""CPU-side checks of the C ABI: the library loads, exports every declared
symbol, and its host helpers agree with the reference semantics."""
import ctypes
import os
import re
import subprocess

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_library_builds_and_exports_all_declared_symbols():
    from fluidloom_gb300 import build, _capi
    path = build.build()
    declared = set()
    for h in os.listdir(os.path.join(ROOT, "include")):
        if h.endswith(".h"):
            declared |= set(_capi.parse_header(os.path.join(ROOT, "include", h)))
    assert len(declared) >= 20
    out = subprocess.run(["nm", "-D", "--defined-only", path], capture_output=True, text=True, check=True).stdout
    exported = set(re.findall(r"\bT (fl_\w+)", out))
    missing = declared - exported
    assert not missing, missing
    L = _capi.lib()
    for name in declared:
        assert getattr(L, name) is not None


def test_host_helpers():
    from fluidloom_gb300 import _capi
    L = _capi.lib()
    assert L.fl_hilbert_get_parent(0o1234, 4) == 0o123
    assert L.fl_hilbert_get_child(0o123, 3, 4) == 0o1234
    assert L.fl_hilbert_get_child(1, 21, 0) == 0xFFFFFFFFFFFFFFFF
    assert L.fl_hilbert_is_valid(0xFFFFFFFFFFFFFFFF, 8) == 0
    assert L.fl_hilbert_is_valid(1 << 63, 21) == 0
    assert L.fl_hilbert_is_valid(1 << 15, 5) == 0  # bits above 3*level
    assert L.fl_hilbert_is_valid((1 << 15) - 1, 5) == 1
    assert L.fl_status_string(0) == b"ok"


def test_no_device_is_reported_not_faked():
    from fluidloom_gb300 import _capi
    L = _capi.lib()
    h = ctypes.c_void_p()
    st = L.fl_ctx_create(0, ctypes.byref(h))
    try:
        import torch
        has = torch.cuda.is_available()
    except Exception:
        has = False
    if not has:
        assert st == -8  # FL_E_NO_DEVICE: no silent CPU path
    else:
        assert st == 0
        L.fl_ctx_destroy(h)
