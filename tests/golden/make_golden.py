"""Generate tests/golden/hilbert_ref.npz from the reference's own key codecs.

Builds oracle/_ref/ref_harness from the reference sources in place
(oracle/Makefile.ref: src/core/hilbert/HilbertCodec.cpp and
src/adaptation/utils/HilbertCodec3D.cpp) and records what they return for the
cases of tests/unit/hilbert/test_hilbert_codec.cpp:33-125 (same RNG and draw
order) plus 21-level, all-level and 8-level-encoder sweeps.  Run here, where
the reference tree exists; the .npz is committed and read by the tests.
"""
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle.build import build_reference  # noqa: E402

SECTIONS = ["corners_l1", "roundtrip_l1_8", "canonical", "parent_child", "l21_random",
            "all_levels", "morton8", "parent21"]


def main():
    ref = build_reference()
    if ref is None:
        raise SystemExit("reference tree not present")
    out = os.path.join(ref, "kat.bin")
    subprocess.run([os.path.join(ref, "ref_harness"), out], check=True)
    raw = open(out, "rb").read()
    rec = np.dtype([("x", "<i4"), ("y", "<i4"), ("z", "<i4"), ("level", "<u4"), ("key", "<u8")])
    pos = 0
    arrays = {}
    for name in SECTIONS:
        n = int(np.frombuffer(raw, "<u4", 1, pos)[0])
        pos += 4
        a = np.frombuffer(raw, rec, n, pos)
        pos += n * rec.itemsize
        arrays[name + "_xyz"] = np.stack([a["x"], a["y"], a["z"]], 1).astype(np.int32)
        arrays[name + "_level"] = a["level"].astype(np.uint8)
        arrays[name + "_key"] = a["key"].astype(np.uint64)
    assert pos == len(raw)
    np.savez_compressed(os.path.join(HERE, "hilbert_ref.npz"), **arrays)
    print({k: v.shape for k, v in arrays.items()})


if __name__ == "__main__":
    main()
