"""Build the CPU oracle (test infrastructure only) into oracle/_build/liboracle.so.

Compiled with -ffp-contract=off so FP32 results are the plain IEEE sequence of
operations written in the sources on every host (x86-64 and aarch64).
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SOURCES = ["or_keys_prims.cpp", "or_amr.cpp", "or_lbm.cpp", "or_geometry.cpp"]
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "liboracle.so")


def build(force=False):
    os.makedirs(OUT_DIR, exist_ok=True)
    srcs = [os.path.join(HERE, s) for s in SOURCES] + [os.path.join(HERE, "oracle.h")]
    if not force and os.path.exists(LIB):
        t = os.path.getmtime(LIB)
        if all(os.path.getmtime(s) <= t for s in srcs):
            return LIB
    cmd = ["g++", "-O2", "-std=c++17", "-fopenmp", "-fPIC", "-shared", "-ffp-contract=off",
           "-o", LIB] + [os.path.join(HERE, s) for s in SOURCES]
    subprocess.run(cmd, check=True)
    return LIB


# The reference tree, read only by the in-place compile recipe (Makefile.ref) and
# the tests that parse its scripts; absent on hosts without it.
REF_ROOT = os.environ.get("FLUIDLOOM_REF_ROOT", "/root/reference")
REF_DIR = os.path.join(HERE, "_ref")


def build_reference(ref_root=None):
    """Compile parts of the reference in place (only where the tree exists):
    its key codecs, geometry placement and regrid/hash kernels."""
    ref_root = ref_root or REF_ROOT
    if not os.path.isdir(ref_root):
        return None
    subprocess.run(["make", "-s", "-f", os.path.join(HERE, "Makefile.ref"), "REF=" + ref_root],
                   check=True)
    return REF_DIR


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
    print(build_reference())
