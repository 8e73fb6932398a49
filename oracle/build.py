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


def build_reference(ref_root="/root/reference"):
    """Compile the reference's key codecs in place (only where the tree exists)."""
    if not os.path.isdir(ref_root):
        return None
    subprocess.run(["make", "-s", "-f", os.path.join(HERE, "Makefile.ref"), "REF=" + ref_root],
                   check=True)
    return os.path.join(HERE, "_ref")


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
    print(build_reference())
