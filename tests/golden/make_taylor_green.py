"""Generate tests/golden/taylor_green_ref.npz from the reference's analytic
Taylor-Green solution (tests/validation/analytical/TaylorGreenSolution.h:25-47),
compiled in place by oracle/Makefile.ref (oracle/_ref/ref_taylor_green).
Run here, where the reference tree exists; the .npz is committed and read by
the tests."""
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle.build import build_reference  # noqa: E402


def main():
    ref = build_reference()
    if ref is None:
        raise SystemExit("reference tree not present")
    out = os.path.join(ref, "taylor_green.bin")
    subprocess.run([os.path.join(ref, "ref_taylor_green"), out], check=True)
    raw = open(out, "rb").read()
    n = int(np.frombuffer(raw, "<i4", 1, 0)[0])
    a = np.frombuffer(raw, "<f8", n * 9, 4).reshape(n, 9)
    np.savez_compressed(os.path.join(HERE, "taylor_green_ref.npz"), xyz=a[:, 0:3], t=a[:, 3], re=a[:, 4],
                        uvw=a[:, 5:8], energy=a[:, 8])
    print(n, "records")


if __name__ == "__main__":
    main()
