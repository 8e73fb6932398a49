"""VTK PolyData writer on the host (the reference's VTKTest.GeneratesVTPFile,
tests/integration/VTKTest.cpp:11-112, with four level-0 cells), against a
stand-in pool that serves bricks and site fields from numpy."""
import numpy as np

from fluidloom_gb300 import io


class FakePool:
    def __init__(self, bricks, rho, vel):
        self._b, self._rho, self._vel = bricks, rho, vel

    def bricks(self):
        return dict(self._b)

    def macroscopic(self):
        return {"density": self._rho, "velocity": self._vel}


def _fake():
    b = {"x": np.array([0, 1, 0, 0], np.int32), "y": np.array([0, 0, 1, 0], np.int32),
         "z": np.array([0, 0, 0, 1], np.int32), "level": np.zeros(4, np.uint8), "case_id": np.zeros(4, np.uint16)}
    rng = np.random.default_rng(0)
    return FakePool(b, rng.random((4, 512), dtype=np.float32) + 0.5, rng.random((4, 512, 3), dtype=np.float32))


def test_generates_vtp_file(tmp_path):
    w = io.VTKWriter(str(tmp_path / "test_output"), per="brick")
    path = w.write_snapshot(0, 0.0, _fake())
    assert path.endswith("snapshot_000000.vtp")
    text = open(path).read()
    assert "<VTKFile" in text and 'NumberOfPoints="4"' in text


def test_site_arrays_round_trip(tmp_path):
    pool = _fake()
    for ascii_ in (False, True):
        p = io.write_vtp(str(tmp_path / ("s%d.vtp" % ascii_)), pool, ascii=ascii_)
        a = io.read_vtp_arrays(p)
        assert a["Points"].shape == (4 * 512, 3)
        np.testing.assert_array_equal(a["Density"], pool._rho.reshape(-1))
        np.testing.assert_array_equal(a["Velocity"], pool._vel.reshape(-1, 3))
        # site (x, y, z) of brick 1 sits at (8 + x + 0.5, y + 0.5, z + 0.5)
        np.testing.assert_array_equal(a["Points"][512 + 3 + 8 * 2 + 64 * 1], np.float32([11.5, 2.5, 1.5]))
        assert a["Level"].max() == 0 and len(a["offsets"]) == 4 * 512
