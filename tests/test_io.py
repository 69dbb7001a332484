"""On-disk formats (sphinxsys_gb300/io.py): VTK XML PolyData state files and restart files in
the reference's layouts; host-side, so these run without a GPU."""
import os
import tempfile
import xml.etree.ElementTree as ET

import numpy as np

from sphinxsys_gb300 import io as IO


def test_vtp_layout_and_round_trip():
    rng = np.random.default_rng(0)
    n = 7
    pos = rng.random((n, 2))
    rho = rng.random(n)
    vel = rng.random((n, 2))
    ids = np.arange(n, dtype=np.uint32)[::-1].copy()
    B = rng.random((n, 2, 2))
    with tempfile.TemporaryDirectory() as d:
        p = os.path.join(d, "WaterBody_ite_0000000010.vtp")
        IO.write_vtp(p, "WaterBody", pos, [("OriginalID", ids), ("Density", rho), ("Velocity", vel),
                                           ("LinearCorrectionMatrix", B)], physical_time=1.25)
        root = ET.parse(p).getroot()
        assert root.tag == "VTKFile" and root.get("type") == "PolyData"
        piece = root.find("PolyData/Piece")
        assert piece.get("NumberOfPoints") == str(n) and piece.get("NumberOfVerts") == str(n)
        got = IO.read_vtp(p)
    assert abs(got["TimeValue"][0] - 1.25) < 1e-12
    assert np.allclose(got["Position"][:, :2], pos, atol=1e-9) and np.all(got["Position"][:, 2] == 0)
    assert np.array_equal(got["SortedParticle_ID"], np.arange(n))
    assert np.array_equal(got["OriginalID"], ids)
    assert np.allclose(got["Density"], rho, atol=1e-9)
    assert np.allclose(got["Velocity"][:, :2], vel, atol=1e-9)
    m = got["LinearCorrectionMatrix"].reshape(n, 3, 3)  # column-major entries
    assert np.allclose(np.transpose(m, (0, 2, 1))[:, :2, :2], B, atol=1e-9)
    assert np.array_equal(got["connectivity"], np.arange(n)) and np.array_equal(got["offsets"], np.arange(1, n + 1))


def test_file_sequences():
    assert IO.vtp_sequence(iteration=42) == "ite_0000000042"
    assert IO.vtp_sequence(physical_time=0.5) == "0000500000"
    assert IO.pad(7) == "0000000007"


def test_restart_round_trip_is_exact():
    rng = np.random.default_rng(1)
    fluid = {"Position": rng.random((5, 3)), "Density": rng.random(5) + 1.0, "Mass": np.full(5, 1e-3)}
    wall = {"Position": rng.random((3, 3)), "NormalDirection": rng.random((3, 3))}
    with tempfile.TemporaryDirectory() as d:
        p = os.path.join(d, "Restart_0000000100.xml")
        IO.write_restart(p, 0.123456789012345678, [("WaterBody", fluid), ("WallBoundary", wall)])
        root = ET.parse(p).getroot()
        assert root.tag == "restart_data" and [b.get("name") for b in root.findall("body")] == [
            "WaterBody", "WallBoundary"]
        assert len(root.find("body").findall("particle")) == 5
        t, data = IO.read_restart(p)
    assert t == 0.123456789012345678
    for nm, v in fluid.items():
        assert np.array_equal(data["WaterBody"][nm], v)
    for nm, v in wall.items():
        assert np.array_equal(data["WallBoundary"][nm], v)
