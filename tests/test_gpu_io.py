"""Restart and state files of a GPU run: a dam break restarted from a restart file written
after 5 advection steps continues bit for bit like the uninterrupted run; the state file
holds the device positions."""
import os
import tempfile

import numpy as np
import pytest

from sphinxsys_gb300 import cases
from sphinxsys_gb300 import io as IO
from sphinxsys_gb300.dambreak import DamBreak

pytestmark = pytest.mark.gpu


def test_restart_continues_bit_for_bit():
    case = cases.dambreak_2d()
    a = DamBreak(case)
    for _ in range(10):
        a.advection_step()
    b = DamBreak(case)
    for _ in range(5):
        b.advection_step()
    with tempfile.TemporaryDirectory() as d:
        rio = IO.RestartIO(b.sph_system, restart_folder=d)
        rio.writeToFile(5, b.physical_time)
        c = DamBreak(case)
        c.physical_time = IO.RestartIO(c.sph_system, restart_folder=d).readRestartFiles(5)
        c.number_of_iterations = 5
        # rebuild what the restart file does not hold: cell lists and configurations
        c.water_block.updateCellLinkedList()
        c.water_wall_complex.updateConfiguration()
        c.fluid_observer_contact.updateConfiguration()
        vtp = IO.BodyStatesRecordingToVtp(c.sph_system, output_folder=d)
        vtp.addToWrite(c.water_block, "Density")
        paths = vtp.writeToFile(iteration=5, physical_time=c.physical_time)
        assert {os.path.basename(p) for p in paths} >= {"WaterBody_ite_0000000005.vtp"}
        got = IO.read_vtp(os.path.join(d, "WaterBody_ite_0000000005.vtp"))
        assert np.allclose(got["Position"][:, :2], c.water_block.download("Position"), atol=1e-8)
    assert c.physical_time == b.physical_time
    for _ in range(5):
        c.advection_step()
    assert c.physical_time == a.physical_time
    for nm in ("Position", "Velocity", "Density", "Pressure"):
        assert np.array_equal(c.water_block.download(nm), a.water_block.download(nm)), nm
