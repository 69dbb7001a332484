"""Checked entry points: non-finite values and particles outside the mesh are counted on the
device and returned as SPHX_ERR_NUMERIC, never trapped.  The faults are planted on the host
(a NaN or an infinity written into an uploaded variable, a position moved out of the tank);
nothing here makes a GPU fault."""
import numpy as np
import pytest

from sphinxsys_gb300 import cases
from sphinxsys_gb300 import native as N
from sphinxsys_gb300.dambreak import DamBreak, MixedPrecisionDamBreak

pytestmark = pytest.mark.gpu


def test_body_check_counts_planted_non_finite_values():
    sim = DamBreak(cases.dambreak_2d())
    body = sim.water_block
    assert body.count_non_finite("Velocity") == 0
    assert body.count_non_finite("Density") == 0
    v = body.download("Velocity")
    v[7, 1] = np.nan
    v[100, 0] = np.inf
    v[100, 1] = -np.inf  # the same particle counts once
    body.upload("Velocity", v)
    assert body.count_non_finite("Velocity") == 2
    with pytest.raises(N.SphxError) as e:
        N.call("sphx_body_check_finite", body.handle, b"Velocity", None)
    assert e.value.code == 7
    with pytest.raises(N.SphxError) as e:
        N.call("sphx_body_check_finite", body.handle, b"NoSuchVariable", None)
    assert e.value.code == 5
    with pytest.raises(N.SphxError) as e:  # an index variable is not floating point
        N.call("sphx_body_check_finite", body.handle, b"OriginalID", None)
    assert e.value.code == 1


@pytest.mark.parametrize("dim", [2, 3])
def test_mixed_state_check_finds_planted_faults(dim):
    case = cases.dambreak_2d(0.05) if dim == 2 else cases.dambreak_3d(0.05)
    mp = MixedPrecisionDamBreak(case)
    mp.advection_step()
    assert mp.check_state() == (0, 0)
    body = mp.fp64.water_block
    mp.download(body)
    x = body.download("Position")
    v = body.download("Velocity")
    v[3, 0] = np.nan
    x[11, dim - 1] = case.sys_upper[dim - 1] + 10.0 * case.dp  # above the mesh
    x[12, 0] = case.sys_lower[0] - 10.0 * case.dp  # below it
    body.upload("Velocity", v)
    body.upload("Position", x)
    mp.upload(body)
    assert mp.check_state() == (1, 2)
    with pytest.raises(N.SphxError) as e:
        N.call("sphx_mp_check_state", mp.handle, None, None)
    assert e.value.code == 7
