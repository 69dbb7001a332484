"""Mixed precision against FP64 where the accuracy bound of the headline applies.

The 3D dam break of the benchmark geometry (tank 3.2 x 1.0 x 1.8, water column 1.2 x 1.0 x
0.6) at dp = 0.02 (90,000 fluid particles), both solvers from the same initial state, the
same number of advection steps, recorded every 5 steps:

* before the collapse turns irregular (t <= 0.75; the front reaches the far wall at
  t ~ 1.3): the wall-pressure probe at (0, 0.5, 0.2), wetted from t = 0, within 1e-4 of the
  FP64 reading, relative to max(|p_fp64|, 0.1 rho0 g (H - z)): the floor, a tenth of the
  probe's hydrostatic pressure, keeps the instants where the column's acoustic ringing
  passes through zero gauge pressure from dividing by a vanishing reading; the
  free-surface height (UpperFrontInAxisDirection over the initial column) within 1e-4 at
  every record;
* over the whole run to t = 2.0, through the impact: the flow amplifies any perturbation
  (an FP64 run whose initial positions are moved by 1e-7 h, the size of the FP32 rounding
  of the solver's cell offsets, departs from the unperturbed FP64 run the same way), so
  the bound there is relative to that control: the largest probe and free-surface
  differences of mixed against FP64 stay within C_CHAOS times those of the perturbed FP64
  run against FP64."""
import numpy as np
import pytest

from sphinxsys_gb300 import cases
from sphinxsys_gb300 import sph as S
from sphinxsys_gb300.dambreak import DamBreak, MixedPrecisionDamBreak

pytestmark = pytest.mark.gpu

DP = 0.02
REL_BOUND = 1e-4
T_SMOOTH = 0.75
T_END = 2.0
EVERY = 5
C_CHAOS = 10.0
PERTURBATION = 1e-7  # of h


def probe_index(case):
    return case.observers.index((0.0, 0.5, 0.2))


def gauge(case):
    """The initial water column over the full height: UpperFrontInAxisDirection region."""
    lo, up = list(case.sys_lower), list(case.sys_upper)
    lo[0] = case.water_center[0] - case.water_halfsize[0]
    up[0] = case.water_center[0] + case.water_halfsize[0]
    return lo, up


def record_mixed(case, t_end):
    mp = MixedPrecisionDamBreak(case)
    lo, up = gauge(case)
    k = probe_index(case)

    def sample():
        return mp.physical_time, float(mp.observe_pressure_view()[k]), mp.upper_front(case.vertical_axis, lo, up)

    rows, steps = [sample()], 0
    while mp.physical_time < t_end:
        mp.advection_step()
        steps += 1
        if steps % EVERY == 0:
            rows.append(sample())
    return np.array(rows), steps


def record_fp64(case, steps, perturb=0.0):
    sim = DamBreak(case)
    if perturb:
        x = sim.water_block.download("Position")
        rng = np.random.default_rng(0)
        sim.water_block.upload("Position", x + perturb * case.h * rng.uniform(-1.0, 1.0, x.shape))
        sim.update_configuration()
        sim.number_of_iterations = 0
    lo, up = gauge(case)
    k = probe_index(case)

    def sample():
        return (sim.physical_time, float(sim.recorded_pressure.exec()[k]),
                S.UpperFrontInAxisDirection(sim.water_block, lo, up, case.vertical_axis).exec())

    rows = [sample()]
    for s in range(1, steps + 1):
        sim.advection_step()
        if s % EVERY == 0:
            rows.append(sample())
    return np.array(rows)


@pytest.fixture(scope="module")
def runs():
    case = cases.dambreak_3d(DP)
    mixed, steps = record_mixed(case, T_END)
    fp64 = record_fp64(case, steps)
    control = record_fp64(case, steps, PERTURBATION)
    return case, mixed, fp64, control


def test_wetted_probe_and_free_surface_within_bound_before_impact(runs):
    case, mixed, fp64, _ = runs
    assert fp64[-1, 0] >= T_END
    sel = (fp64[:, 0] > 0) & (fp64[:, 0] <= T_SMOOTH)
    assert sel.sum() >= 25
    z = case.observers[probe_index(case)][2]
    floor = 0.1 * case.rho0 * case.gravity_g * (2.0 * case.water_halfsize[2] - z)
    p_rel = np.abs(mixed[sel, 1] - fp64[sel, 1]) / np.maximum(np.abs(fp64[sel, 1]), floor)
    fs_rel = np.abs(mixed[sel, 2] / fp64[sel, 2] - 1.0)
    print("probe rel", p_rel.max(), "free surface rel", fs_rel.max(), "records", sel.sum())
    assert np.all(np.abs(fp64[sel, 1]) > 0)  # wetted throughout
    assert p_rel.max() <= REL_BOUND, p_rel
    assert fs_rel.max() <= REL_BOUND, fs_rel


def test_differences_through_impact_bounded_by_fp64_perturbation_control(runs):
    _, mixed, fp64, control = runs
    d_mixed_p = np.abs(mixed[:, 1] - fp64[:, 1]).max()
    d_ctrl_p = np.abs(control[:, 1] - fp64[:, 1]).max()
    d_mixed_fs = np.abs(mixed[:, 2] / fp64[:, 2] - 1.0).max()
    d_ctrl_fs = np.abs(control[:, 2] / fp64[:, 2] - 1.0).max()
    print("probe: mixed", d_mixed_p, "control", d_ctrl_p, "| free surface: mixed", d_mixed_fs, "control",
          d_ctrl_fs)
    assert d_ctrl_p > 0 and d_ctrl_fs > 0
    assert d_mixed_p <= C_CHAOS * d_ctrl_p
    assert d_mixed_fs <= C_CHAOS * d_ctrl_fs
