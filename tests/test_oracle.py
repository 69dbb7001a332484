"""The oracle itself: pinned against the reference's regression databases."""
import numpy as np
import pytest

from oracle import oracle as O
from sphinxsys_gb300 import cases, regression


def series_keys(golden, prefix):
    return [golden[k] for k in golden.files if k.startswith(prefix + "/Run_")]


def test_exclusive_scan_known_answer_fixture(golden):
    inp, exp = golden["exclusive_scan/input"], golden["exclusive_scan/expected"]
    # exclusive_scan over all but the last entry (test_exclusive_scan.cpp:10-36)
    assert np.array_equal(np.concatenate([[0], np.cumsum(inp[:-1])]), exp)


def test_dtw_matches_reference_rule_on_stored_runs(golden):
    runs = series_keys(golden, "dambreak2d/FluidObserver_Pressure")
    d = regression.dtw_distance(runs[0][0], runs[1][0])
    assert 0 < d <= golden["dambreak2d/FluidObserver_Pressure/dtw"][0] * 1.01


def test_cell_list_is_counting_sort_of_positions():
    oc = O.OracleCase(cases.dambreak_2d())
    off, idx = oc.cell_list(O.FLUID)
    lo, gs, ac = oc.mesh()
    x = oc.get("Position")
    c = np.clip(np.floor((x - lo[:2]) / gs).astype(int), 0, np.array(ac[:2]) - 1)
    lin = c[:, 0] * ac[1] + c[:, 1]
    expect = np.argsort(lin, kind="stable")
    assert np.array_equal(idx, expect)
    assert np.array_equal(off, np.concatenate([[0], np.cumsum(np.bincount(lin, minlength=len(off) - 1))]))


def test_neighbor_lists_symmetric_and_within_cutoff():
    oc = O.OracleCase(cases.dambreak_2d())
    nb = oc.neighbors(O.INNER)
    i = np.repeat(np.arange(len(nb["counts"])), nb["counts"])
    pairs = set(zip(i.tolist(), nb["j"].tolist()))
    assert all((j, k) in pairs for (k, j) in pairs)
    assert np.all(nb["r"] < oc.constant("rc"))
    assert nb["counts"].max() == 20  # 2D lattice, r < 2.6 dp


@pytest.mark.slow
def test_oracle_2d_dambreak_passes_reference_dtw_regression(golden):
    """Runs the 2D dam break to t = 20 with the Dambreak.cpp loop and observation schedule
    and applies RegressionTestDynamicTimeWarping::resultTest to every stored run."""
    case = cases.dambreak_2d()
    oc = O.OracleCase(case)
    pressure = [oc.observe_pressure()[0]]
    energy = [oc.total_mechanical_energy()]
    while oc.physical_time.value < 20.0:
        integration_time = 0.0
        while integration_time < 0.1:
            t0 = oc.physical_time.value
            observe = oc.iteration % 200 == 0 and oc.iteration != 0
            _, _, obs, en = oc.advection_step(observe=observe)
            integration_time += oc.physical_time.value - t0
            if observe:
                pressure.append(obs[0])
                energy.append(en)
    assert len(pressure) == 23
    for q, cur in (("FluidObserver_Pressure", pressure), ("WaterBody_TotalMechanicalEnergy", energy)):
        ok, d = regression.passes(series_keys(golden, "dambreak2d/" + q), cur, golden[f"dambreak2d/{q}/dtw"])
        assert ok, (q, d)
