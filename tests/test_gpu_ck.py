"""CK numerics on the GPU (sphx_ck_*) against the oracle's restatement of the tests_sycl
dam-break driver, and the reference's regression rule on the GPU run.

Tolerances: set-up fields (compression, correction matrices) within 1e-12 relative; fields
after 20 advection steps (about 100 acoustic steps) within 1e-10 relative (FP64 on both
sides, sums in the same neighbour order; the difference is FMA contraction)."""
import numpy as np
import pytest

from oracle import oracle as O
from sphinxsys_gb300 import cases, regression
from sphinxsys_gb300.dambreak import DamBreakCK

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.max(np.abs(np.asarray(a) - np.asarray(b))) / max(np.max(np.abs(b)), 1e-300))


@pytest.mark.parametrize("case", [cases.dambreak_2d(), cases.dambreak_3d(0.04)], ids=lambda c: c.name)
def test_ck_setup_matches_oracle(case):
    gpu = DamBreakCK(case)
    oc = O.OracleCase(case)
    oc.ck_initialize()
    f = gpu.water_block
    d = case.dim
    assert rel(f.download("Compression"), oc.ck_get("Compression")) < 1e-12
    assert rel(f.download("Density"), oc.get("Density")) < 1e-12
    assert rel(f.download("VolumetricMeasure"), oc.get("VolumetricMeasure")) < 1e-12
    B = f.download("LinearCorrectionMatrix").reshape(-1, d, d)
    assert rel(B, oc.ck_get("LinearCorrectionMatrix")) < 1e-12


@pytest.mark.parametrize("case", [cases.dambreak_2d(), cases.dambreak_3d(0.04)], ids=lambda c: c.name)
def test_ck_advection_steps_match_oracle(case):
    gpu = DamBreakCK(case)
    oc = O.OracleCase(case)
    oc.ck_initialize()
    steps = 0
    while steps < 20:
        due_g = gpu.acoustic_step()
        due_o = oc.ck_acoustic_step()
        assert due_g == due_o
        assert abs(gpu.physical_time / oc.physical_time.value - 1) < 1e-12
        if due_g:
            gpu.configuration()
            oc.ck_configuration()
            steps += 1
    f = gpu.water_block
    errs = {nm: rel(f.download(nm), oc.get(nm)) for nm in ("Position", "Velocity", "Density", "Pressure")}
    errs["Compression"] = rel(f.download("Compression"), oc.ck_get("Compression"))
    print(case.name, gpu.acoustic_steps, errs)
    assert max(errs.values()) < 1e-10, errs


def test_ck_gpu_dambreak_2d_passes_reference_regression(golden):
    """dambreak_sycl.cpp's observation schedule (every 200 advection steps) to t = 20 on the
    GPU, against the series stored with that test."""
    sim = DamBreakCK(cases.dambreak_2d())
    pressure, energy = [sim.observe_pressure()[0]], [sim.mechanical_energy()]
    while sim.physical_time < 20.0:
        if sim.acoustic_step():
            if sim.advection_steps % 200 == 0:
                energy.append(sim.mechanical_energy())
                pressure.append(sim.observe_pressure()[0])
            sim.configuration()
    assert 20 <= len(pressure) <= 26
    for q, cur in (("FluidObserver_Pressure", pressure), ("WaterBody_TotalMechanicalEnergy", energy)):
        runs = [golden[k] for k in golden.files if k.startswith(f"dambreak2d_ck/{q}/Run_")]
        ok, d = regression.passes(runs, cur, golden[f"dambreak2d_ck/{q}/dtw"])
        print(q, d.ravel())
        assert ok, (q, d)


def test_ck_free_surface_indicator_matches_oracle():
    """FreeSurfaceIndicationCK on the initial 3D lattice: interior position divergence about
    3 (the lattice sum of -dW V r), surface particles below 0.75 d, and the same
    PositionDivergence / Indicator as the oracle."""
    from sphinxsys_gb300.dambreak import DamBreakCKNested
    case = cases.dambreak_3d_reference()
    gpu = DamBreakCKNested(case)
    oc = O.OracleCase(case)
    gpu.indication.exec()
    oc.ck_free_surface_indication()
    f = gpu.water_block
    assert rel(f.download("PositionDivergence"), oc.ck_get("PositionDivergence")) < 1e-12
    assert np.array_equal(f.download("Indicator").astype(np.int64), oc.ck_get("Indicator").astype(np.int64))
    ind = f.download("Indicator")
    assert 0 < ind.sum() < len(ind)


def test_ck_nested_loop_matches_oracle():
    """The nested-loop CK driver of the 3D SYCL dam break: 10 advection steps on the GPU
    against the oracle (fields within 1e-10, indicator equal, same sub-step counts)."""
    from sphinxsys_gb300.dambreak import DamBreakCKNested
    case = cases.dambreak_3d_reference()
    gpu = DamBreakCKNested(case)
    oc = O.OracleCase(case)
    for step in range(10):
        s_g, dt_g = gpu.advection_step()
        s_o, dt_o = oc.ck_nested_advection_step()
        assert s_g == s_o, step
        assert abs(dt_g / dt_o - 1) < 1e-12, step
    assert abs(gpu.physical_time / oc.physical_time.value - 1) < 1e-12
    f = gpu.water_block
    errs = {nm: rel(f.download(nm), oc.get(nm)) for nm in ("Position", "Velocity", "Density", "Pressure")}
    errs["Compression"] = rel(f.download("Compression"), oc.ck_get("Compression"))
    errs["PositionDivergence"] = rel(f.download("PositionDivergence"), oc.ck_get("PositionDivergence"))
    print(errs)
    assert max(errs.values()) < 1e-10, errs
    assert np.array_equal(f.download("Indicator").astype(np.int64), oc.ck_get("Indicator").astype(np.int64))
    assert np.allclose(gpu.observe_pressure(), oc.ck_observe_pressure(), rtol=1e-9, atol=1e-9)


def test_ck_gpu_dambreak_3d_passes_reference_regression(golden):
    """tests_sycl/3d_examples/test_3d_dambreak_sycl to t = 20 on the GPU: the six wall probes
    after every advection step (and at the start) and the energy every unit of time,
    against the series stored with that test, in both orders of the DTW table."""
    from sphinxsys_gb300.dambreak import DamBreakCKNested
    sim = DamBreakCKNested(cases.dambreak_3d_reference())
    pressure, energy = [sim.observe_pressure()], [sim.mechanical_energy()]
    while sim.physical_time < 20.0:
        integration_time = 0.0
        while integration_time < 1.0:
            t0 = sim.physical_time
            sim.advection_step()
            integration_time += sim.physical_time - t0
            pressure.append(sim.observe_pressure())
        energy.append(sim.mechanical_energy())
    assert len(energy) == 21 and 0.8 * 2281 <= len(pressure) <= 1.2 * 2281
    for q, cur in (("FluidObserver_Pressure", np.array(pressure).T), ("WaterBody_TotalMechanicalEnergy", [energy])):
        runs = [golden[k] for k in golden.files if k.startswith(f"dambreak3d_ck/{q}/Run_")]
        ok, d = regression.passes(runs, cur, golden[f"dambreak3d_ck/{q}/dtw"], both_orders=True)
        assert ok, (q, d)
