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
