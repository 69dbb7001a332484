"""Taylor-Green vortex (periodic box, viscous force, transport-velocity correction) on the
CUDA execution policy against the oracle, and the reference's regression rule on the GPU.

Tolerance: FP64 fields within 1e-10 relative (max |gpu - oracle| / max |oracle|) after
several advection steps: the device sums neighbours in the same order as the oracle but
fuses multiply-adds, so the two agree to a few ulp per step.  The mixed-precision solver
(sphx_mp_create_periodic) against the FP64 GPU run: velocity within 1e-5 relative and
positions within 1e-6 of the box size after 10 advection steps, kinetic energy within
1e-5 relative after 20."""
import numpy as np
import pytest

from sphinxsys_gb300 import cases, regression
from sphinxsys_gb300.taylor_green import MixedPrecisionTaylorGreen, TaylorGreen

from oracle import oracle as O

pytestmark = pytest.mark.gpu

TOL = 1e-10


def rel_err(a, b):
    return float(np.max(np.abs(np.asarray(a) - np.asarray(b))) / max(np.max(np.abs(b)), 1e-300))


def small_3d():
    # the 3D vortex on [0, 2 pi]^3 with 20 particles per side
    return cases.TaylorGreenCase("taylor_green3d_20", 3, 2.0 * np.pi, 2.0 * np.pi / 20, 1)


@pytest.mark.parametrize("case", [cases.taylor_green_2d(40), small_3d()], ids=lambda c: c.name)
def test_taylor_green_matches_oracle(case):
    g = TaylorGreen(case)
    o = O.OracleTGV(case)
    # the periodic images of the cell list: one entry per particle plus one per image
    assert int(g.water_block.cell_list_entries()) == o.cell_entries()
    assert abs(g.kinetic_energy.exec() / o.kinetic_energy() - 1) < 1e-12
    for step in range(8):
        s_g, dt_g = g.advection_step()
        s_o, dt_o = o.advection_step()
        assert s_g == s_o, step
        assert abs(dt_g / dt_o - 1) < 1e-12, step
    assert abs(g.physical_time / o.physical_time.value - 1) < 1e-12
    assert int(g.water_block.cell_list_entries()) == o.cell_entries()
    for name in ("Position", "Velocity", "Density", "Pressure", "Force", "ForcePrior"):
        err = rel_err(g.water_block.download(name), o.get(name))
        assert err < TOL, (name, err)
    assert abs(g.kinetic_energy.exec() / o.kinetic_energy() - 1) < 1e-10
    assert abs(g.maximum_speed.exec() / o.maximum_speed() - 1) < 1e-10


def test_periodic_bounding_keeps_particles_in_the_box():
    case = cases.taylor_green_2d(40)
    g = TaylorGreen(case)
    for _ in range(30):
        g.advection_step()
    x = g.water_block.download("Position")
    assert np.all(x >= 0.0) and np.all(x <= case.L)


def test_gpu_taylor_green_passes_reference_dtw_regression(golden):
    """taylor_green.cpp to t = 5 on the GPU: kinetic energy at t = 0 and every 0.1 and
    maximum speed every 0.1 against every stored run, with
    RegressionTestDynamicTimeWarping's rule."""
    g = TaylorGreen(cases.taylor_green_2d())
    ke, ms = [g.kinetic_energy.exec()], []
    while g.physical_time < 5.0:
        integ = 0.0
        while integ < 0.1:
            t0 = g.physical_time
            g.advection_step()
            integ += g.physical_time - t0
        ke.append(g.kinetic_energy.exec())
        ms.append(g.maximum_speed.exec())
    for q, cur in (("WaterBody_TotalKineticEnergy", ke), ("WaterBody_MaximumSpeed", ms)):
        runs = [golden[k] for k in golden.files if k.startswith(f"taylor_green2d/{q}/Run_")]
        ok, d = regression.passes(runs, cur, golden[f"taylor_green2d/{q}/dtw"])
        assert ok, (q, d)


def small_2d():
    return cases.taylor_green_2d(50)


@pytest.mark.parametrize("case", [small_2d(), small_3d()], ids=lambda c: c.name)
def test_mixed_precision_taylor_green_tracks_fp64(case):
    """Pointwise agreement for 10 advection steps, then norms to 20 steps.

    From about the 12th step of the 2D vortex at 50 x 50 the particles near the hyperbolic
    stagnation points amplify any rounding difference about threefold per advection step:
    the FP64 GPU run and the FP64 oracle (equal to ~1e-16 per step) grow apart from 3e-14
    at step 12 to 1.5e-10 at step 23 in the same way.  The mixed-precision run starts
    from ~1e-7 differences, so the pointwise comparison stops at step 10 and the later
    steps are checked through the kinetic energy and the RMS velocity difference."""
    ref = TaylorGreen(case)
    mp = MixedPrecisionTaylorGreen(case)
    assert abs(mp.kinetic_energy() / ref.kinetic_energy.exec() - 1) < 1e-6
    # the viscous force of the initial state (the solver computes it in its first build)
    probe = TaylorGreen(case)
    probe.update_density_by_summation.exec()
    probe.viscous_force.exec()
    mp.download()
    assert rel_err(mp.water_block.download("ForcePrior"), probe.water_block.download("ForcePrior")) < 1e-4
    for step in range(20):
        s_r, dt_r = ref.advection_step()
        s_m, dt_m = mp.advection_step()
        assert abs(s_r - s_m) <= 1, step
        assert abs(dt_m / dt_r - 1) < 1e-5, step
        if step == 9:
            mp.download()
            errs = {n: rel_err(mp.water_block.download(n), ref.water_block.download(n))
                    for n in ("Velocity", "Density")}
            d = mp.water_block.download("Position") - ref.water_block.download("Position")
            d = (d + 0.5 * case.L) % case.L - 0.5 * case.L  # a particle may sit on either side of a face
            errs["Position"] = float(np.max(np.abs(d)) / case.L)
            print(case.name, errs)
            assert errs["Velocity"] < 1e-5, errs
            assert errs["Density"] < 1e-6, errs
            assert errs["Position"] < 1e-6, errs
    mp.download()
    vm, vr = mp.water_block.download("Velocity"), ref.water_block.download("Velocity")
    rms = np.sqrt(np.mean(np.sum((vm - vr) ** 2, axis=1)) / np.mean(np.sum(vr * vr, axis=1)))
    ke = abs(mp.kinetic_energy() / ref.kinetic_energy.exec() - 1)
    print(case.name, "rms", rms, "ke", ke)
    assert rms < 1e-3 and ke < 1e-5, (rms, ke)


def test_mixed_precision_taylor_green_strategies_bitwise_equal():
    case = small_3d()
    outs = []
    for block, strategy in ((128, 0), (64, 0), (256, 1), (96, 1)):
        mp = MixedPrecisionTaylorGreen(case, block=block, strategy=strategy)
        for _ in range(5):
            mp.advection_step()
        mp.download()
        outs.append([mp.water_block.download(n) for n in ("Position", "Velocity", "Density")])
    for other in outs[1:]:
        for a, b in zip(outs[0], other):
            assert np.array_equal(a, b)


def test_mixed_precision_taylor_green_3d_early_decay_is_viscous():
    """The 3D vortex at 32^3 to t = 0.5: kinetic energy follows exp(-6 nu t) (the decay
    of the linearised flow, |k|^2 = 3) within 2 %, as the FP64 oracle does at this
    resolution."""
    case = cases.TaylorGreenCase("taylor_green3d_32", 3, 2.0 * np.pi, 2.0 * np.pi / 32, 1)
    mp = MixedPrecisionTaylorGreen(case)
    ke0, nu = mp.kinetic_energy(), case.mu / case.rho0
    while mp.physical_time < 0.5:
        mp.advection_step()
        ratio = mp.kinetic_energy() / ke0
        assert abs(ratio / np.exp(-6.0 * nu * mp.physical_time) - 1) < 0.02, (mp.physical_time, ratio)


def test_mixed_precision_taylor_green_passes_reference_dtw_regression(golden):
    g = MixedPrecisionTaylorGreen(cases.taylor_green_2d())
    ke, ms = [g.kinetic_energy()], []
    while g.physical_time < 5.0:
        integ = 0.0
        while integ < 0.1:
            t0 = g.physical_time
            g.advection_step()
            integ += g.physical_time - t0
        ke.append(g.kinetic_energy())
        ms.append(g.maximum_speed())
    for q, cur in (("WaterBody_TotalKineticEnergy", ke), ("WaterBody_MaximumSpeed", ms)):
        runs = [golden[k] for k in golden.files if k.startswith(f"taylor_green2d/{q}/Run_")]
        ok, d = regression.passes(runs, cur, golden[f"taylor_green2d/{q}/dtw"])
        assert ok, (q, d)


def test_mixed_precision_periodic_search_finds_every_neighbour():
    """Wrapped, pruned sub-cell search against the FP64 periodic relation on the same lattice."""
    case = small_3d()
    mp = MixedPrecisionTaylorGreen(case)
    ref = TaylorGreen(case)
    n_in = int(ref.water_block_inner.neighbors()["counts"].sum())
    assert mp.list_sizes()["nnz_inner"] == n_in == 80 * ref.water_block.n


def test_periodic_set_up_rejects_invalid_boxes():
    """The periodic cell list needs 2 cut-offs < L; the mixed periodic solver a cube with at
    least 5 sub-cells per axis; both refuse with SPHX_ERR_INVALID_ARG and keep the context
    usable."""
    import ctypes as C
    from sphinxsys_gb300 import native as N
    g = TaylorGreen(cases.taylor_green_2d(40))
    cl = g.water_block._cl_handle()
    with pytest.raises(N.SphxError) as e:
        N.call("sphx_cell_list_set_periodic", cl, 0, 0.0, 0.1, 0.05)  # 2 x 0.05 is not below 0.1
    assert e.value.code == 1
    with pytest.raises(N.SphxError) as e:
        N.call("sphx_cell_list_set_periodic", cl, 2, 0.0, 1.0, 0.05)  # no third axis in 2D
    assert e.value.code == 1
    p = g.pressure_relaxation.params
    h = C.c_void_p()
    pd = C.POINTER(C.c_double)
    lo, up = np.zeros(3), np.array([1.0, 0.5, 0.0])
    with pytest.raises(N.SphxError) as e:  # not a cube
        N.call("sphx_mp_create_periodic", g.water_block.handle, C.byref(p), lo.ctypes.data_as(pd),
               up.ctypes.data_as(pd), 0.01, 0.2, C.byref(h))
    assert e.value.code == 1
    up = np.array([0.1, 0.1, 0.0])  # 0.1 / h = 3 sub-cells per axis
    with pytest.raises(N.SphxError) as e:
        N.call("sphx_mp_create_periodic", g.water_block.handle, C.byref(p), lo.ctypes.data_as(pd),
               up.ctypes.data_as(pd), 0.01, 0.2, C.byref(h))
    assert e.value.code == 1
    # the context still runs the flow
    g.advection_step()
    assert np.all(np.isfinite(g.water_block.download("Velocity")))


def test_host_row_load_refuses_a_periodic_solver():
    """sphx_mp_upload_host serves the dam-break solvers; a periodic solver answers
    SPHX_ERR_INVALID_ARG and keeps running."""
    import ctypes as C
    from sphinxsys_gb300 import native as N
    case = small_3d()
    mp = MixedPrecisionTaylorGreen(case)
    n = mp.water_block.n
    rows = [np.zeros((n, 3)), np.zeros((n, 3)), np.zeros((n, 3)), np.ones(n), np.zeros(n)]
    with pytest.raises(N.SphxError) as e:
        N.call("sphx_mp_upload_host", mp.handle, *[C.c_void_p(a.ctypes.data) for a in rows])
    assert e.value.code == 1
    ke = mp.kinetic_energy()
    mp.advection_step()
    assert 0 < mp.kinetic_energy() < 1.01 * ke
