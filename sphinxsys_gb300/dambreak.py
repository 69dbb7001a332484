"""Dam-break driver on the CUDA execution policy.

``DamBreak(case)`` sets up the bodies, relations and dynamics exactly as
tests/2d_examples/test_2d_dambreak/Dambreak.cpp:56-127 does (and its 3D counterpart
tests/3d_examples/test_3d_dambreak/dambreak.cpp), and ``advection_step`` runs one pass
of the main loop (Dambreak.cpp:166-220): advection dt, density summation, the acoustic
sub-steps, the Morton re-sort every 100 steps and the configuration update.
"""
from __future__ import annotations

import numpy as np

from . import sph as S
from .cases import DamBreakCase


class DamBreak:
    def __init__(self, case: DamBreakCase, device: int = 0):
        self.case = case
        d = case.dim
        self.sph_system = S.SPHSystem(case.sys_lower[:d], case.sys_upper[:d], case.dp, device=device,
                                      h_spacing_ratio=case.h_ratio)
        water_shape = S.ComplexShape("WaterBody").add(
            S.GeometricShapeBox(case.water_center[:d], case.water_halfsize[:d]))
        wall_shape = S.ComplexShape("WallBoundary")
        wall_shape.add(S.GeometricShapeBox(case.outer_center[:d], case.outer_halfsize[:d]))
        wall_shape.subtract(S.GeometricShapeBox(case.inner_center[:d], case.inner_halfsize[:d]))

        self.water_block = S.FluidBody(self.sph_system, water_shape)
        self.water_block.defineMatterMaterial(S.WeaklyCompressibleFluid(case.rho0, case.c0))
        self.water_block.generateParticles(S.Lattice)

        self.wall_boundary = S.SolidBody(self.sph_system, wall_shape)
        self.wall_boundary.defineMatterMaterial(S.Solid())
        self.wall_boundary.generateParticles(S.Lattice)

        self.fluid_observer = S.ObserverBody(self.sph_system, name="FluidObserver")
        obs = np.array([o[:d] for o in case.observers]) if case.observers else np.zeros((0, d))
        self.fluid_observer.generateParticles(positions=obs)

        self.water_block_inner = S.InnerRelation(self.water_block)
        self.water_wall_contact = S.ContactRelation(self.water_block, [self.wall_boundary])
        self.fluid_observer_contact = S.ContactRelation(self.fluid_observer, [self.water_block])
        self.water_wall_complex = S.ComplexRelation(self.water_block_inner, self.water_wall_contact)

        self.gravity = S.Gravity(case.gravity[:d])
        self.constant_gravity = S.SimpleDynamics(S.GravityForce, self.water_block, self.gravity)
        self.wall_boundary_normal_direction = S.SimpleDynamics(S.NormalDirectionFromBodyShape, self.wall_boundary)

        self.fluid_pressure_relaxation = S.Dynamics1Level(S.Integration1stHalfWithWallRiemann,
                                                          self.water_block_inner, self.water_wall_contact)
        self.fluid_density_relaxation = S.Dynamics1Level(S.Integration2ndHalfWithWallRiemann,
                                                         self.water_block_inner, self.water_wall_contact)
        self.fluid_density_by_summation = S.InteractionWithUpdate(S.DensitySummationComplexFreeSurface,
                                                                  self.water_block_inner, self.water_wall_contact)
        self.fluid_advection_time_step = S.ReduceDynamics(S.AdvectionTimeStep, self.water_block, case.U_ref)
        self.fluid_acoustic_time_step = S.ReduceDynamics(S.AcousticTimeStep, self.water_block)
        self.particle_sorting = S.ParticleSorting(self.water_block)
        self.recorded_pressure = S.ObservedQuantityRecording("Pressure", self.fluid_observer_contact)
        self.mechanical_energy = S.TotalMechanicalEnergy(self.water_block, self.gravity)

        # Dambreak.cpp:124-127
        self.sph_system.initializeSystemCellLinkedLists()
        self.water_wall_complex.updateConfiguration()
        if self.fluid_observer.n:
            self.fluid_observer_contact.updateConfiguration()
        self.wall_boundary_normal_direction.exec()
        self.constant_gravity.exec()

        self.number_of_iterations = 0
        self.physical_time = 0.0
        self.acoustic_dt = 0.0
        self.total_substeps = 0

    @property
    def ctx(self):
        return self.sph_system.ctx

    def relax(self):
        """Advection dt, density summation and the acoustic sub-steps of one advection step."""
        advection_dt = self.fluid_advection_time_step.exec()
        self.fluid_density_by_summation.exec()
        relaxation_time = 0.0
        dt = self.acoustic_dt
        substeps = 0
        while relaxation_time < advection_dt:
            if self.case.loop_style == 0:
                dt = self.fluid_acoustic_time_step.exec()
            self.fluid_pressure_relaxation.exec(dt)
            self.fluid_density_relaxation.exec(dt)
            if self.case.loop_style == 1:
                dt = self.fluid_acoustic_time_step.exec()
            relaxation_time += dt
            self.physical_time += dt
            substeps += 1
        self.acoustic_dt = dt
        self.total_substeps += substeps
        return substeps, advection_dt

    def update_configuration(self):
        """Particle sort every 100 steps, then cell list and configuration update."""
        self.number_of_iterations += 1
        if self.number_of_iterations % 100 == 0 and self.number_of_iterations != 1:
            self.particle_sorting.exec()
        self.water_block.updateCellLinkedList()
        self.water_wall_complex.updateConfiguration()
        if self.fluid_observer.n:
            self.fluid_observer_contact.updateConfiguration()

    def advection_step(self, observe: bool = False):
        substeps, Dt = self.relax()
        obs, energy = None, None
        if observe:
            obs = self.recorded_pressure.exec() if self.fluid_observer.n else np.zeros(0)
            energy = self.mechanical_energy.exec()
        self.update_configuration()
        return substeps, Dt, obs, energy


class MixedPrecisionDamBreak:
    """The same dam break advanced by the mixed-precision fused solver (sphx_mp_*).

    Set-up is the FP64 one of ``DamBreak`` (bodies, relations, gravity, normals); the
    solver then takes the FP64 state over.  ``sync_fp64`` writes the state back into the
    FP64 fluid body (and refreshes its cell list and observer relation) for outputs.
    """

    def __init__(self, case: DamBreakCase, device: int = 0, block: int = 128, strategy: int = 0):
        import ctypes as C
        from . import native as N
        self._C, self._N = C, N
        self.fp64 = DamBreak(case, device=device)
        self.case = case
        sim = self.fp64
        g = np.zeros(3)
        g[: case.dim] = case.gravity[: case.dim]
        self._g = g
        h = C.c_void_p()
        N.call("sphx_mp_create", sim.water_block_inner.handle, sim.water_wall_contact.handle,
               C.byref(sim.fluid_advection_time_step.params), g.ctypes.data_as(C.POINTER(C.c_double)),
               C.byref(h))
        self.handle = h
        self.set_tuning(block, strategy)
        self.physical_time = 0.0
        self.number_of_iterations = 0
        self.total_substeps = 0

    @property
    def ctx(self):
        return self.fp64.ctx

    @property
    def n_fluid(self) -> int:
        return self.fp64.water_block.n

    def set_tuning(self, block: int, strategy: int) -> None:
        self._N.call("sphx_mp_set_tuning", self.handle, int(block), int(strategy))

    def set_tile(self, tx: int, ty: int, tz: int = 0) -> None:
        """Tile-grouped traversal (sphx_mp_set_tile); 0, 0, 0 keeps the cell order."""
        self._N.call("sphx_mp_set_tile", self.handle, int(tx), int(ty), int(tz))

    def advection_step(self):
        C, N = self._C, self._N
        sub = C.c_int()
        Dt = C.c_double()
        t = C.c_double()
        N.call("sphx_mp_advection_step", self.handle, self.case.loop_style, C.byref(sub), C.byref(Dt), C.byref(t))
        self.physical_time = t.value
        self.number_of_iterations += 1
        self.total_substeps += sub.value
        return sub.value, Dt.value

    def autotune(self, reps: int = 3):
        """Picks the fastest block size, neighbour strategy and tile shape on the current
        state; returns (block, strategy, ms per sub-step)."""
        C = self._C
        b, st, ms = C.c_int(), C.c_int(), C.c_double()
        self._N.call("sphx_mp_autotune", self.handle, int(reps), C.byref(b), C.byref(st), C.byref(ms))
        return b.value, st.value, ms.value

    def tuning(self) -> dict:
        """Current block size, strategy and tile shape (sphx_mp_get_tuning)."""
        C = self._C
        b, st = C.c_int(), C.c_int()
        t = (C.c_int * 3)()
        self._N.call("sphx_mp_get_tuning", self.handle, C.byref(b), C.byref(st), t)
        return {"block": b.value, "strategy": st.value, "tile": list(t)}

    def set_profiling(self, on: bool) -> None:
        self._N.call("sphx_mp_set_profiling", self.handle, int(on))

    def kernel_times(self):
        """(ms per 1st-half sweep, ms per 2nd-half sweep) averaged over the recorded sweeps."""
        C = self._C
        out = np.zeros(4)
        self._N.call("sphx_mp_kernel_times", self.handle, out.ctypes.data_as(C.POINTER(C.c_double)))
        return out[0] / max(out[1], 1), out[2] / max(out[3], 1), int(out[1])

    def list_sizes(self):
        C = self._C
        out = np.zeros(6, dtype=np.uint64)
        self._N.call("sphx_mp_list_sizes", self.handle, out.ctypes.data_as(C.POINTER(C.c_uint64)))
        return dict(n=int(out[0]), nw=int(out[1]), nnz_inner=int(out[2]), nnz_wall=int(out[3]),
                    cap_inner=int(out[4]), cap_wall=int(out[5]))

    def upload(self, body) -> None:
        """Reloads the solver from an FP64 fluid body (sphx_mp_upload)."""
        self._N.call("sphx_mp_upload", self.handle, body.handle)

    def download(self, body) -> None:
        """Writes the solver state into an FP64 fluid body (sphx_mp_download)."""
        self._N.call("sphx_mp_download", self.handle, body.handle)

    def upload_host(self, position, velocity, force, density, density_change_rate) -> None:
        """Loads the solver from host rows in the body's particle order
        (sphx_mp_upload_host): C-contiguous float64 arrays, n x dim for the vectors."""
        rows = [position, velocity, force, density, density_change_rate]
        for a, nc in zip(rows, (self.case.dim, self.case.dim, self.case.dim, 1, 1)):
            if a.dtype != np.float64 or not a.flags["C_CONTIGUOUS"] or a.size != self.n_fluid * nc:
                raise ValueError("host rows must be C-contiguous float64 of the fluid's size")
        C = self._C
        self._N.call("sphx_mp_upload_host", self.handle, *[C.c_void_p(a.ctypes.data) for a in rows])

    def download_host(self, position, velocity, density, pressure) -> None:
        """Writes position, velocity, density and pressure rows into host arrays
        (sphx_mp_download_host)."""
        rows = [position, velocity, density, pressure]
        for a, nc in zip(rows, (self.case.dim, self.case.dim, 1, 1)):
            if a.dtype != np.float64 or not a.flags["C_CONTIGUOUS"] or a.size != self.n_fluid * nc:
                raise ValueError("host rows must be C-contiguous float64 of the fluid's size")
        C = self._C
        self._N.call("sphx_mp_download_host", self.handle, *[C.c_void_p(a.ctypes.data) for a in rows])

    def set_host_rows(self, position=None, velocity=None, density=None, pressure=None) -> None:
        """Registers host rows (the layout of download_host) that every later advection
        step fills with its final state (sphx_mp_set_host_rows); no arguments unregister.
        The arrays are kept referenced while registered."""
        rows = [position, velocity, density, pressure]
        C = self._C
        if all(a is None for a in rows):
            self._N.call("sphx_mp_set_host_rows", self.handle, None, None, None, None)
            self._host_rows = None
            return
        for a, nc in zip(rows, (self.case.dim, self.case.dim, 1, 1)):
            if (a is None or a.dtype != np.float64 or not a.flags["C_CONTIGUOUS"]
                    or a.size != self.n_fluid * nc):
                raise ValueError("host rows must be C-contiguous float64 of the fluid's size")
        self._N.call("sphx_mp_set_host_rows", self.handle, *[C.c_void_p(a.ctypes.data) for a in rows])
        self._host_rows = rows

    def sync_fp64(self) -> None:
        sim = self.fp64
        self._N.call("sphx_mp_download", self.handle, sim.water_block.handle)
        sim.water_block.updateCellLinkedList()
        if sim.fluid_observer.n:
            sim.fluid_observer_contact.updateConfiguration()

    def observe_pressure(self) -> np.ndarray:
        self.sync_fp64()
        return self.fp64.recorded_pressure.exec()

    # The FP64 body doubles as the FP64 reference run in the benchmark; these views write
    # the mixed state into a scratch body so that the FP64 body stays untouched.
    def _scratch(self):
        if getattr(self, "_scratch_body", None) is None:
            from . import sph as S
            sim = self.fp64
            body = S.FluidBody(sim.sph_system, sim.water_block.shape)
            body.defineMatterMaterial(sim.water_block.material)
            body.generateParticles(S.Lattice)
            body.upload("Mass", sim.water_block.download("Mass"))
            self._scratch_body = body
            self._scratch_obs = S.ContactRelation(sim.fluid_observer, [body]) if sim.fluid_observer.n else None
        self._N.call("sphx_mp_download", self.handle, self._scratch_body.handle)
        return self._scratch_body

    def fp64_view(self, name: str) -> np.ndarray:
        return self._scratch().download(name)

    def observe_pressure_view(self) -> np.ndarray:
        body = self._scratch()
        if self._scratch_obs is None:
            return np.zeros(0)
        from . import sph as S
        body.updateCellLinkedList()
        self._scratch_obs.updateConfiguration()
        return S.ObservedQuantityRecording("Pressure", self._scratch_obs).exec()

    def conservation(self) -> np.ndarray:
        C = self._C
        out = np.zeros(5)
        self._N.call("sphx_mp_conservation", self.handle, out.ctypes.data_as(C.POINTER(C.c_double)))
        return out

    def check_state(self):
        """(particles with a non-finite value, finite particles outside the mesh) of the
        solver state (sphx_mp_check_state)."""
        C = self._C
        nf, om = C.c_uint64(), C.c_uint64()
        st = self._N.load().sphx_mp_check_state(self.handle, C.byref(nf), C.byref(om))
        if st not in (self._N.SPHX_OK, 7):  # 7: SPHX_ERR_NUMERIC, reported through the counts
            self._N.check(st)
        return int(nf.value), int(om.value)

    def upper_front(self, axis: int, lower, upper) -> float:
        C = self._C
        lo = np.zeros(3)
        up = np.zeros(3)
        lo[: len(lower)] = lower
        up[: len(upper)] = upper
        out = C.c_double()
        pd = C.POINTER(C.c_double)
        self._N.call("sphx_mp_upper_front", self.handle, axis, lo.ctypes.data_as(pd), up.ctypes.data_as(pd),
                     C.byref(out))
        return out.value

    def __del__(self):
        if getattr(self, "handle", None) is not None and self._N._lib is not None:
            self._N._lib.sphx_mp_destroy(self.handle)
            self.handle = None


class DamBreakCK:
    """The dam break with the CK particle methods of
    tests/tests_sycl/2d_examples/test_2d_dambreak_sycl/dambreak_sycl.cpp (FP64 on the CUDA
    policy): set-up as ``DamBreak`` (bodies, relations, normals, gravity), then the CK
    loop: every pass one acoustic step (AcousticTimeStepCK, both halves) and, when the
    advection trigger fires, UpdateParticlePosition and the configuration update with
    density regularization, advection-step set-up and correction matrices.  The driver's
    Morton re-sort only permutes particles and is not applied."""

    def __init__(self, case: DamBreakCase, device: int = 0):
        self.fp64 = DamBreak(case, device=device)
        self.case = case
        sim = self.fp64
        f, inner, contact = sim.water_block, sim.water_block_inner, sim.water_wall_contact
        self.water_block = f
        self.correction = S.LinearCorrectionMatrixCK(inner, contact, 0.5)
        self.first_half = S.AcousticStep1stHalfCK(inner, contact)
        self.second_half = S.AcousticStep2ndHalfCK(inner, contact)
        self.regularization = S.DensityRegularizationCK(inner, contact)
        self.setup = S.AdvectionStepSetupCK(f)
        self.update_position = S.UpdateParticlePositionCK(f)
        self.acoustic_dt = S.AcousticTimeStepCK(f)
        self.advection_dt = S.AdvectionTimeStepCK(f, case.U_ref)
        self.observe = S.ObservingQuantityCK(sim.fluid_observer_contact, "Pressure")
        # dambreak_sycl.cpp:156-169: trigger from the initial state, then the set-up passes
        self.advection_trigger = S.TriggerByInterval(self.advection_dt.exec())
        self.regularization.exec()
        self.setup.exec()
        self.correction.exec()
        self.physical_time = 0.0
        self.advection_steps = 1  # RestartStep() + 1
        self.acoustic_steps = 0

    def acoustic_step(self) -> bool:
        """One loop pass up to the trigger; True when an advection step fell due (positions
        moved; observe, then call ``configuration``)."""
        dt = self.acoustic_dt.exec()
        self.physical_time += dt
        self.advection_trigger.increment(dt)
        self.first_half.exec(dt)
        self.second_half.exec(dt)
        self.acoustic_steps += 1
        if self.advection_trigger(self.advection_dt):
            self.advection_steps += 1
            self.update_position.exec()
            return True
        return False

    def configuration(self) -> None:
        sim = self.fp64
        self.water_block.updateCellLinkedList()
        sim.water_block_inner.updateConfiguration()
        sim.water_wall_contact.updateConfiguration()
        self.regularization.exec()
        self.setup.exec()
        self.correction.exec()

    def observe_pressure(self) -> np.ndarray:
        sim = self.fp64
        sim.water_block.updateCellLinkedList()
        sim.fluid_observer_contact.updateConfiguration()
        return self.observe.exec()

    def mechanical_energy(self) -> float:
        return self.fp64.mechanical_energy.exec()


class DamBreakCKNested:
    """The dam break with the CK particle methods in the nested-loop form of
    tests/tests_sycl/3d_examples/test_3d_dambreak_sycl/dambreak.cpp:155-224 (FP64 on the
    CUDA policy): per advection step CompressionSummation + DensityRegularization,
    AdvectionStepSetup, AdvectionTimeStepCK, the free-surface indicator, the correction
    matrices, then acoustic sub-steps (acoustic dt first) until the advection dt is
    covered, UpdateParticlePosition, cell list and relations.  The driver's Morton re-sort
    only permutes particles and is not applied."""

    def __init__(self, case: DamBreakCase, device: int = 0):
        self.fp64 = DamBreak(case, device=device)
        self.case = case
        sim = self.fp64
        f, inner, contact = sim.water_block, sim.water_block_inner, sim.water_wall_contact
        self.water_block = f
        self.regularization = S.DensityRegularizationCK(inner, contact)
        self.setup = S.AdvectionStepSetupCK(f)
        self.advection_dt = S.AdvectionTimeStepCK(f, case.U_ref)
        self.indication = S.FreeSurfaceIndicationCK(inner, contact)
        self.correction = S.LinearCorrectionMatrixCK(inner, contact, 0.5)
        self.acoustic_dt = S.AcousticTimeStepCK(f)
        self.first_half = S.AcousticStep1stHalfCK(inner, contact)
        self.second_half = S.AcousticStep2ndHalfCK(inner, contact)
        self.update_position = S.UpdateParticlePositionCK(f)
        self.observe = S.ObservingQuantityCK(sim.fluid_observer_contact, "Pressure")
        self.physical_time = 0.0
        self.number_of_iterations = 0

    def advection_step(self):
        sim = self.fp64
        self.regularization.exec()
        self.setup.exec()
        Dt = self.advection_dt.exec()
        self.indication.exec()
        self.correction.exec()
        relaxation, sub = 0.0, 0
        while relaxation < Dt:
            dt = self.acoustic_dt.exec()
            self.first_half.exec(dt)
            self.second_half.exec(dt)
            relaxation += dt
            self.physical_time += dt
            sub += 1
        self.update_position.exec()
        self.number_of_iterations += 1
        self.water_block.updateCellLinkedList()
        sim.water_block_inner.updateConfiguration()
        sim.water_wall_contact.updateConfiguration()
        if sim.fluid_observer.n:
            sim.fluid_observer_contact.updateConfiguration()
        return sub, Dt

    def observe_pressure(self) -> np.ndarray:
        return self.observe.exec()

    def mechanical_energy(self) -> float:
        return self.fp64.mechanical_energy.exec()


def _by_original_id(body, name: str) -> np.ndarray:
    """A variable in creation order (undoes the Morton re-sorts)."""
    v = body.download(name)
    out = np.empty_like(v)
    out[body.download("OriginalID").astype(np.int64)] = v
    return out


def mixed_vs_fp64(case: DamBreakCase, t_end: float, device: int = 0, record_every: int = 100,
                  realizations=("resorted", "perturbed")) -> dict:
    """Runs the mixed-precision solver until t_end, then the FP64 path the same number of
    advection steps from the same initial state, recording every `record_every` steps the
    wall-probe pressure, the free-surface height over the initial water column and the
    mechanical energy, and at the end the max-norm field errors (relative to the field
    maximum).  Further FP64 realizations give the spread of the flow itself at the same
    step count: "resorted" re-sorts the particles once before the first step (same
    physics, another neighbour summation order: perturbations at FP64 rounding),
    "perturbed" moves every initial position by up to 1e-7 h (seeded), the size of the
    FP32 rounding of the solver's in-cell offsets."""
    import time
    mp = MixedPrecisionDamBreak(case, device=device)
    vert = case.vertical_axis
    lo, up = list(case.sys_lower[: case.dim]), list(case.sys_upper[: case.dim])
    lo[0] = case.water_center[0] - case.water_halfsize[0]
    up[0] = case.water_center[0] + case.water_halfsize[0]
    fields = ("Position", "Velocity", "Density", "Pressure")

    def sample_mixed():
        return {"t": mp.physical_time, "probe_pressure": [float(x) for x in mp.observe_pressure_view()],
                "free_surface_height": mp.upper_front(vert, lo, up),
                "mechanical_energy": float(mp.conservation()[4])}

    series = {"mixed": [sample_mixed()]}
    t0 = time.perf_counter()
    steps = 0
    while mp.physical_time < t_end:
        mp.advection_step()
        steps += 1
        if steps % record_every == 0:
            series["mixed"].append(sample_mixed())
    wall = {"mixed": time.perf_counter() - t0}
    if steps % record_every:
        series["mixed"].append(sample_mixed())
    end = {"mixed": {nm: mp.fp64_view(nm) for nm in fields}}  # creation order

    def sample_fp64(sim):
        return {"t": sim.physical_time, "probe_pressure": [float(x) for x in sim.recorded_pressure.exec()],
                "free_surface_height": S.UpperFrontInAxisDirection(sim.water_block, lo, up, vert).exec(),
                "mechanical_energy": sim.mechanical_energy.exec()}

    def run_fp64(name, sim):
        if name == "resorted":
            sim.particle_sorting.exec()
        elif name == "perturbed":
            x = sim.water_block.download("Position")
            rng = np.random.default_rng(0)
            sim.water_block.upload("Position", x + 1e-7 * case.h * rng.uniform(-1.0, 1.0, x.shape))
        if name != "fp64":
            sim.update_configuration()
            sim.number_of_iterations = 0
        series[name] = [sample_fp64(sim)]
        t1 = time.perf_counter()
        for k in range(1, steps + 1):
            sim.advection_step()
            if k % record_every == 0:
                series[name].append(sample_fp64(sim))
        wall[name] = time.perf_counter() - t1
        if steps % record_every:
            series[name].append(sample_fp64(sim))
        end[name] = {nm: _by_original_id(sim.water_block, nm) for nm in fields}

    run_fp64("fp64", mp.fp64)
    del mp
    for name in realizations:
        run_fp64(name, DamBreak(case, device=device))

    def diff(a, b):
        sa, sb = series[a], series[b]
        rows = [{"t": x["t"], "probe_pressure_abs": [abs(p - q) for p, q in zip(x["probe_pressure"], y["probe_pressure"])],
                 "free_surface_rel": abs(x["free_surface_height"] / y["free_surface_height"] - 1.0),
                 "mechanical_energy_rel": abs(x["mechanical_energy"] / y["mechanical_energy"] - 1.0)}
                for x, y in zip(sa, sb)]
        fe = {nm + "_max_rel": float(np.max(np.abs(end[a][nm] - end[b][nm])) / max(np.max(np.abs(end[b][nm])), 1e-300))
              for nm in fields}
        return {"series": rows, "end_fields": fe}

    return {"workload": case.name, "t_end": t_end, "advection_steps": steps, "record_every": record_every,
            "wall_s": wall, "series": series,
            "vs_fp64": {name: diff(name, "fp64") for name in ("mixed",) + tuple(realizations)}}


if __name__ == "__main__":
    import argparse
    import json

    from .cases import dambreak_2d, dambreak_3d
    ap = argparse.ArgumentParser(description="Dam break: mixed precision against FP64 at a given time")
    ap.add_argument("--dim", type=int, default=3)
    ap.add_argument("--dp", type=float, default=0.006)
    ap.add_argument("--t-end", type=float, default=2.0)
    ap.add_argument("--record-every", type=int, default=100)
    ap.add_argument("--run", default=None, choices=["fp64", "mixed"],
                    help="only advance one solver to t_end and report its throughput")
    ap.add_argument("--out", default=None)
    ap.add_argument("--block", type=int, default=128, help="mixed solver: sweep block size")
    ap.add_argument("--strategy", type=int, default=0, help="mixed solver: neighbour strategy 0-6")
    ap.add_argument("--tile", type=int, nargs=3, default=None, help="mixed solver: tile shape (sub-cells)")
    a = ap.parse_args()
    c = dambreak_3d(a.dp) if a.dim == 3 else dambreak_2d(a.dp)
    if a.run:
        import time
        if a.run == "mixed":
            sim = MixedPrecisionDamBreak(c, block=a.block, strategy=a.strategy)
            if a.tile:
                sim.set_tile(*a.tile)
        else:
            sim = DamBreak(c)
        n = sim.n_fluid if a.run == "mixed" else sim.water_block.n
        t0, steps, subs = time.perf_counter(), 0, 0
        while sim.physical_time < a.t_end:
            subs += sim.advection_step()[0]
            steps += 1
        wall = time.perf_counter() - t0
        text = json.dumps({"workload": c.name, "solver": a.run, "n_fluid": n, "t": sim.physical_time,
                           "advection_steps": steps, "acoustic_substeps": subs, "wall_s": wall,
                           "particle_steps_per_s": n * subs / wall})
    else:
        text = json.dumps(mixed_vs_fp64(c, a.t_end, record_every=a.record_every))
    if a.out:
        with open(a.out, "w") as f:
            f.write(text)
    else:
        print(text)
