"""Taylor-Green vortex on the CUDA execution policy (FP64).

``TaylorGreen(case)`` sets the case up as tests/2d_examples/test_2d_taylor_green/
taylor_green.cpp:57-107 does (lattice particles in the periodic box, the vortex velocity,
viscosity mu = rho0 U L / Re, periodic conditions along every axis) and ``advection_step``
runs one pass of its loop (taylor_green.cpp:133-164): AdvectionViscousTimeStep,
DensitySummationInner, ViscousForceInner, TransportVelocityCorrectionInner, the acoustic
sub-steps with dt = min(AcousticTimeStep, Dt), then periodic bounding, cell list with
periodic images and the inner configuration."""
from __future__ import annotations

import math

import numpy as np

from . import sph as S
from .cases import TaylorGreenCase


def initial_velocity(case: TaylorGreenCase, x: np.ndarray) -> np.ndarray:
    if case.velocity_kind == 0:  # taylor_green.cpp:34-44
        v = np.zeros_like(x)
        v[:, 0] = -np.cos(2.0 * math.pi * x[:, 0]) * np.sin(2.0 * math.pi * x[:, 1])
        v[:, 1] = np.sin(2.0 * math.pi * x[:, 0]) * np.cos(2.0 * math.pi * x[:, 1])
        return v
    v = np.zeros_like(x)
    v[:, 0] = np.sin(x[:, 0]) * np.cos(x[:, 1]) * np.cos(x[:, 2])
    v[:, 1] = -np.cos(x[:, 0]) * np.sin(x[:, 1]) * np.cos(x[:, 2])
    return v


class _Box:
    def __init__(self, dim: int, L: float):
        self.dim, self.L = dim, L

    def contain(self, x: np.ndarray) -> np.ndarray:
        return np.ones(len(x), dtype=bool)


class TaylorGreen:
    def __init__(self, case: TaylorGreenCase, device: int = 0):
        d = case.dim
        self.case = case
        lo, up = [0.0] * d, [case.L] * d
        self.sph_system = S.SPHSystem(lo, up, case.dp, device=device, h_spacing_ratio=case.h_ratio)
        self.water_block = S.FluidBody(self.sph_system, None, name="WaterBody")
        self.water_block.defineMatterMaterial(S.WeaklyCompressibleFluid(case.rho0, case.c0))
        S.addMaterialProperty(self.water_block, S.Viscosity(case.mu))
        x = S.lattice_positions(d, lo, up, case.dp, _Box(d, case.L))
        self.water_block.generateParticles(positions=x)
        self.water_block_inner = S.InnerRelation(self.water_block)
        f, inner = self.water_block, self.water_block_inner
        self.pressure_relaxation = S.Integration1stHalfInnerRiemann(inner)
        self.density_relaxation = S.Integration2ndHalfInnerNoRiemann(inner)
        self.update_density_by_summation = S.DensitySummationInnerDynamics(inner)
        self.viscous_force = S.ViscousForceInner(inner)
        self.transport_velocity_correction = S.TransportVelocityCorrectionInner(inner)
        self.advection_time_step = S.AdvectionViscousTimeStep(f, case.U)
        self.acoustic_time_step = S.ReduceDynamics(S.AcousticTimeStep, f)
        self.periodic = [S.PeriodicConditionUsingCellLinkedList(f, S.PeriodicAlongAxis(lo, up, a)) for a in range(d)]
        self.kinetic_energy = S.TotalKineticEnergy(f)
        self.maximum_speed = S.MaximumSpeed(f)
        f.upload("Velocity", initial_velocity(case, x))  # initial_condition.exec()
        # taylor_green.cpp:104-107
        f.updateCellLinkedList()
        for p in self.periodic:
            p.update_cell_linked_list_.exec()
        inner.updateConfiguration()
        self.physical_time = 0.0
        self.number_of_iterations = 0

    def advection_step(self):
        Dt = self.advection_time_step.exec()
        self.update_density_by_summation.exec()
        self.viscous_force.exec()
        self.transport_velocity_correction.exec()
        relaxation, sub = 0.0, 0
        while relaxation < Dt:
            dt = min(self.acoustic_time_step.exec(), Dt)
            relaxation += dt
            self.pressure_relaxation.exec(dt)
            self.density_relaxation.exec(dt)
            self.physical_time += dt
            sub += 1
        self.number_of_iterations += 1
        for p in self.periodic:
            p.bounding_.exec()
        self.water_block.updateCellLinkedList()
        for p in self.periodic:
            p.update_cell_linked_list_.exec()
        self.water_block_inner.updateConfiguration()
        return sub, Dt


class MixedPrecisionTaylorGreen:
    """The same periodic flow advanced by the mixed-precision solver
    (sphx_mp_create_periodic): the FP64 body holds the initial lattice state only (no FP64
    cell list or relation is built, so the case can be as large as the solver's own
    memory allows); ``download`` writes the solver state into it."""

    def __init__(self, case: TaylorGreenCase, device: int = 0, block: int = 128, strategy: int = 0):
        import ctypes as C
        from . import native as N
        self._C, self._N = C, N
        d = case.dim
        self.case = case
        lo, up = [0.0] * d, [case.L] * d
        self.sph_system = S.SPHSystem(lo, up, case.dp, device=device, h_spacing_ratio=case.h_ratio)
        self.water_block = S.FluidBody(self.sph_system, None, name="WaterBody")
        self.water_block.defineMatterMaterial(S.WeaklyCompressibleFluid(case.rho0, case.c0))
        S.addMaterialProperty(self.water_block, S.Viscosity(case.mu))
        x = S.lattice_positions(d, lo, up, case.dp, _Box(d, case.L))
        self.water_block.generateParticles(positions=x)
        self.water_block.upload("Velocity", initial_velocity(case, x))
        del x
        params = S.fluid_params(self.water_block, U_ref=case.U)
        params.limiter_slope = 0.0  # Integration2ndHalfInnerNoRiemann
        self._params = params
        l3, u3 = np.zeros(3), np.zeros(3)
        u3[:d] = case.L
        h = C.c_void_p()
        N.call("sphx_mp_create_periodic", self.water_block.handle, C.byref(params),
               l3.ctypes.data_as(C.POINTER(C.c_double)), u3.ctypes.data_as(C.POINTER(C.c_double)), case.mu, 0.2,
               C.byref(h))
        self.handle = h
        N.call("sphx_mp_set_tuning", h, int(block), int(strategy))
        self.physical_time = 0.0
        self.number_of_iterations = 0
        self.total_substeps = 0

    @property
    def n_fluid(self) -> int:
        return self.water_block.n

    def set_tuning(self, block: int, strategy: int) -> None:
        self._N.call("sphx_mp_set_tuning", self.handle, int(block), int(strategy))

    def autotune(self, reps: int = 3):
        C = self._C
        b, st, ms = C.c_int(), C.c_int(), C.c_double()
        self._N.call("sphx_mp_autotune", self.handle, int(reps), C.byref(b), C.byref(st), C.byref(ms))
        return b.value, st.value, ms.value

    def set_profiling(self, on: bool) -> None:
        self._N.call("sphx_mp_set_profiling", self.handle, int(on))

    def kernel_times(self):
        out = np.zeros(4)
        self._N.call("sphx_mp_kernel_times", self.handle, out.ctypes.data_as(self._C.POINTER(self._C.c_double)))
        return out[0] / max(out[1], 1), out[2] / max(out[3], 1), int(out[1])

    def list_sizes(self):
        out = np.zeros(6, dtype=np.uint64)
        self._N.call("sphx_mp_list_sizes", self.handle, out.ctypes.data_as(self._C.POINTER(self._C.c_uint64)))
        return dict(n=int(out[0]), nnz_inner=int(out[2]), cap_inner=int(out[4]))

    def advection_step(self):
        C, N = self._C, self._N
        sub, Dt, t = C.c_int(), C.c_double(), C.c_double()
        N.call("sphx_mp_advection_step", self.handle, 0, C.byref(sub), C.byref(Dt), C.byref(t))
        self.physical_time = t.value
        self.number_of_iterations += 1
        self.total_substeps += sub.value
        return sub.value, Dt.value

    def kinetic_energy(self) -> float:
        out = np.zeros(5)
        self._N.call("sphx_mp_conservation", self.handle, out.ctypes.data_as(self._C.POINTER(self._C.c_double)))
        return float(out[4])

    def download(self) -> None:
        self._N.call("sphx_mp_download", self.handle, self.water_block.handle)

    def maximum_speed(self) -> float:
        self.download()
        v = self.water_block.download("Velocity")
        return float(np.sqrt(np.max(np.sum(v * v, axis=1))))

    def __del__(self):
        if getattr(self, "handle", None) is not None and self._N._lib is not None:
            self._N._lib.sphx_mp_destroy(self.handle)
            self.handle = None


def run(case: TaylorGreenCase, steps: int, precision: str = "mixed", record_every: int = 10, device: int = 0):
    """Advances the vortex `steps` advection steps and records the kinetic energy every
    `record_every` steps (and at the start); returns the series with the wall time."""
    import time
    sim = MixedPrecisionTaylorGreen(case, device=device) if precision == "mixed" else TaylorGreen(case, device=device)
    energy = (lambda: sim.kinetic_energy()) if precision == "mixed" else (lambda: sim.kinetic_energy.exec())
    t, ke, subs = [0.0], [energy()], 0
    t0 = time.perf_counter()
    for k in range(1, steps + 1):
        s, _ = sim.advection_step()
        subs += s
        if k % record_every == 0 or k == steps:
            t.append(sim.physical_time)
            ke.append(energy())
    wall = time.perf_counter() - t0
    return {"workload": case.name, "precision": precision, "n_fluid": sim.water_block.n, "steps": steps,
            "acoustic_substeps": subs, "wall_s": wall, "t": t, "kinetic_energy": ke}


if __name__ == "__main__":
    import argparse
    import json

    from .cases import taylor_green_2d, taylor_green_3d
    ap = argparse.ArgumentParser(description="Taylor-Green vortex: kinetic-energy series on the CUDA policy")
    ap.add_argument("--dim", type=int, default=3)
    ap.add_argument("--resolution", type=int, default=256)
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64", "both"])
    ap.add_argument("--record-every", type=int, default=10)
    ap.add_argument("--out", default=None, help="JSON file for the series (default: stdout)")
    a = ap.parse_args()
    c = taylor_green_3d(a.resolution) if a.dim == 3 else taylor_green_2d(a.resolution)
    res = [run(c, a.steps, p, a.record_every) for p in (("mixed", "fp64") if a.precision == "both" else (a.precision,))]
    text = json.dumps(res)
    if a.out:
        with open(a.out, "w") as f:
            f.write(text)
    else:
        print(text)
