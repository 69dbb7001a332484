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
