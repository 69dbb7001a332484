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
