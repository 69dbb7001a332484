/**
 * 2D Taylor-Green vortex on the GB300 execution policy.  Same case, object names and main
 * loop as the reference example tests/2d_examples/test_2d_taylor_green/taylor_green.cpp,
 * compiled against sphinxsys_gb300/host/sphinxsys_cuda.h and libsphx_cuda.so.  The water
 * block is the box [0, DL] x [0, DH] (the reference describes the same box as a polygon).
 * File output (VTP, reload, regression databases) is replaced by printing the total kinetic
 * energy and the maximum speed at the reference's output interval.
 *
 * usage: taylor_green_2d [end_time] [max_iterations] [resolution]
 */
#include <cstdio>
#include <cstdlib>

#define SPHX_DIMENSION 2
#include "sphinxsys_cuda.h"
using namespace SPH;

Real DL = 1.0;
Real DH = 1.0;
Real global_resolution = 1.0 / 100.0;
Real rho0_f = 1.0;
Real U_f = 1.0;
Real c_f = 10.0 * U_f;
Real Re = 100;
Real mu_f = rho0_f * U_f * DL / Re;

class WaterBlock : public ComplexShape
{
  public:
    explicit WaterBlock(const std::string &shape_name) : ComplexShape(shape_name)
    {
        Vec2d halfsize(0.5 * DL, 0.5 * DH);
        add<GeometricShapeBox>(Transform(halfsize), halfsize);
    }
};

// taylor_green.cpp:43-56: the initial velocity profile
struct TaylorGreenInitialCondition
{
    static Vecd velocity(const Vecd &x)
    {
        return Vecd(-cos(2.0 * Pi * x[0]) * sin(2.0 * Pi * x[1]), sin(2.0 * Pi * x[0]) * cos(2.0 * Pi * x[1]));
    }
};

int main(int ac, char *av[])
{
    Real end_time = ac > 1 ? atof(av[1]) : 5.0;
    long max_iterations = ac > 2 ? atol(av[2]) : -1;
    if (ac > 3)
        global_resolution = 1.0 / atof(av[3]);
    try
    {
        BoundingBoxd system_domain_bounds(Vec2d(0.0, 0.0), Vec2d(DL, DH));
        SPHSystem sph_system(system_domain_bounds, global_resolution);
        sph_system.handleCommandlineOptions(ac, av);

        FluidBody water_block(sph_system, makeShared<WaterBlock>("WaterBody"));
        water_block.defineMatterMaterial<WeaklyCompressibleFluid>(rho0_f, c_f);
        water_block.addMaterialProperty<Viscosity>(mu_f);
        water_block.generateParticles<BaseParticles, Lattice>();

        InnerRelation water_block_inner(water_block);

        SimpleDynamics<TaylorGreenInitialCondition> initial_condition(water_block);
        Dynamics1Level<fluid_dynamics::Integration1stHalfInnerRiemann> pressure_relaxation(water_block_inner);
        Dynamics1Level<fluid_dynamics::Integration2ndHalfInnerNoRiemann> density_relaxation(water_block_inner);
        InteractionWithUpdate<fluid_dynamics::DensitySummationInner> update_density_by_summation(water_block_inner);
        InteractionWithUpdate<fluid_dynamics::ViscousForceInner> viscous_force(water_block_inner);
        InteractionWithUpdate<fluid_dynamics::TransportVelocityCorrectionInner<TruncatedLinear, AllParticles>>
            transport_velocity_correction(water_block_inner);
        ReduceDynamics<fluid_dynamics::AdvectionViscousTimeStep> get_fluid_advection_time_step_size(water_block, U_f);
        ReduceDynamics<fluid_dynamics::AcousticTimeStep> get_fluid_time_step_size(water_block);
        PeriodicAlongAxis periodic_along_x(water_block.getSPHBodyBounds(), xAxis);
        PeriodicAlongAxis periodic_along_y(water_block.getSPHBodyBounds(), yAxis);
        PeriodicConditionUsingCellLinkedList periodic_condition_x(water_block, periodic_along_x);
        PeriodicConditionUsingCellLinkedList periodic_condition_y(water_block, periodic_along_y);
        TotalKineticEnergy write_total_kinetic_energy(water_block);
        MaximumSpeed write_maximum_speed(water_block);

        initial_condition.exec();
        sph_system.initializeSystemCellLinkedLists();
        periodic_condition_x.update_cell_linked_list_.exec();
        periodic_condition_y.update_cell_linked_list_.exec();
        sph_system.initializeSystemConfigurations();

        Real &physical_time = *sph_system.getSystemVariableDataByName<Real>("PhysicalTime");
        long number_of_iterations = 0;
        Real output_interval = 0.1;
        Real dt = 0.0;
        printf("output 0 %.17g %.17g\n", physical_time, write_total_kinetic_energy.exec());
        while (physical_time < end_time && (max_iterations < 0 || number_of_iterations < max_iterations))
        {
            Real integration_time = 0.0;
            while (integration_time < output_interval && (max_iterations < 0 || number_of_iterations < max_iterations))
            {
                Real Dt = get_fluid_advection_time_step_size.exec();
                update_density_by_summation.exec();
                viscous_force.exec();
                transport_velocity_correction.exec();

                Real relaxation_time = 0.0;
                while (relaxation_time < Dt)
                {
                    // avoid possible smaller acoustic time step size for viscous flow
                    dt = std::min(get_fluid_time_step_size.exec(), Dt);
                    relaxation_time += dt;
                    integration_time += dt;
                    pressure_relaxation.exec(dt);
                    density_relaxation.exec(dt);
                    physical_time += dt;
                }
                number_of_iterations++;

                periodic_condition_x.bounding_.exec();
                periodic_condition_y.bounding_.exec();
                water_block.updateCellLinkedList();
                periodic_condition_x.update_cell_linked_list_.exec();
                periodic_condition_y.update_cell_linked_list_.exec();
                water_block_inner.updateConfiguration();
            }
            printf("output %ld %.17g %.17g %.17g\n", number_of_iterations, physical_time,
                   write_total_kinetic_energy.exec(), write_maximum_speed.exec());
        }
        printf("final %ld %.17g %.17g %.17g\n", number_of_iterations, physical_time, write_total_kinetic_energy.exec(),
               write_maximum_speed.exec());
    }
    catch (const SphxException &e)
    {
        fprintf(stderr, "%s\n", e.what());
        return 1;
    }
    return 0;
}
