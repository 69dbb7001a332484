/**
 * 2D dam break on the GB300 execution policy.  Same case, object names and main loop as
 * the reference example tests/2d_examples/test_2d_dambreak/Dambreak.cpp, compiled against
 * sphinxsys_gb300/host/sphinxsys_cuda.h and libsphx_cuda.so.  The regression recorders
 * write the .dat series under ./output and, after a run to the end time, run the
 * reference's dynamic-time-warping test against ./input (exit status 1 on failure); stdout
 * carries "observe <step> <time> <p> <E>" at the reference's observation interval and
 * "final <step> <time> <p> <E>".  VTP and restart output are left out.
 *
 * usage: dambreak_2d [end_time] [max_iterations]
 */
#include <cstdio>
#include <cstdlib>

#define SPHX_DIMENSION 2
#include "sphinxsys_cuda.h"
using namespace SPH;

Real DL = 5.366;
Real DH = 5.366;
Real LL = 2.0;
Real LH = 1.0;
Real particle_spacing_ref = 0.025;
Real BW = particle_spacing_ref * 4;
Real rho0_f = 1.0;
Real gravity_g = 1.0;
Real U_ref = 2.0 * sqrt(gravity_g * LH);
Real c_f = 10.0 * U_ref;
Vec2d water_block_halfsize = Vec2d(0.5 * LL, 0.5 * LH);
Vec2d water_block_translation = water_block_halfsize;
Vec2d outer_wall_halfsize = Vec2d(0.5 * DL + BW, 0.5 * DH + BW);
Vec2d outer_wall_translation = Vec2d(-BW, -BW) + outer_wall_halfsize;
Vec2d inner_wall_halfsize = Vec2d(0.5 * DL, 0.5 * DH);
Vec2d inner_wall_translation = inner_wall_halfsize;

class WallBoundary : public ComplexShape
{
  public:
    explicit WallBoundary(const std::string &shape_name) : ComplexShape(shape_name)
    {
        add<GeometricShapeBox>(Transform(outer_wall_translation), outer_wall_halfsize);
        subtract<GeometricShapeBox>(Transform(inner_wall_translation), inner_wall_halfsize);
    }
};

int main(int ac, char *av[])
{
    Real end_time = ac > 1 ? atof(av[1]) : 20.0;
    long max_iterations = ac > 2 ? atol(av[2]) : -1;
    try
    {
        BoundingBoxd system_domain_bounds(Vec2d(-BW, -BW), Vec2d(DL + BW, DH + BW));
        SPHSystem sph_system(system_domain_bounds, particle_spacing_ref);
        sph_system.handleCommandlineOptions(ac, av);

        GeometricShapeBox initial_water_block(Transform(water_block_translation), water_block_halfsize, "WaterBody");
        FluidBody water_block(sph_system, initial_water_block);
        water_block.defineMatterMaterial<WeaklyCompressibleFluid>(rho0_f, c_f);
        water_block.generateParticles<BaseParticles, Lattice>();

        SolidBody wall_boundary(sph_system, makeShared<WallBoundary>("WallBoundary"));
        wall_boundary.defineMatterMaterial<Solid>();
        wall_boundary.generateParticles<BaseParticles, Lattice>();

        ObserverBody fluid_observer(sph_system, "FluidObserver");
        StdVec<Vecd> observation_location = {Vecd(DL, 0.2)};
        fluid_observer.generateParticles<ObserverParticles>(observation_location);

        InnerRelation water_block_inner(water_block);
        ContactRelation water_wall_contact(water_block, {&wall_boundary});
        ContactRelation fluid_observer_contact(fluid_observer, {&water_block});
        ComplexRelation water_wall_complex(water_block_inner, water_wall_contact);

        Gravity gravity(Vecd(0.0, -gravity_g));
        SimpleDynamics<GravityForce<Gravity>> constant_gravity(water_block, gravity);
        SimpleDynamics<NormalDirectionFromBodyShape> wall_boundary_normal_direction(wall_boundary);

        Dynamics1Level<fluid_dynamics::Integration1stHalfWithWallRiemann> fluid_pressure_relaxation(water_block_inner, water_wall_contact);
        Dynamics1Level<fluid_dynamics::Integration2ndHalfWithWallRiemann> fluid_density_relaxation(water_block_inner, water_wall_contact);
        InteractionWithUpdate<fluid_dynamics::DensitySummationComplexFreeSurface> fluid_density_by_summation(water_block_inner, water_wall_contact);

        ReduceDynamics<fluid_dynamics::AdvectionTimeStep> fluid_advection_time_step(water_block, U_ref);
        ReduceDynamics<fluid_dynamics::AcousticTimeStep> fluid_acoustic_time_step(water_block);
        ParticleSorting particle_sorting(water_block);
        TotalMechanicalEnergy water_mechanical_energy(water_block, gravity);
        ObservedQuantity recorded_water_pressure("Pressure", fluid_observer_contact);
        RegressionTestDynamicTimeWarping<ReducedQuantityRecording<TotalMechanicalEnergy>> write_water_mechanical_energy(
            water_block, gravity);
        RegressionTestDynamicTimeWarping<ObservedQuantityRecording<Real>> write_recorded_water_pressure(
            "Pressure", fluid_observer_contact);

        sph_system.initializeSystemCellLinkedLists();
        sph_system.initializeSystemConfigurations();
        wall_boundary_normal_direction.exec();
        constant_gravity.exec();

        Real &physical_time = *sph_system.getSystemVariableDataByName<Real>("PhysicalTime");
        size_t number_of_iterations = 0;
        int screen_output_interval = 100;
        int observation_sample_interval = screen_output_interval * 2;
        Real output_interval = 0.1;
        write_water_mechanical_energy.writeToFile(number_of_iterations);
        write_recorded_water_pressure.writeToFile(number_of_iterations);
        printf("observe %zu %.17g %.17g %.17g\n", number_of_iterations, physical_time,
               recorded_water_pressure.exec()[0], water_mechanical_energy.exec());
        bool cut_short = false;
        while (physical_time < end_time)
        {
            Real integration_time = 0.0;
            while (integration_time < output_interval)
            {
                Real advection_dt = fluid_advection_time_step.exec();
                fluid_density_by_summation.exec();
                Real relaxation_time = 0.0;
                Real acoustic_dt = 0.0;
                while (relaxation_time < advection_dt)
                {
                    acoustic_dt = fluid_acoustic_time_step.exec();
                    fluid_pressure_relaxation.exec(acoustic_dt);
                    fluid_density_relaxation.exec(acoustic_dt);
                    relaxation_time += acoustic_dt;
                    integration_time += acoustic_dt;
                    physical_time += acoustic_dt;
                }
                if (number_of_iterations % screen_output_interval == 0 &&
                    number_of_iterations % observation_sample_interval == 0 && number_of_iterations != 0)
                {
                    write_water_mechanical_energy.writeToFile(number_of_iterations);
                    write_recorded_water_pressure.writeToFile(number_of_iterations);
                    printf("observe %zu %.17g %.17g %.17g\n", number_of_iterations, physical_time,
                           recorded_water_pressure.exec()[0], water_mechanical_energy.exec());
                }
                number_of_iterations++;
                if (number_of_iterations % 100 == 0 && number_of_iterations != 1)
                    particle_sorting.exec();
                water_block.updateCellLinkedList();
                water_wall_complex.updateConfiguration();
                fluid_observer_contact.updateConfiguration();
                cut_short = max_iterations >= 0 && long(number_of_iterations) >= max_iterations;
                if (cut_short)
                    break;
            }
            if (cut_short)
                break;
        }
        printf("final %zu %.17g %.17g %.17g\n", number_of_iterations, physical_time,
               recorded_water_pressure.exec()[0], water_mechanical_energy.exec());
        if (sph_system.GenerateRegressionData())
        {
            write_water_mechanical_energy.generateDataBase(1.0e-3);
            write_recorded_water_pressure.generateDataBase(1.0e-3);
        }
        else if (!cut_short)
        {
            write_water_mechanical_energy.testResult();
            write_recorded_water_pressure.testResult();
        }
    }
    catch (const SphxException &e)
    {
        fprintf(stderr, "%s\n", e.what());
        return 1;
    }
    return 0;
}
