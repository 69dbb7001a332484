/**
 * 3D dam break with the classic dynamics on the GB300 execution policy: same case, object
 * names and main loop as the reference example tests/3d_examples/test_3d_dambreak/
 * dambreak.cpp, compiled against sphinxsys_gb300/host/sphinxsys_cuda.h and
 * libsphx_cuda.so.  The regression recorders write the .dat series under ./output and, at the end, run the
 * reference's dynamic-time-warping test against ./input (exit status 1 on failure) unless
 * the run was cut short by max_iterations; stdout carries "energy <step> <time> <E>" at
 * every output interval and "final <step> <time> <E>".
 *
 * usage: dambreak_3d [end_time] [max_iterations] [--state_recording=0|1]
 */
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#define SPHX_DIMENSION 3
#include "sphinxsys_cuda.h"
using namespace SPH;

Real global_resolution = 0.05;
Real BW = global_resolution * 4;
Real DL = 5.366;
Real DH = 2.0;
Real DW = 0.5;
Real LL = 2.0;
Real LH = 1.0;
Real LW = 0.5;
Real rho0_f = 1.0;
Real gravity_g = 1.0;
Real U_f = 2.0 * sqrt(gravity_g * LH);
Real c_f = 10.0 * U_f;

class WaterBlock : public ComplexShape
{
  public:
    explicit WaterBlock(const std::string &shape_name) : ComplexShape(shape_name)
    {
        Vecd halfsize_water(0.5 * LL, 0.5 * LH, 0.5 * LW);
        add<GeometricShapeBox>(Transform(halfsize_water), halfsize_water);
    }
};
class WallBoundary : public ComplexShape
{
  public:
    explicit WallBoundary(const std::string &shape_name) : ComplexShape(shape_name)
    {
        Vecd halfsize_outer(0.5 * DL + BW, 0.5 * DH + BW, 0.5 * DW + BW);
        Vecd halfsize_inner(0.5 * DL, 0.5 * DH, 0.5 * DW);
        add<GeometricShapeBox>(Transform(halfsize_inner), halfsize_outer);
        subtract<GeometricShapeBox>(Transform(halfsize_inner), halfsize_inner);
    }
};
StdVec<Vecd> createObservationPoints()
{
    StdVec<Vecd> observation_points;
    for (Real y : {0.01, 0.1, 0.2, 0.24, 0.252, 0.266})
        observation_points.push_back(Vecd(DL, y, 0.5 * DW));
    return observation_points;
}

int main(int ac, char *av[])
{
    std::vector<std::string> positional;
    for (int i = 1; i < ac; ++i)
        if (std::string(av[i]).rfind("--", 0) != 0)
            positional.push_back(av[i]);
    Real end_time = positional.size() > 0 ? atof(positional[0].c_str()) : 20.0;
    long max_iterations = positional.size() > 1 ? atol(positional[1].c_str()) : -1;
    try
    {
        BoundingBoxd system_domain_bounds(Vecd(-BW, -BW, -BW), Vecd(DL + BW, DH + BW, DW + BW));
        SPHSystem sph_system(system_domain_bounds, global_resolution);
        sph_system.handleCommandlineOptions(ac, av);
        WaterBlock initial_water_block("WaterBody");
        FluidBody water_block(sph_system, initial_water_block);
        water_block.defineMatterMaterial<WeaklyCompressibleFluid>(rho0_f, c_f);
        water_block.generateParticles<BaseParticles, Lattice>();

        SolidBody wall_boundary(sph_system, makeShared<WallBoundary>("WallBoundary"));
        wall_boundary.defineMatterMaterial<Solid>();
        wall_boundary.generateParticles<BaseParticles, Lattice>();

        ObserverBody fluid_observer(sph_system, "FluidObserver");
        fluid_observer.generateParticles<ObserverParticles>(createObservationPoints());
        InnerRelation water_block_inner(water_block);
        ContactRelation water_wall_contact(water_block, {&wall_boundary});
        ContactRelation fluid_observer_contact(fluid_observer, {&water_block});
        ComplexRelation water_block_complex(water_block_inner, water_wall_contact);

        Gravity gravity(Vec3d(0.0, -gravity_g, 0.0));
        SimpleDynamics<GravityForce<Gravity>> constant_gravity(water_block, gravity);
        SimpleDynamics<NormalDirectionFromBodyShape> wall_boundary_normal_direction(wall_boundary);
        Dynamics1Level<fluid_dynamics::Integration1stHalfWithWallRiemann> pressure_relaxation(water_block_inner,
                                                                                            water_wall_contact);
        Dynamics1Level<fluid_dynamics::Integration2ndHalfWithWallRiemann> density_relaxation(water_block_inner,
                                                                                           water_wall_contact);
        InteractionWithUpdate<fluid_dynamics::DensitySummationComplexFreeSurface> update_density_by_summation(
            water_block_inner, water_wall_contact);
        ReduceDynamics<fluid_dynamics::AdvectionTimeStep> get_fluid_advection_time_step_size(water_block, U_f);
        ReduceDynamics<fluid_dynamics::AcousticTimeStep> get_fluid_time_step_size(water_block);
        ParticleSorting particle_sorting(water_block);
        BodyStatesRecordingToVtp write_water_block_states(sph_system);
        write_water_block_states.addToWrite<Vec3d>(wall_boundary, "NormalDirection");
        RegressionTestDynamicTimeWarping<ReducedQuantityRecording<TotalMechanicalEnergy>> write_water_mechanical_energy(
            water_block, gravity);
        RegressionTestDynamicTimeWarping<ObservedQuantityRecording<Real>> write_recorded_water_pressure(
            "Pressure", fluid_observer_contact);

        sph_system.initializeSystemCellLinkedLists();
        sph_system.initializeSystemConfigurations();
        wall_boundary_normal_direction.exec();
        constant_gravity.exec();
        Real &physical_time = *sph_system.getSystemVariableDataByName<Real>("PhysicalTime");
        size_t number_of_iterations = sph_system.RestartStep();
        int screen_output_interval = 100;
        Real output_interval = end_time / 20.0;
        Real dt = 0.0;
        TickCount t1 = TickCount::now();
        TimeInterval interval;
        write_water_block_states.writeToFile(0);
        write_water_mechanical_energy.writeToFile(0);
        printf("energy %zu %.17g %.17g\n", number_of_iterations, physical_time,
               write_water_mechanical_energy.snapshots().back()[0]);
        bool cut_short = false;
        while (physical_time < end_time && !cut_short)
        {
            Real integration_time = 0.0;
            while (integration_time < output_interval && !cut_short)
            {
                Real Dt = get_fluid_advection_time_step_size.exec();
                update_density_by_summation.exec();
                Real relaxation_time = 0.0;
                while (relaxation_time < Dt)
                {
                    pressure_relaxation.exec(dt);
                    density_relaxation.exec(dt);
                    dt = get_fluid_time_step_size.exec();
                    relaxation_time += dt;
                    integration_time += dt;
                    physical_time += dt;
                }
                if (number_of_iterations % screen_output_interval == 0)
                    std::cout << std::fixed << std::setprecision(9) << "N=" << number_of_iterations
                              << "\tTime = " << physical_time << "\tDt = " << Dt << "\tdt = " << dt << "\n";
                number_of_iterations++;
                if (number_of_iterations % 100 == 0 && number_of_iterations != 1)
                    particle_sorting.exec();
                water_block.updateCellLinkedList();
                water_block_complex.updateConfiguration();
                fluid_observer_contact.updateConfiguration();
                write_recorded_water_pressure.writeToFile(number_of_iterations);
                cut_short = max_iterations >= 0 && long(number_of_iterations) >= max_iterations;
            }
            write_water_mechanical_energy.writeToFile(number_of_iterations);
            printf("energy %zu %.17g %.17g\n", number_of_iterations, physical_time,
                   write_water_mechanical_energy.snapshots().back()[0]);
            TickCount t2 = TickCount::now();
            write_water_block_states.writeToFile();
            interval += TickCount::now() - t2;
        }
        TimeInterval tt = TickCount::now() - t1 - interval;
        std::cout << "Total wall time for computation: " << tt.seconds() << " seconds." << std::endl;
        printf("final %zu %.17g %.17g\n", number_of_iterations, physical_time,
               write_water_mechanical_energy.snapshots().back()[0]);

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
