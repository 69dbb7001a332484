/**
 * 2D dam break with the particle-method containers of the CK drivers on the GB300
 * execution policy: same case, object names, container calls and single time-stepping loop
 * as the reference example tests/tests_sycl/2d_examples/test_2d_dambreak_sycl/
 * dambreak_sycl.cpp, compiled against sphinxsys_gb300/host/sphinxsys_cuda.h and
 * libsphx_cuda.so.  Output: VTP states every 0.1 (--state_recording), restart files every
 * 1000 advection steps, the .dat series of the two regression quantities, and on stdout the
 * observation lines "energy <step> <time> <E>" / "probe <step> <time> <p>"; at the end the
 * dynamic-time-warping test against ./input (exit status 1 on failure) unless the run was
 * cut short by max_iterations or restarted.
 *
 * usage: dambreak_sycl_2d [end_time] [max_iterations] [--restart_step=N] [--state_recording=0|1]
 */
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

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
        BoundingBoxd system_domain_bounds(Vec2d(-BW, -BW), Vec2d(DL + BW, DH + BW));
        SPHSystem sph_system(system_domain_bounds, particle_spacing_ref);
        sph_system.handleCommandlineOptions(ac, av);

        GeometricShapeBox initial_water_block(Transform(water_block_translation), water_block_halfsize, "WaterBody");
        FluidBody water_block(sph_system, initial_water_block);
        water_block.defineMatterMaterial<WeaklyCompressibleFluid>(rho0_f, c_f);
        water_block.generateParticles<BaseParticles, Lattice>();

        ComplexShape wall_complex_shape("WallBoundary");
        wall_complex_shape.add<GeometricShapeBox>(Transform(outer_wall_translation), outer_wall_halfsize);
        wall_complex_shape.subtract<GeometricShapeBox>(Transform(inner_wall_translation), inner_wall_halfsize);
        SolidBody wall_boundary(sph_system, wall_complex_shape);
        wall_boundary.defineMatterMaterial<Solid>();
        wall_boundary.generateParticles<BaseParticles, Lattice>();

        ObserverBody fluid_observer(sph_system, "FluidObserver");
        StdVec<Vecd> observation_location = {Vecd(DL, 0.2)};
        fluid_observer.generateParticles<ObserverParticles>(observation_location);

        Inner<> water_block_inner(water_block);
        Contact<> water_wall_contact(water_block, {&wall_boundary});
        Contact<> fluid_observer_contact(fluid_observer, {&water_block});

        SPHSolver sph_solver(sph_system);
        auto &main_methods = sph_solver.addParticleMethodContainer(par_ck);
        auto &host_methods = sph_solver.addParticleMethodContainer(par_host);

        auto &water_cell_linked_list = main_methods.addCellLinkedListDynamics(water_block);
        auto &wall_cell_linked_list = main_methods.addCellLinkedListDynamics(wall_boundary);
        auto &water_block_update_complex_relation = main_methods.addRelationDynamics(water_block_inner, water_wall_contact);
        auto &fluid_observer_contact_relation = main_methods.addRelationDynamics(fluid_observer_contact);
        auto &particle_sort = main_methods.addSortDynamics(water_block);

        Gravity gravity(Vecd(0.0, -gravity_g));
        auto &constant_gravity = main_methods.addStateDynamics<GravityForceCK<Gravity>>(water_block, gravity);
        auto &wall_boundary_normal_direction = host_methods.addStateDynamics<NormalFromBodyShapeCK>(wall_boundary);
        auto &water_advection_step_setup = main_methods.addStateDynamics<fluid_dynamics::AdvectionStepSetup>(water_block);
        auto &water_update_particle_position = main_methods.addStateDynamics<fluid_dynamics::UpdateParticlePosition>(water_block);

        auto &fluid_linear_correction_matrix =
            main_methods.addInteractionDynamics<LinearCorrectionMatrix, WithUpdate>(water_block_inner, 0.5)
                .addPostContactInteraction(water_wall_contact);
        auto &fluid_acoustic_step_1st_half =
            main_methods.addInteractionDynamics<fluid_dynamics::AcousticStep1stHalf, OneLevel,
                                                AcousticRiemannSolverCK, LinearCorrectionCK>(water_block_inner)
                .addPostContactInteraction<Wall, AcousticRiemannSolverCK, LinearCorrectionCK>(water_wall_contact);
        auto &fluid_acoustic_step_2nd_half =
            main_methods.addInteractionDynamics<fluid_dynamics::AcousticStep2ndHalf, OneLevel,
                                                AcousticRiemannSolverCK, LinearCorrectionCK>(water_block_inner)
                .addPostContactInteraction<Wall, AcousticRiemannSolverCK, LinearCorrectionCK>(water_wall_contact);
        auto &fluid_density_regularization =
            main_methods.addInteractionDynamics<fluid_dynamics::CompressionSummation>(water_block_inner)
                .addPostContactInteraction(water_wall_contact)
                .addPostStateDynamics<fluid_dynamics::DensityRegularization, WeaklyCompressibleFluid, FreeSurface>(water_block);

        auto &fluid_advection_time_step = main_methods.addReduceDynamics<fluid_dynamics::AdvectionTimeStepCK>(water_block, U_ref);
        auto &fluid_acoustic_time_step =
            main_methods.addReduceDynamics<fluid_dynamics::AcousticTimeStepCK<WeaklyCompressibleFluid>>(water_block);

        auto &body_state_recorder = main_methods.addBodyStateRecorder<BodyStatesRecordingToVtpCK>(sph_system);
        body_state_recorder.addToWrite<Vecd>(wall_boundary, "NormalDirection");
        body_state_recorder.addToWrite<Real>(water_block, "Density");
        auto &restart_io = main_methods.addIODynamics<RestartIOCK>(sph_system);
        auto &record_water_mechanical_energy =
            main_methods.addReduceRegression<RegressionTestDynamicTimeWarping, TotalMechanicalEnergyCK>(water_block, gravity);
        auto &fluid_observer_pressure =
            main_methods.addObserveRegression<RegressionTestDynamicTimeWarping, Real>(fluid_observer_contact, "Pressure");

        TimeStepper &time_stepper = sph_solver.getTimeStepper();
        if (sph_system.RestartStep() != 0)
        {
            restart_io.readRestartFiles(sph_system.RestartStep());
            printf("restart %d %.17g\n", sph_system.RestartStep(), time_stepper.getPhysicalTime());
        }

        auto &advection_step = time_stepper.addTriggerByInterval(fluid_advection_time_step.exec());
        size_t advection_steps = sph_system.RestartStep() + 1;
        int screening_interval = 100;
        int observation_interval = screening_interval * 2;
        int restart_output_interval = screening_interval * 10;
        auto &state_recording = time_stepper.addTriggerByInterval(0.1);

        wall_boundary_normal_direction.exec();
        constant_gravity.exec();
        water_cell_linked_list.exec();
        wall_cell_linked_list.exec();
        water_block_update_complex_relation.exec();
        fluid_observer_contact_relation.exec();
        fluid_density_regularization.exec();
        water_advection_step_setup.exec();
        fluid_linear_correction_matrix.exec();

        auto observe = [&]() {
            record_water_mechanical_energy.writeToFile(advection_steps);
            fluid_observer_pressure.writeToFile(advection_steps);
            printf("energy %zu %.17g %.17g\n", advection_steps, time_stepper.getPhysicalTime(),
                   record_water_mechanical_energy.snapshots().back()[0]);
            printf("probe %zu %.17g %.17g\n", advection_steps, time_stepper.getPhysicalTime(),
                   fluid_observer_pressure.snapshots().back()[0]);
        };
        body_state_recorder.writeToFile();
        observe();

        TimeInterval interval_output, interval_advection_step, interval_acoustic_step, interval_updating_configuration;
        TickCount t0 = TickCount::now();
        long iterations = 0;
        bool cut_short = false;
        while (!time_stepper.isEndTime(end_time))
        {
            TickCount time_instance = TickCount::now();
            Real acoustic_dt = time_stepper.incrementPhysicalTime(fluid_acoustic_time_step);
            fluid_acoustic_step_1st_half.exec(acoustic_dt);
            fluid_acoustic_step_2nd_half.exec(acoustic_dt);
            interval_acoustic_step += TickCount::now() - time_instance;

            if (advection_step(fluid_advection_time_step))
            {
                advection_steps++;
                water_update_particle_position.exec();

                time_instance = TickCount::now();
                if (advection_steps % screening_interval == 0)
                    std::cout << std::fixed << std::setprecision(9) << "N=" << advection_steps
                              << "\tTime = " << time_stepper.getPhysicalTime() << "\t"
                              << "\tadvection_dt = " << advection_step.getInterval()
                              << "\tacoustic_dt = " << time_stepper.getGlobalTimeStepSize() << "\n";
                if (advection_steps % observation_interval == 0)
                {
                    record_water_mechanical_energy.writeToFile(advection_steps);
                    fluid_observer_contact_relation.exec();
                    fluid_observer_pressure.writeToFile(advection_steps);
                    printf("energy %zu %.17g %.17g\n", advection_steps, time_stepper.getPhysicalTime(),
                           record_water_mechanical_energy.snapshots().back()[0]);
                    printf("probe %zu %.17g %.17g\n", advection_steps, time_stepper.getPhysicalTime(),
                           fluid_observer_pressure.snapshots().back()[0]);
                }
                if (advection_steps % restart_output_interval == 0)
                    restart_io.writeToFile(advection_steps);
                if (state_recording())
                    body_state_recorder.writeToFile();
                interval_output += TickCount::now() - time_instance;

                time_instance = TickCount::now();
                if (advection_steps % 100)
                    particle_sort.exec();
                water_cell_linked_list.exec();
                water_block_update_complex_relation.exec();
                interval_updating_configuration += TickCount::now() - time_instance;

                time_instance = TickCount::now();
                fluid_density_regularization.exec();
                water_advection_step_setup.exec();
                fluid_linear_correction_matrix.exec();
                interval_advection_step += TickCount::now() - time_instance;

                ++iterations;
                if (max_iterations >= 0 && iterations >= max_iterations)
                {
                    cut_short = true;
                    break;
                }
            }
        }
        TimeInterval tt = TickCount::now() - t0 - interval_output;
        std::cout << "Total wall time for computation: " << tt.seconds() << " seconds." << std::endl;
        std::cout << std::fixed << std::setprecision(9) << "interval_advection_step =" << interval_advection_step.seconds()
                  << "\n";
        std::cout << std::fixed << std::setprecision(9) << "interval_acoustic_step = " << interval_acoustic_step.seconds()
                  << "\n";
        std::cout << std::fixed << std::setprecision(9)
                  << "interval_updating_configuration = " << interval_updating_configuration.seconds() << "\n";
        printf("final %zu %.17g\n", advection_steps, time_stepper.getPhysicalTime());

        if (sph_system.GenerateRegressionData())
        {
            record_water_mechanical_energy.generateDataBase(1.0e-3);
            fluid_observer_pressure.generateDataBase(1.0e-3);
        }
        else if (sph_system.RestartStep() == 0 && !cut_short)
        {
            record_water_mechanical_energy.testResult();
            fluid_observer_pressure.testResult();
        }
    }
    catch (const SphxException &e)
    {
        fprintf(stderr, "%s\n", e.what());
        return 1;
    }
    return 0;
}
