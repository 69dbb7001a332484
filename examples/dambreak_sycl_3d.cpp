/**
 * 3D dam break with the computing-kernel (CK) dynamics on the GB300 execution policy.  Same
 * case, object names and main loop as the reference example
 * tests/tests_sycl/3d_examples/test_3d_dambreak_sycl/dambreak.cpp, with
 * MainExecutionPolicy = execution::CudaDevicePolicy, compiled against
 * sphinxsys_gb300/host/sphinxsys_cuda.h and libsphx_cuda.so.  File output (VTP, regression
 * databases) is replaced by printing the six wall probes after every advection step and the
 * mechanical energy at every output interval.
 *
 * usage: dambreak_sycl_3d [end_time] [max_iterations]
 */
#include <cstdio>
#include <cstdlib>

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

static void print_probes(const char *tag, size_t iteration, Real time, const std::vector<Real> &p)
{
    printf("%s %zu %.17g", tag, iteration, time);
    for (Real v : p)
        printf(" %.17g", v);
    printf("\n");
}

int main(int ac, char *av[])
{
    Real end_time = ac > 1 ? atof(av[1]) : 20.0;
    long max_iterations = ac > 2 ? atol(av[2]) : -1;
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

        Inner<> water_block_inner(water_block);
        Contact<> water_wall_contact(water_block, {&wall_boundary});
        Contact<> fluid_observer_contact(fluid_observer, {&water_block});

        UpdateCellLinkedList<MainExecutionPolicy, RealBody> water_cell_linked_list(water_block);
        UpdateCellLinkedList<MainExecutionPolicy, RealBody> wall_cell_linked_list(wall_boundary);
        UpdateRelation<MainExecutionPolicy, Inner<>, Contact<>> water_block_update_complex_relation(water_block_inner, water_wall_contact);
        UpdateRelation<MainExecutionPolicy, Contact<>> fluid_observer_contact_relation(fluid_observer_contact);
        ParticleSortCK<MainExecutionPolicy> particle_sort(water_block);

        Gravity gravity(Vec3d(0.0, -gravity_g, 0.0));
        StateDynamics<MainExecutionPolicy, GravityForceCK<Gravity>> constant_gravity(water_block, gravity);
        StateDynamics<execution::CudaDevicePolicy, NormalFromBodyShapeCK> wall_boundary_normal_direction(wall_boundary);
        StateDynamics<MainExecutionPolicy, fluid_dynamics::AdvectionStepSetup> water_advection_step_setup(water_block);
        StateDynamics<MainExecutionPolicy, fluid_dynamics::UpdateParticlePosition> water_update_particle_position(water_block);

        InteractionDynamicsCK<MainExecutionPolicy, LinearCorrectionMatrixComplex>
            fluid_linear_correction_matrix(DynamicsArgs(water_block_inner, 0.5), water_wall_contact);
        InteractionDynamicsCK<MainExecutionPolicy, fluid_dynamics::AcousticStep1stHalfWithWallRiemannCorrectionCK>
            fluid_acoustic_step_1st_half(water_block_inner, water_wall_contact);
        InteractionDynamicsCK<MainExecutionPolicy, fluid_dynamics::AcousticStep2ndHalfWithWallRiemannCorrectionCK>
            fluid_acoustic_step_2nd_half(water_block_inner, water_wall_contact);
        InteractionDynamicsCK<MainExecutionPolicy, fluid_dynamics::CompressionSummation<Inner<>, Contact<>>>
            fluid_density_summation(water_block_inner, water_wall_contact);
        StateDynamics<MainExecutionPolicy, fluid_dynamics::DensityRegularization<SPHBody, WeaklyCompressibleFluid, FreeSurface>>
            fluid_density_regularization(water_block);
        InteractionDynamicsCK<MainExecutionPolicy, fluid_dynamics::FreeSurfaceIndicationComplexSpatialTemporalCK>
            fluid_boundary_indicator(water_block_inner, water_wall_contact);
        ReduceDynamicsCK<MainExecutionPolicy, fluid_dynamics::AdvectionTimeStepCK> fluid_advection_time_step(water_block, U_f);
        ReduceDynamicsCK<MainExecutionPolicy, fluid_dynamics::AcousticTimeStepCK<WeaklyCompressibleFluid>> fluid_acoustic_time_step(water_block);

        TotalMechanicalEnergy record_water_mechanical_energy(water_block, gravity);
        ObservedQuantityCK fluid_observer_pressure("Pressure", fluid_observer_contact);

        SPHSystem::SingleVariable<Real> *sv_physical_time = sph_system.getSystemVariableByName<Real>("PhysicalTime");
        wall_boundary_normal_direction.exec();
        constant_gravity.exec();
        water_cell_linked_list.exec();
        wall_cell_linked_list.exec();
        water_block_update_complex_relation.exec();
        fluid_observer_contact_relation.exec();

        size_t number_of_iterations = 0;
        Real output_interval = end_time / 20.0;
        printf("energy %zu %.17g %.17g\n", number_of_iterations, sv_physical_time->getValue(),
               record_water_mechanical_energy.exec());
        print_probes("probe", number_of_iterations, sv_physical_time->getValue(), fluid_observer_pressure.exec());
        bool done = false;
        while (sv_physical_time->getValue() < end_time && !done)
        {
            Real integration_time = 0.0;
            while (integration_time < output_interval && !done)
            {
                fluid_density_summation.exec();
                fluid_density_regularization.exec();
                water_advection_step_setup.exec();
                Real advection_dt = fluid_advection_time_step.exec();
                fluid_boundary_indicator.exec();
                fluid_linear_correction_matrix.exec();

                Real relaxation_time = 0.0;
                Real acoustic_dt = 0.0;
                while (relaxation_time < advection_dt)
                {
                    acoustic_dt = fluid_acoustic_time_step.exec();
                    fluid_acoustic_step_1st_half.exec(acoustic_dt);
                    fluid_acoustic_step_2nd_half.exec(acoustic_dt);
                    relaxation_time += acoustic_dt;
                    integration_time += acoustic_dt;
                    sv_physical_time->incrementValue(acoustic_dt);
                }
                water_update_particle_position.exec();
                number_of_iterations++;

                if (number_of_iterations % 100 == 0 && number_of_iterations != 1)
                    particle_sort.exec();
                water_cell_linked_list.exec();
                water_block_update_complex_relation.exec();
                fluid_observer_contact_relation.exec();
                print_probes("probe", number_of_iterations, sv_physical_time->getValue(),
                             fluid_observer_pressure.exec());
                done = max_iterations >= 0 && long(number_of_iterations) >= max_iterations;
            }
            printf("energy %zu %.17g %.17g\n", number_of_iterations, sv_physical_time->getValue(),
                   record_water_mechanical_energy.exec());
        }
    }
    catch (const SphxException &e)
    {
        fprintf(stderr, "%s\n", e.what());
        return 1;
    }
    return 0;
}
