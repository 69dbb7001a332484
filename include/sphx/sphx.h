/*
 * sphx.h -- C ABI of the GB300 (sm_103a) execution policy for SPHinXsys'
 * weakly-compressible fluid step.
 *
 * Every entry point returns an int status (SPHX_OK or an SPHX_ERR_* code), never
 * calls exit(), and records a message readable with sphx_last_error().  Work is
 * enqueued on the stream of the context; entry points that return a value to the
 * host (time steps, reductions, capacities) synchronise that stream, like the
 * reference's ReduceDynamics::exec.  A context is used from one host thread at a
 * time, as the reference drives its single in-order device queue
 * (src/src_sycl/shared/particle_dynamics/implementation_sycl.h:43-94).
 *
 * Data layout: every particle variable lives on the device as structure-of-arrays
 * (component c of particle i at base[c * n + i]); sphx_body_upload/download do the
 * AoS <-> SoA transpose of the reference's Eigen Vecd arrays at the boundary.
 * Reference paths below are relative to the SPHinXsys source tree.
 */
#ifndef SPHX_H
#define SPHX_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------------ status codes */
#define SPHX_OK 0
#define SPHX_ERR_INVALID_ARG 1  /* bad handle, size, name or parameter */
#define SPHX_ERR_CUDA 2         /* a CUDA runtime call failed */
#define SPHX_ERR_CAPACITY 3     /* neighbour or cell storage too small (after retry) */
#define SPHX_ERR_OUT_OF_MEMORY 4
#define SPHX_ERR_NOT_FOUND 5    /* unknown variable name */
#define SPHX_ERR_TIMEOUT 6      /* a bounded device wait gave up */
#define SPHX_ERR_NUMERIC 7      /* non-finite value detected by a checked entry point */
#define SPHX_ERR_NO_DEVICE 8
#define SPHX_ERR_BOUNDS 9       /* an index test of the bounds-checked build failed */

typedef struct sphx_ctx_s *sphx_ctx;
typedef struct sphx_body_s *sphx_body;
typedef struct sphx_cell_list_s *sphx_cell_list;
typedef struct sphx_relation_s *sphx_relation;

typedef enum { SPHX_F64 = 0, SPHX_U32 = 1, SPHX_F32 = 2, SPHX_I32 = 3 } sphx_dtype;

/* Message of the last failing call on this host thread (static storage). */
const char *sphx_last_error(void);
/* Library version string. */
const char *sphx_version(void);
/* 1 when the library was built with -DSPHX_CHECK (bounds-checked build), else 0. */
int sphx_checked_build(void);
/* Bounds-checked build: the kernels test the neighbour-list entries, cell-list ranges and
 * cell indices they read through, count each failed test, skip its access and keep the
 * first one (site in the high 16 bits: 1 list entry, 2 cell range, 3 cell index; the
 * offending value in the low 48).  Synchronises the device, outputs (may be null) the
 * count and the first record since the last reset, clears them when reset != 0, and
 * returns SPHX_ERR_BOUNDS when the count is non-zero.  In other builds the count is 0.
 * The reference indexes its containers unchecked (no counterpart). */
int sphx_check_violations(uint64_t *count, uint64_t *first, int reset);

/* ------------------------------------------------------------------ context
 * Replaces the SYCL device queue singleton and USM helpers
 * (src/src_sycl/shared/particle_dynamics/implementation_sycl.h:43-139).  `stream`
 * may be 0 to let the context create its own non-blocking stream; otherwise it is a
 * cudaStream_t owned by the caller. */
int sphx_ctx_create(int device, void *stream, sphx_ctx *out);
int sphx_ctx_destroy(sphx_ctx ctx);
int sphx_ctx_synchronize(sphx_ctx ctx);
/* Number of kernels this context has launched so far. */
int sphx_ctx_launch_count(sphx_ctx ctx, uint64_t *count);
/* The cudaStream_t the context enqueues on. */
int sphx_ctx_stream(sphx_ctx ctx, void **stream);

/* ------------------------------------------------------------------ particles
 * A body's particle variables, the device mirror of BaseParticles' DiscreteVariable
 * registry (src/shared/common/sphinxsys_variable.h:119-378; DelegatedData at :282-289,
 * prepareForOutput/finalizeLoadIn at :350-356).  `dim` is 2 or 3.  Variables used by
 * the fluid step: Position, Velocity, Force, ForcePrior (dim components); Density,
 * Pressure, DensityChangeRate, Mass, VolumetricMeasure, DensitySummation (scalars);
 * OriginalID, SortedID (u32).  Wall bodies add NormalDirection, Velocity and
 * Acceleration (the Solid averages, src/shared/materials/base_material.cpp:57-72). */
int sphx_body_create(sphx_ctx ctx, int dim, size_t n, sphx_body *out);
int sphx_body_destroy(sphx_body body);
int sphx_body_size(sphx_body body, size_t *n);
/* registerStateVariable: creates (zero-filled) a variable if absent. */
int sphx_body_register(sphx_body body, const char *name, sphx_dtype dtype, int ncomp);
/* Host AoS (n x ncomp) -> device SoA; registers the variable if needed. */
int sphx_body_upload(sphx_body body, const char *name, sphx_dtype dtype, int ncomp, const void *host, size_t n);
/* Device SoA -> host AoS (n x ncomp); synchronises the stream. */
int sphx_body_download(sphx_body body, const char *name, void *host, size_t n);
/* Rows [first, first + count) of a registered variable from / to a host AoS buffer of
 * count x ncomp values (the ghost-layer exchange of a slab decomposition refreshes a block
 * of rows; the reference's host-side counterpart is a loop over the variable's data).
 * Synchronous; a pinned host buffer is copied at full link speed. */
int sphx_body_upload_rows(sphx_body body, const char *name, const void *host, size_t first, size_t count);
int sphx_body_download_rows(sphx_body body, const char *name, void *host, size_t first, size_t count);
/* DelegatedData(CudaDevicePolicy): device base pointer of a variable (SoA). */
int sphx_body_device_ptr(sphx_body body, const char *name, void **dev, sphx_dtype *dtype, int *ncomp);
/* Checked entry point: counts the particles of a floating-point variable with a
 * non-finite component (NaN or infinity) into *non_finite (may be null) and returns
 * SPHX_ERR_NUMERIC when there are any (synchronises).  The reference has no such check;
 * its failures end the process (`exit(1)`, sphinxsys_variable.h:269-274,
 * cell_linked_list.cpp:242-246), where this returns a status. */
int sphx_body_check_finite(sphx_body body, const char *name, uint64_t *non_finite);

/* ------------------------------------------------------------------ mesh + cell list */
typedef struct
{
    int dim;
    int all_cells[3];   /* cells per axis (all_grid_points - 1) */
    double lower[3];    /* mesh_lower_bound_ */
    double grid_spacing;
} sphx_mesh_desc;

/* Mesh::Mesh(tentative_bounds, grid_spacing, buffer_width)
 * (src/shared/meshes/base_mesh.cpp:6-16). */
int sphx_mesh_from_bounds(int dim, const double *lower, const double *upper, double grid_spacing, int buffer_width,
                          sphx_mesh_desc *out);

/* CellLinkedList<SPHAdaptation> storage: CellOffset[ncells+1] and ParticleIndex
 * (src/shared/meshes/cell_linked_list.cpp:160-175). */
int sphx_cell_list_create(sphx_ctx ctx, const sphx_mesh_desc *mesh, size_t particle_capacity, sphx_cell_list *out);
int sphx_cell_list_destroy(sphx_cell_list cl);
/* UpdateCellLinkedList::exec / BaseCellLinkedList::UpdateCellLists
 * (update_cell_linked_list.hpp:40-106, cell_linked_list.cpp:84-101): hash by
 * CellIndexFromPosition (base_mesh.hxx:9-15), count, exclusive scan, scatter.  Inside a
 * cell the particles ascend by index, a canonical form of the reference's
 * unordered atomic / concurrent_vector fill. */
int sphx_cell_list_update(sphx_cell_list cl, sphx_body body);
int sphx_cell_list_num_cells(sphx_cell_list cl, size_t *ncells);
/* Copies CellOffset (ncells+1) and ParticleIndex (n) to the host. */
int sphx_cell_list_download(sphx_cell_list cl, uint32_t *cell_offset, uint32_t *particle_index, size_t n);

/* PeriodicConditionUsingCellLinkedList (domain_bounding.cpp:16-60): once an axis is set, every
 * update also inserts periodic images: along each periodic axis in turn, each entry (a
 * particle or an image of an earlier axis) with lower < x < lower + cutoff gets an image at
 * x + (upper - lower), each with upper - cutoff < x < upper one at x - (upper - lower).
 * Relations built on the list see the images at their translated positions and record the
 * real particle's index.  Requires 2 cutoff < upper - lower. */
int sphx_cell_list_set_periodic(sphx_cell_list cl, int axis, double lower, double upper, double cutoff);
/* Entries (particles + periodic images) of the last update. */
int sphx_cell_list_num_entries(sphx_cell_list cl, size_t *n_entries);
/* PeriodicBounding (domain_bounding.h:103-113): x < lower -> x + L, x > upper -> x - L. */
int sphx_periodic_bounding(sphx_body body, int axis, double lower, double upper);

/* exclusive_scan(ParallelDevicePolicy, ...) (src/src_sycl/shared/common/
 * algorithm_primitive_sycl.h:96-122): device u32 exclusive prefix sum of n entries,
 * returns the total through *total (synchronises). */
int sphx_exclusive_scan_u32(sphx_ctx ctx, const uint32_t *d_in, uint32_t *d_out, size_t n, uint32_t *total);
/* The same scan for callers that cannot allocate device memory while they run (their
 * device memory belongs to another allocator, or their loop must not pay the device-wide
 * synchronisation of cudaMalloc / cudaFree).  It has no counterpart in the reference.
 * Needs no context: enqueues on `stream` (0 = the legacy default stream) of the current
 * device, and calls no cudaMalloc, cudaFree or other allocating routine; its scratch is a
 * fixed 128 KiB device array of the library that every GPU loading the library holds until
 * the process exits.  At most SPHX_SCAN_NOALLOC_MAX_N entries (larger n returns
 * SPHX_ERR_INVALID_ARG).  The first call on a device looks up the array's address and
 * should come before any stream capture.  The looked-up address is kept for the life of
 * the process, so calls after a cudaDeviceReset of that device are not supported.  Calls
 * share the array: calls that overlap on the GPU race, so serialise them on one stream.
 * With `total` non-null the call synchronises `stream` to return the sum of all n inputs. */
#define SPHX_SCAN_NOALLOC_MAX_N 67108864u
int sphx_exclusive_scan_u32_noalloc(void *stream, const uint32_t *d_in, uint32_t *d_out, size_t n, uint32_t *total);

/* ------------------------------------------------------------------ relations
 * InnerRelation (src/shared/body_relations/inner_body_relation.cpp:10-20) and
 * ContactRelation (contact_body_relation.cpp:11-32).  The Wendland C2 kernel of
 * smoothing length h (kernel_wendland_c2.cpp:8-45) is evaluated once per
 * configuration update, as NeighborBuilderInner/Contact do (neighborhood.cpp:26-160).
 * Contact `search_depth` is SearchDepthContact (base_body_relation.cpp:10-16). */
int sphx_inner_relation_create(sphx_body body, sphx_cell_list cl, double h, sphx_relation *out);
int sphx_contact_relation_create(sphx_body body, sphx_body target, sphx_cell_list target_cl, double h,
                                 int search_depth, double target_rho0, sphx_relation *out);
int sphx_relation_destroy(sphx_relation rel);
/* updateConfiguration(): neighbour search on the current positions.  Grows its
 * storage and searches again when a list overflows (synchronises once). */
int sphx_relation_update(sphx_relation rel);
/* Neighbour lists as CSR on the host: counts[n_src] and, when non-null, j/W/dW/r of
 * total = sum(counts) entries and e (total x dim); lists follow cell scan order. */
int sphx_relation_download(sphx_relation rel, uint32_t *counts, uint32_t *j, double *W, double *dW, double *r,
                           double *e, size_t *total);

/* ------------------------------------------------------------------ fluid dynamics */
typedef struct
{
    double rho0, c0;        /* WeaklyCompressibleFluid (weakly_compressible_fluid.cpp:8-30) */
    double h;               /* smoothing length (adaptation.h:71, h = 1.3 dp) */
    double sigma0;          /* SPHAdaptation::LatticeNumberDensity (adaptation.cpp:25-58) */
    double limiter_slope;   /* TruncatedLinear slope of AcousticRiemannSolver (riemann_solver.h:87), 3 */
    double acoustic_cfl;    /* AcousticTimeStep default 0.6 (fluid_time_step.h) */
    double advection_cfl;   /* AdvectionTimeStep default 0.25 */
    double U_ref;           /* AdvectionTimeStep reference speed */
} sphx_fluid_params;

/* SPHAdaptation::computeLatticeNumberDensity for Wendland C2 (adaptation.cpp:25-58). */
int sphx_lattice_number_density(int dim, double h, double dp, double *sigma0);

/* InteractionWithUpdate<DensitySummationComplexFreeSurface>::exec
 * (density_summation.cpp:74-82,124-144; density_summation.hpp:28-32). */
int sphx_density_summation_complex_free_surface(sphx_relation inner, sphx_relation wall_contact,
                                                const sphx_fluid_params *p);
/* Dynamics1Level<Integration1stHalfWithWallRiemann>::exec(dt)
 * (dynamics_algorithms.h:336-352; fluid_integration.hpp:49-113). */
int sphx_integration_1st_half_with_wall_riemann(sphx_relation inner, sphx_relation wall_contact,
                                                const sphx_fluid_params *p, double dt);
/* Dynamics1Level<Integration2ndHalfWithWallRiemann>::exec(dt) (fluid_integration.hpp:166-231). */
int sphx_integration_2nd_half_with_wall_riemann(sphx_relation inner, sphx_relation wall_contact,
                                                const sphx_fluid_params *p, double dt);
/* ReduceDynamics<AcousticTimeStep>::exec (fluid_time_step.cpp:21-31). */
int sphx_acoustic_time_step(sphx_body fluid, const sphx_fluid_params *p, double *dt);
/* ReduceDynamics<AdvectionTimeStep>::exec (fluid_time_step.cpp:54-65). */
int sphx_advection_time_step(sphx_body fluid, const sphx_fluid_params *p, double *dt);
/* SimpleDynamics<GravityForce<Gravity>>::exec (force_prior.hpp:20-41). */
int sphx_gravity_force(sphx_body fluid, const double *gravity);
/* ParticleSorting::exec (particle_sorting.cpp:25-58): Morton order of the cell of
 * `mesh` (base_mesh.hxx:80-99), stable in the current index; permutes every variable
 * of the body and refreshes SortedID. */
int sphx_particle_sorting(sphx_body body, const sphx_mesh_desc *mesh);

/* ------------------------------------------------------------------ observation */
/* ObservingAQuantity<Real> over a contact relation from observer points
 * (general_interpolation.h:58-78): out[i] = sum W V q / (sum W V + TinyReal). */
int sphx_observe_quantity(sphx_relation observer_contact, const char *name, double *out);
/* ReduceDynamics<TotalMechanicalEnergy> (general_reduce.cpp:75-79). */
int sphx_total_mechanical_energy(sphx_body fluid, const double *gravity, double *energy);
/* UpperFrontInAxisDirection over an axis-aligned box region (general_reduce.h:82-99). */
int sphx_upper_front_in_axis_direction(sphx_body fluid, int axis, const double *region_lower,
                                       const double *region_upper, double *front);

/* Keeps r_ij in the relation's storage from its next update on (the viscous force needs the
 * configuration-time distances; dam-break inner relations do without). */
int sphx_relation_keep_distances(sphx_relation rel);
/* InteractionWithUpdate<DensitySummationInner> (density_summation.hpp, Inner<> update:
 * rho = rho_sum, no free-surface bound). */
int sphx_density_summation_inner(sphx_relation inner, const sphx_fluid_params *p);
/* InteractionWithUpdate<ViscousForceInner> (viscous_dynamics.hpp:25-53 with the ForcePrior
 * update of force_prior.hpp:22-26): ViscousForce from the configuration-time r, e, dW
 * (needs sphx_relation_keep_distances), ForcePrior += ViscousForce - PreviousViscousForce. */
int sphx_viscous_force_inner(sphx_relation inner, double mu);
/* InteractionWithUpdate<TransportVelocityCorrectionInner<TruncatedLinear, AllParticles>>
 * (transport_velocity_correction.hpp:32-66): Position += coefficient h^2 min(100 h^2 |g|^2, 1) g,
 * g = -sum 2 dW_ij V_j e_ij; the reference's coefficient default is 0.2. */
int sphx_transport_velocity_correction_inner(sphx_relation inner, double coefficient);
/* ReduceDynamics<MaximumSpeed> (general_reduce.h): max |v| (synchronises).  The total
 * kinetic energy is sphx_total_mechanical_energy with zero gravity. */
int sphx_maximum_speed(sphx_body body, double *out);

/* ------------------------------------------------------------------ CK numerics
 * The particle methods of the tests_sycl dam-break drivers
 * (tests/tests_sycl/2d_examples/test_2d_dambreak_sycl/dambreak_sycl.cpp:97-123), FP64,
 * on the relations above: pair geometry from the current Position with the tabulated
 * Wendland C2 (KernelTabulatedCK, kernel_tabulated_ck.h:37-62); the state variables
 * Compression, CompressionRate, Displacement, LinearCorrectionMatrix (dim x dim,
 * row-major components), VolumetricMeasureRef and CompressionSummation are registered on
 * first use with their reference initial values (1, 0, 0, identity, a copy of
 * VolumetricMeasure, 1). */
/* CompressionSummation<Inner, Contact> + DensityRegularization<FreeSurface>
 * (density_regularization.hpp:40-118). */
int sphx_ck_density_regularization(sphx_relation inner, sphx_relation wall_contact, const sphx_fluid_params *p);
/* The two parts of the above as separate dynamics (the 3D SYCL driver constructs them
 * separately): InteractionDynamicsCK<CompressionSummation<Inner<>, Contact<>>> writes
 * CompressionSummation; StateDynamics<DensityRegularization<SPHBody, WeaklyCompressibleFluid,
 * FreeSurface>> sets Compression = max(CompressionSummation, 1) and Density. */
int sphx_ck_compression_summation(sphx_relation inner, sphx_relation wall_contact);
int sphx_ck_free_surface_regularization(sphx_body fluid, double rho0);
/* AdvectionStepSetup (fluid_time_step_ck.h:145-149): Vol = m / rho, Displacement = 0. */
int sphx_ck_advection_step_setup(sphx_body fluid);
/* UpdateParticlePosition (fluid_time_step_ck.h:173-176): Position += Displacement. */
int sphx_ck_update_particle_position(sphx_body fluid);
/* LinearCorrectionMatrix<Inner<WithUpdate>> + <Contact> (kernel_correction_ck.hpp:25-80). */
int sphx_ck_linear_correction_matrix(sphx_relation inner, sphx_relation wall_contact, double alpha);
/* FreeSurfaceIndicationCK<Inner<WithUpdate>, Contact<>> (surface_indication_ck.hpp:49-150,
 * the boundary indicator of the 3D SYCL dam break): PositionDivergence = -sum dW V r with
 * the spatial-temporal rule, Indicator (I32, 1 at the free surface) and
 * PreviousSurfaceIndicator (I32, registered with 1), threshold 0.75 dim. */
int sphx_ck_free_surface_indication(sphx_relation inner, sphx_relation wall_contact);
/* AcousticStep1stHalf / 2ndHalf <Inner<OneLevel, AcousticRiemannSolverCK, LinearCorrectionCK>>
 * + <Contact<Wall, ...>> (acoustic_step_1st_half.hpp, acoustic_step_2nd_half.hpp). */
int sphx_ck_acoustic_step_1st_half(sphx_relation inner, sphx_relation wall_contact, const sphx_fluid_params *p,
                                   double dt);
int sphx_ck_acoustic_step_2nd_half(sphx_relation inner, sphx_relation wall_contact, const sphx_fluid_params *p,
                                   double dt);
/* AcousticTimeStepCK / AdvectionTimeStepCK (fluid_time_step_ck.hpp:25-57,
 * fluid_time_step_ck.cpp:16-20); synchronise. */
int sphx_ck_acoustic_time_step(sphx_body fluid, const sphx_fluid_params *p, double *dt);
int sphx_ck_advection_time_step(sphx_body fluid, const sphx_fluid_params *p, double *dt);
/* Interpolation<Contact<Real>> of a fluid variable at the observer points with the
 * tabulated kernel and the current volumes (interpolation_dynamics.hpp:46-60); out has
 * one value per observer (synchronises). */
int sphx_ck_observe_quantity(sphx_relation observer_contact, const char *name, double *out);

/* ------------------------------------------------------------------ mixed precision
 * A fused solver for one fluid body against one static wall body (the dam-break
 * configuration of Dambreak.cpp) in mixed precision; it has no single reference
 * counterpart: it runs the same sequence as one pass of the Dambreak.cpp:166-220 loop
 * (AdvectionTimeStep, DensitySummationComplexFreeSurface, the acoustic sub-steps of
 * Integration1stHalf/2ndHalfWithWallRiemann, and the cell-list / configuration update).
 *
 * Precision: pair kernels, gradients, pressure and dissipation in FP32 with
 * Kahan-compensated neighbour sums; positions as an FP32 offset from the lower corner of
 * an integer cell; density held as the FP32 deviation rho - rho0; position integration,
 * the time-step reductions and the conservation sums in FP64.  Particles are kept in
 * cell order, re-sorted at every configuration update.
 *
 * Requirements checked at creation: uniform particle mass and volume in each body, a
 * static wall (zero wall velocity and acceleration), gravity as the only prior force,
 * at most 16384 cells per mesh axis in 2D and 512 in 3D (the solver searches sub-cells of
 * half the spacing, packed 15 / 10 bits per axis). */
typedef struct sphx_mp_s *sphx_mp;

/* Builds the solver from the current FP64 state of the relations' bodies. */
int sphx_mp_create(sphx_relation inner, sphx_relation wall_contact, const sphx_fluid_params *p,
                   const double *gravity, sphx_mp *out);
/* Periodic viscous flow without walls, periodic along every axis of the cube
 * [lower, upper]: the taylor_green.cpp loop (taylor_green.cpp:133-164) with
 * DensitySummationInner, ViscousForceInner with the fixed viscosity `viscosity`
 * (viscous_dynamics.hpp:25-53; ForcePrior = the viscous force),
 * TransportVelocityCorrectionInner with `tvc_coefficient` (transport_velocity_correction.hpp:32-66),
 * Integration1stHalfInnerRiemann, Integration2ndHalf with p->limiter_slope (0 gives
 * Integration2ndHalfInnerNoRiemann), AdvectionViscousTimeStep (reference speed
 * max(p->U_ref, viscosity / rho0 / h)) and dt = min(acoustic dt, Dt) in the sub-steps
 * (loop_style 0 of sphx_mp_advection_step).  Sub-cells tile the cube exactly:
 * N = floor(L / h) per axis, 5 <= N <= 32768 (2D) / 1024 (3D); at most 2^26 particles.
 * sphx_mp_download also writes ForcePrior. */
int sphx_mp_create_periodic(sphx_body fluid, const sphx_fluid_params *p, const double *lower, const double *upper,
                            double viscosity, double tvc_coefficient, sphx_mp *out);
int sphx_mp_destroy(sphx_mp mp);
/* One advection step.  loop_style 0: acoustic dt taken before each relaxation
 * (Dambreak.cpp:181-190); 1: after it (test_3d_dambreak/dambreak.cpp:193-201).
 * Outputs (any may be null): acoustic sub-steps taken, the advection dt used, and the
 * physical time after the step.  The configuration update for the moved positions
 * (re-hash, re-sort, neighbour lists, density sums) runs at the start of the next step,
 * or not at all when sphx_mp_upload replaces the state first. */
int sphx_mp_advection_step(sphx_mp mp, int loop_style, int *substeps, double *advection_dt,
                           double *physical_time);
/* Reloads the solver from the FP64 fluid body (Position, Velocity, Force, Density,
 * DensityChangeRate; any particle order): re-sorts, rebuilds the configuration and the
 * time-step maxima.  Physical time and the last acoustic dt are kept (synchronises). */
int sphx_mp_upload(sphx_mp mp, sphx_body fluid);
/* Writes Position, Velocity, Density, Pressure, Force and DensityChangeRate back into the
 * FP64 fluid body, in the body's particle order (synchronises). */
int sphx_mp_download(sphx_mp mp, sphx_body fluid);
/* The same load as sphx_body_upload of each row followed by sphx_mp_upload, straight from
 * host rows in the body's particle order (position and velocity and force n x dim,
 * density and density change rate n; FP64; page-locked memory lets the copies run
 * asynchronously): the positions are copied first, and the copies of the other rows
 * overlap the re-sort and the neighbour search.  The FP64 body is not written.  Dam-break
 * solvers only (a periodic solver: SPHX_ERR_INVALID_ARG).  No counterpart in the
 * reference: the host state of a caller that keeps it in its own arrays (synchronises). */
int sphx_mp_upload_host(sphx_mp mp, const double *position, const double *velocity, const double *force,
                        const double *density, const double *density_change_rate);
/* Position and velocity (n x dim), density and pressure (n) rows in the body's particle
 * order, the values sphx_mp_download writes into the body (synchronises). */
int sphx_mp_download_host(sphx_mp mp, double *position, double *velocity, double *density, double *pressure);
/* Host rows (body order, the layout of sphx_mp_download_host) that every later
 * sphx_mp_advection_step fills with the state it ends on: the velocity and pressure rows
 * are copied while the last sub-step's 2nd half still runs (it changes neither), the
 * position and density rows after it; the step returns once they are in host memory.  The
 * same values as sphx_mp_download_host after the step.  Four nulls unregister.  Pinned
 * rows (cudaHostAlloc) copy at the link's rate.  No counterpart in the reference, whose
 * state lives in host memory: the device-to-host half of a caller that keeps its state in
 * its own arrays (with sphx_mp_upload_host). */
int sphx_mp_set_host_rows(sphx_mp mp, double *position, double *velocity, double *density, double *pressure);
/* FP64 conservation sums: out[0] total mass, out[1..3] momentum, out[4] mechanical energy
 * (kinetic + potential with gravity and zero reference at the origin). */
int sphx_mp_conservation(sphx_mp mp, double *out);
/* UpperFrontInAxisDirection of the fluid inside an axis-aligned box region. */
int sphx_mp_upper_front(sphx_mp mp, int axis, const double *region_lower, const double *region_upper,
                        double *front);
/* Checked entry point on the solver state: particles with a non-finite value in any
 * evolving field (position offset, velocity, pressure, density, density rate, force) and
 * finite particles whose position lies outside the cell mesh (a particle that left the
 * tank); outputs may be null.  Returns SPHX_ERR_NUMERIC when either count is non-zero
 * (synchronises; reads the state only).  No counterpart in the reference, which clamps
 * such particles into the boundary cells (base_mesh.hxx:9-15) or ends the process. */
int sphx_mp_check_state(sphx_mp mp, uint64_t *non_finite, uint64_t *out_of_mesh);
/* Kernel launch shape and neighbour strategy: block size (64..256, multiple of 32) of
 * the sweep kernels, and 0 = stored neighbour index lists, 1 = cell sweep every
 * sub-step, 2 = tiled (dam-break solver): one block per tile of sub-cells with the tile's
 * neighbour window staged in shared memory and lists of indices into it (tile shape from
 * sphx_mp_set_tile, 4 x 4 (x 4) by default, at most 8 per axis), 3 = the stored lists with
 * the neighbour records gathered by cp.async into a per-thread ring in shared memory,
 * 4 = the stored lists on persistent warps that take chunks of 32 particles, 5 and 6 =
 * the stored lists with 2 and 4 lanes per particle (16 and 8 particles per warp; each
 * lane takes every 2nd / 4th list slot, sums combined by warp shuffles) (3 to 6 dam-break
 * solver only).  Strategies 0 to 4 give the same results bit for bit; 5 and 6 sum each
 * particle's neighbours in another order and agree with them to FP32 rounding. */
int sphx_mp_set_tuning(sphx_mp mp, int block, int strategy);
/* Tile-grouped traversal of the sweeps and the neighbour build (dam-break solver): the
 * particles of each box of tx x ty (x tz) sub-cells go to consecutive threads, so a thread
 * block's neighbour records form a compact window; 0, 0, 0 turns it off.  Results do not
 * change (same particle order, lists and arithmetic).  Replaces the index-range launch of
 * particle_for (particle_iterators_sycl.h:229-241), whose work-groups follow the storage
 * order. */
int sphx_mp_set_tile(sphx_mp mp, int tx, int ty, int tz);
/* Current launch block, neighbour strategy and tile shape (tile: 3 ints; any may be null). */
int sphx_mp_get_tuning(sphx_mp mp, int *block, int *strategy, int *tile);
/* Times one acoustic sub-step for every block size (64, 128, 256) with each neighbour
 * strategy (the tiled one with several tile shapes, the lane-split ones with 2 and 4
 * lanes per particle), restores the state it advanced,
 * and keeps the fastest setting; outputs (any may be null) the chosen block, strategy and
 * ms per sub-step (sphx_mp_get_tuning gives the tile shape). */
int sphx_mp_autotune(sphx_mp mp, int reps, int *best_block, int *best_strategy, double *best_ms);
/* CUDA-event timing of the two sweep kernels of every sub-step (on the context's
 * stream); switching it resets the totals. */
int sphx_mp_set_profiling(sphx_mp mp, int on);
/* out[0] total ms of the 1st-half sweeps, out[1] their count, out[2] / out[3] the same
 * for the 2nd-half sweeps (synchronises). */
int sphx_mp_kernel_times(sphx_mp mp, double *out);
/* out[0] fluid particles, out[1] wall particles, out[2] stored inner pairs, out[3] stored
 * wall pairs, out[4] / out[5] list capacities (synchronises). */
int sphx_mp_list_sizes(sphx_mp mp, uint64_t *out);

/* ------------------------------------------------------------------ batched instances
 * Many independent dam breaks of one dimension advanced together in mixed precision (the
 * numerics of sphx_mp_*).  No single reference counterpart: each instance runs its own
 * pass of the Dambreak.cpp:166-220 loop (own advection dt, own acoustic dt and sub-step
 * count, own configuration update), and every kernel launch covers all instances.
 * Particles of all instances are concatenated in one cell-ordered array over one cell
 * index space in which each instance owns a disjoint range; per-instance time steps,
 * relaxation times and sub-step counters stay on the device.
 *
 * Each instance: fluid at rest (rho = rho0) on the given positions, one static wall body
 * with its normals, uniform masses and volumes, gravity as the only prior force, and a
 * cell mesh with grid spacing 2h (at most 16384 cells per axis in 2D, 512 in 3D). */
typedef struct sphx_batch_s *sphx_batch;

typedef struct
{
    sphx_mesh_desc mesh;     /* cell mesh of the instance (grid spacing = 2h) */
    size_t n_fluid, n_wall;
    const double *fluid_pos;   /* n_fluid x dim, AoS */
    const double *wall_pos;    /* n_wall x dim, AoS */
    const double *wall_normal; /* n_wall x dim, AoS (NormalDirectionFromBodyShape) */
    double h;                  /* smoothing length */
    double sigma0;             /* lattice number density (sphx_lattice_number_density) */
    double rho0, c0, U_ref;
    double fluid_mass, fluid_vol;
    double wall_rho0, wall_mass, wall_vol;
    double gravity[3];
} sphx_batch_instance;

/* Copies the descriptions (host arrays may be freed afterwards), sorts the walls, builds
 * the first configuration and the initial time-step maxima (synchronises). */
int sphx_batch_create(sphx_ctx ctx, int dim, int count, const sphx_batch_instance *instances, sphx_batch *out);
int sphx_batch_destroy(sphx_batch batch);
/* One advection step of every instance (the Dambreak.cpp loop order: acoustic dt taken
 * before each relaxation).  use_graph 1: the step runs as one CUDA graph launch whose
 * conditional WHILE node repeats the acoustic sub-step until no instance is active (the
 * graph is built on first use and rebuilt when list storage grows); 0: the same kernels,
 * with the host reading the loop flag after each sub-step.  An instance reaching the
 * sub-step cap (sphx_batch_set_substep_cap) ends the step with SPHX_ERR_TIMEOUT.  Outputs (may be null, else count
 * entries): acoustic sub-steps of this step and physical time per instance. */
int sphx_batch_advection_step(sphx_batch batch, int use_graph, int *substeps, double *physical_time);
/* Block size (64..256, multiple of 32) of the two sweep kernels. */
int sphx_batch_set_tuning(sphx_batch batch, int block);
/* Cap of acoustic sub-steps per instance in one advection step (1..2^20, default 2^20):
 * an instance that reaches it stops relaxing, the step completes its configuration update
 * and returns SPHX_ERR_TIMEOUT.  The device-side loop of the graph therefore always ends.
 * Replaces the reference's unbounded `while (relaxation_time < advection_dt)` of
 * Dambreak.cpp:181-198, which has no failure path. */
int sphx_batch_set_substep_cap(sphx_batch batch, int max_substeps);
/* Graph launches made so far. */
int sphx_batch_graph_launches(sphx_batch batch, uint64_t *out);
/* Fluid state of one instance in its input particle order (any output may be null):
 * pos / vel n_fluid x dim AoS, rho and p n_fluid (synchronises). */
int sphx_batch_download(sphx_batch batch, int instance, double *pos, double *vel, double *rho, double *p);
/* Total fluid and wall particles over all instances. */
int sphx_batch_size(sphx_batch batch, size_t *fluid_particles, size_t *wall_particles);

#ifdef __cplusplus
}
#endif
#endif /* SPHX_H */
