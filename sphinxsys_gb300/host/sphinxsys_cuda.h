// sphinxsys_cuda.h -- C++ host layer over the sphx C ABI: the call-site API of SPHinXsys'
// classic weakly-compressible fluid step, with every dynamics object executing on the
// GB300 through libsphx_cuda.so (execution::CudaDevicePolicy).
//
// A driver written against the reference (tests/2d_examples/test_2d_dambreak/Dambreak.cpp)
// compiles against this header with the same object names, constructor arguments and
// exec() calls for the hot path: SPHSystem, FluidBody / SolidBody / ObserverBody,
// GeometricShapeBox / ComplexShape, InnerRelation / ContactRelation / ComplexRelation,
// Dynamics1Level<fluid_dynamics::Integration1stHalfWithWallRiemann>,
// Dynamics1Level<fluid_dynamics::Integration2ndHalfWithWallRiemann>,
// InteractionWithUpdate<fluid_dynamics::DensitySummationComplexFreeSurface>,
// ReduceDynamics<fluid_dynamics::AdvectionTimeStep / AcousticTimeStep>,
// SimpleDynamics<GravityForce<Gravity>>, SimpleDynamics<NormalDirectionFromBodyShape>,
// ParticleSorting; and for the periodic viscous flow of
// tests/2d_examples/test_2d_taylor_green/taylor_green.cpp: addMaterialProperty<Viscosity>,
// PeriodicAlongAxis / PeriodicConditionUsingCellLinkedList,
// Dynamics1Level<fluid_dynamics::Integration1stHalfInnerRiemann / 2ndHalfInnerNoRiemann>,
// InteractionWithUpdate<fluid_dynamics::DensitySummationInner / ViscousForceInner /
// TransportVelocityCorrectionInner<TruncatedLinear, AllParticles>>,
// ReduceDynamics<fluid_dynamics::AdvectionViscousTimeStep>, and an initial condition
// through SimpleDynamics<T> for a T with a static velocity(position) (run once, on the
// host).  Output classes (VTP, restart, regression databases) are not part of this layer;
// ObservedQuantity / TotalMechanicalEnergy / TotalKineticEnergy / MaximumSpeed return
// their values instead.
//
// Errors: a failing C-ABI call throws SPH::SphxException carrying the status and the
// library message (the reference prints and calls exit(1)).
//
// Dimension: define SPHX_DIMENSION 2 or 3 before including (default 2), as the
// reference builds its 2D and 3D libraries separately.
#pragma once

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <initializer_list>
#include <limits>
#include <memory>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <utility>
#include <vector>

#include "../../include/sphx/sphx.h"

#ifndef SPHX_DIMENSION
#define SPHX_DIMENSION 2
#endif

namespace SPH
{
using Real = double;
constexpr int Dimensions = SPHX_DIMENSION;
constexpr Real Pi = Real(M_PI);

struct Vecd
{
    Real v[3] = {0, 0, 0};
    Vecd() = default;
    Vecd(Real x, Real y) : v{x, y, 0} {}
    Vecd(Real x, Real y, Real z) : v{x, y, z} {}
    Real &operator[](int i) { return v[i]; }
    const Real &operator[](int i) const { return v[i]; }
    static Vecd Zero() { return Vecd(); }
    static Vecd Ones() { return Dimensions == 2 ? Vecd(1, 1) : Vecd(1, 1, 1); }
};
inline Vecd operator+(const Vecd &a, const Vecd &b)
{
    Vecd r;
    for (int d = 0; d < 3; ++d)
        r[d] = a[d] + b[d];
    return r;
}
inline Vecd operator-(const Vecd &a, const Vecd &b)
{
    Vecd r;
    for (int d = 0; d < 3; ++d)
        r[d] = a[d] - b[d];
    return r;
}
inline Vecd operator*(Real s, const Vecd &a)
{
    Vecd r;
    for (int d = 0; d < 3; ++d)
        r[d] = s * a[d];
    return r;
}
using Vec2d = Vecd;
using Vec3d = Vecd;
template <typename T>
using StdVec = std::vector<T>;

class SphxException : public std::runtime_error
{
  public:
    int status;
    SphxException(int s, const std::string &m) : std::runtime_error(m), status(s) {}
};

inline void check(int status)
{
    if (status != SPHX_OK)
        throw SphxException(status, std::string("sphx: ") + sphx_last_error());
}

namespace execution
{
struct CudaDevicePolicy
{
};
} // namespace execution
using MainExecutionPolicy = execution::CudaDevicePolicy;

struct BoundingBoxd
{
    Vecd lower_, upper_;
    BoundingBoxd(const Vecd &lo, const Vecd &up) : lower_(lo), upper_(up) {}
};

struct Transform
{
    Vecd translation;
    explicit Transform(const Vecd &t) : translation(t) {}
};

// ------------------------------------------------------------------ shapes
// GeometricShapeBox (geometric_shape.cpp:6-18, geometric_element.cpp:19-55, .h:43-55)
class Shape
{
  public:
    std::string name_;
    explicit Shape(const std::string &name) : name_(name) {}
    virtual ~Shape() = default;
    virtual bool checkContain(const Vecd &x) const = 0;
    virtual Vecd findClosestPoint(const Vecd &x) const = 0;
    Vecd findNormalDirection(const Vecd &x) const // base_geometry.cpp:45-58
    {
        bool in = checkContain(x);
        Vecd d = findClosestPoint(x) - x;
        Real s = d[0] * d[0] + d[1] * d[1];
        if (Dimensions == 3)
            s = s + d[2] * d[2];
        Real n = std::sqrt(s);
        Vecd out;
        for (int a = 0; a < Dimensions; ++a)
            out[a] = (in ? 1.0 : -1.0) * (d[a] / n);
        return out;
    }
};

class GeometricShapeBox : public Shape
{
  public:
    Vecd c_, hs_;
    GeometricShapeBox(const Transform &t, const Vecd &halfsize, const std::string &name = "GeometricShapeBox")
        : Shape(name), c_(t.translation), hs_(halfsize) {}
    bool checkContain(const Vecd &x) const override
    {
        for (int a = 0; a < Dimensions; ++a)
            if (std::abs(x[a] - c_[a]) > hs_[a])
                return false;
        return true;
    }
    Vecd findClosestPoint(const Vecd &x) const override
    {
        Vecd p;
        bool inside = true;
        for (int a = 0; a < Dimensions; ++a)
        {
            p[a] = x[a] - c_[a];
            if (p[a] < -hs_[a])
            {
                p[a] = -hs_[a];
                inside = false;
            }
            else if (p[a] > hs_[a])
            {
                p[a] = hs_[a];
                inside = false;
            }
        }
        if (inside)
        {
            int which = 0;
            Real mind = hs_[0] - std::abs(p[0]);
            for (int a = 1; a < Dimensions; ++a)
            {
                Real d = hs_[a] - std::abs(p[a]);
                if (d < mind)
                {
                    which = a;
                    mind = d;
                }
            }
            p[which] = p[which] < 0 ? -hs_[which] : hs_[which];
        }
        Vecd out;
        for (int a = 0; a < Dimensions; ++a)
            out[a] = p[a] + c_[a];
        return out;
    }
};

// ComplexShape with add/subtract (BinaryShapes, base_geometry.cpp:84-137)
class ComplexShape : public Shape
{
    std::vector<std::pair<std::shared_ptr<Shape>, bool>> parts_;

  public:
    explicit ComplexShape(const std::string &name) : Shape(name) {}
    template <class S, typename... Args>
    void add(Args &&...args) { parts_.emplace_back(std::make_shared<S>(std::forward<Args>(args)...), true); }
    template <class S, typename... Args>
    void subtract(Args &&...args) { parts_.emplace_back(std::make_shared<S>(std::forward<Args>(args)...), false); }
    bool checkContain(const Vecd &x) const override
    {
        bool exist = false;
        for (auto &p : parts_)
        {
            bool inside = p.first->checkContain(x);
            exist = p.second ? (exist || inside) : (exist && !inside);
        }
        return exist;
    }
    Vecd findClosestPoint(const Vecd &x) const override
    {
        Real dmin = std::numeric_limits<Real>::max();
        Vecd best;
        for (auto &p : parts_)
        {
            Vecd q = p.first->findClosestPoint(x);
            Vecd d = x - q;
            Real s = d[0] * d[0] + d[1] * d[1];
            if (Dimensions == 3)
                s = s + d[2] * d[2];
            Real dist = std::sqrt(s);
            if (dist <= dmin)
            {
                dmin = dist;
                best = q;
            }
        }
        return best;
    }
};

template <class T, typename... Args>
std::shared_ptr<T> makeShared(Args &&...args) { return std::make_shared<T>(std::forward<Args>(args)...); }

// ------------------------------------------------------------------ materials
class WeaklyCompressibleFluid
{
  public:
    Real rho0_, c0_;
    WeaklyCompressibleFluid(Real rho0, Real c0) : rho0_(rho0), c0_(c0) {}
    Real ReferenceDensity() const { return rho0_; }
};
class Solid
{
  public:
    Real rho0_;
    explicit Solid(Real rho0 = 1.0) : rho0_(rho0) {}
    Real ReferenceDensity() const { return rho0_; }
};
struct BaseParticles
{
};
struct ObserverParticles
{
};
class Viscosity
{
  public:
    Real mu_;
    explicit Viscosity(Real mu) : mu_(mu) {}
    Real ReferenceViscosity() const { return mu_; }
};

struct Lattice
{
};

class Gravity
{
  public:
    Vecd g_, reference_;
    explicit Gravity(const Vecd &g, const Vecd &reference = Vecd()) : g_(g), reference_(reference) {}
};

// ------------------------------------------------------------------ system and bodies
class SPHBody;

class SPHSystem
{
  public:
    BoundingBoxd bounds_;
    Real resolution_;
    Real physical_time_ = 0;
    sphx_ctx ctx_ = nullptr;
    std::vector<SPHBody *> bodies_;
    SPHSystem(const BoundingBoxd &bounds, Real resolution, int device = 0) : bounds_(bounds), resolution_(resolution)
    {
        check(sphx_ctx_create(device, nullptr, &ctx_));
    }
    ~SPHSystem() { sphx_ctx_destroy(ctx_); }
    SPHSystem(const SPHSystem &) = delete;
    SPHSystem &operator=(const SPHSystem &) = delete;
    // the options of SPHSystem::handleCommandlineOptions (sph_system.cpp:100-200) this policy
    // uses: --restart_step=<int>, --regression=<bool>, --state_recording=<bool>
    // ("--name=value" or "--name value"); the others are accepted and ignored
    void handleCommandlineOptions(int ac, char *av[])
    {
        for (int i = 1; i < ac; ++i)
        {
            std::string arg(av[i]);
            if (arg.rfind("--", 0) != 0)
                continue;
            std::string name = arg.substr(2), value;
            size_t eq = name.find('=');
            if (eq != std::string::npos)
            {
                value = name.substr(eq + 1);
                name = name.substr(0, eq);
            }
            else if (i + 1 < ac && std::string(av[i + 1]).rfind("--", 0) != 0)
                value = av[++i];
            auto flag = [&value]() { return value == "1" || value == "true" || value == "True"; };
            if (name == "restart_step")
                restart_step_ = std::stoi(value);
            else if (name == "regression")
                generate_regression_data_ = flag();
            else if (name == "state_recording")
                state_recording_ = flag();
        }
    }
    std::string input_folder_ = "./input", output_folder_ = "./output", restart_folder_ = "./restart";
    int restart_step_ = 0;
    bool generate_regression_data_ = false, state_recording_ = true;
    inline void initializeSystemCellLinkedLists();
    inline void initializeSystemConfigurations();
    // SingleVariable<Real> of the CK drivers: getValue / incrementValue over PhysicalTime
    template <typename T>
    struct SingleVariable
    {
        T *value_;
        T getValue() const { return *value_; }
        void incrementValue(T dt) { *value_ += dt; }
    };
    template <typename T>
    SingleVariable<T> *getSystemVariableByName(const std::string &name)
    {
        single_time_.value_ = getSystemVariableDataByName<T>(name);
        return &single_time_;
    }
    SingleVariable<Real> single_time_{nullptr};
    template <typename T>
    T *getSystemVariableDataByName(const std::string &name)
    {
        static_assert(std::is_same<T, Real>::value, "PhysicalTime is a Real");
        if (name != "PhysicalTime")
            throw SphxException(SPHX_ERR_NOT_FOUND, "unknown system variable " + name);
        return &physical_time_;
    }
    int RestartStep() const { return restart_step_; }
    bool GenerateRegressionData() const { return generate_regression_data_; }
    bool StateRecording() const { return state_recording_; }
};

class SPHBody
{
  public:
    SPHSystem &system_;
    std::shared_ptr<Shape> shape_;
    std::string name_;
    Real h_, rho0_ = 1.0, c0_ = 0.0, mu_ = 0.0;
    bool is_fluid_ = false;
    sphx_body body_ = nullptr;
    size_t n_ = 0;
    std::vector<class BaseRelation *> relations_;

    SPHBody(SPHSystem &sys, std::shared_ptr<Shape> shape, const std::string &name)
        : system_(sys), shape_(std::move(shape)), name_(name), h_(1.3 * sys.resolution_)
    {
        sys.bodies_.push_back(this);
    }
    SPHBody(SPHSystem &sys, Shape &shape) : SPHBody(sys, std::shared_ptr<Shape>(&shape, [](Shape *) {}), shape.name_) {}
    SPHBody(SPHSystem &sys, std::shared_ptr<Shape> shape) : SPHBody(sys, shape, shape->name_) {}
    SPHBody(SPHSystem &sys, const std::string &name) : SPHBody(sys, nullptr, name) {}
    virtual ~SPHBody() { sphx_body_destroy(body_); }
    SPHBody(const SPHBody &) = delete;

    template <class Material, typename... Args>
    void defineMatterMaterial(Args &&...args)
    {
        Material m(std::forward<Args>(args)...);
        rho0_ = m.ReferenceDensity();
        if constexpr (std::is_same<Material, WeaklyCompressibleFluid>::value)
        {
            c0_ = m.c0_;
            is_fluid_ = true;
        }
    }
    // addMaterialProperty<Viscosity>(mu)
    template <class Property, typename... Args>
    void addMaterialProperty(Args &&...args)
    {
        Property prop(std::forward<Args>(args)...);
        mu_ = prop.ReferenceViscosity();
    }
    // the bounds of the system domain (the bodies of the supported drivers fill it)
    BoundingBoxd getSPHBodyBounds() const { return system_.bounds_; }
    Real CutOffRadius() const { return 2.0 * h_; }
    size_t TotalRealParticles() const { return n_; }

    // ParticleGenerator<BaseParticles, Lattice> (particle_generator_lattice_{2d,3d}.cpp:12-23)
    template <class ParticlesType, class Generator = Lattice>
    void generateParticles()
    {
        static_assert(std::is_same<Generator, Lattice>::value, "lattice generation only");
        const Vecd &lo = system_.bounds_.lower_, &up = system_.bounds_.upper_;
        Real dp = system_.resolution_;
        int n[3] = {1, 1, 1};
        for (int a = 0; a < Dimensions; ++a)
            n[a] = int(std::ceil((up[a] + 0.0 - lo[a]) / dp));
        std::vector<Vecd> pos;
        for (int i = 0; i < n[0]; ++i)
            for (int j = 0; j < n[1]; ++j)
                for (int k = 0; k < n[2]; ++k)
                {
                    int c[3] = {i, j, k};
                    Vecd x;
                    for (int a = 0; a < Dimensions; ++a)
                        x[a] = (lo[a] + Real(c[a]) * dp) + 0.5 * dp;
                    if (shape_->checkContain(x))
                        pos.push_back(x);
                }
        Real vol = Dimensions == 3 ? dp * dp * dp : dp * dp;
        createParticles(pos, vol);
    }
    // generateParticles<ObserverParticles>(positions)
    template <class ParticlesType>
    void generateParticles(const StdVec<Vecd> &positions) { createParticles(positions, 0.0); }

    void createParticles(const std::vector<Vecd> &pos, Real vol)
    {
        n_ = pos.size();
        check(sphx_body_create(system_.ctx_, Dimensions, n_, &body_));
        std::vector<double> x(n_ * Dimensions);
        for (size_t i = 0; i < n_; ++i)
            for (int a = 0; a < Dimensions; ++a)
                x[i * Dimensions + a] = pos[i][a];
        upload("Position", x, Dimensions);
        std::vector<uint32_t> ids(n_);
        for (size_t i = 0; i < n_; ++i)
            ids[i] = uint32_t(i);
        check(sphx_body_upload(body_, "OriginalID", SPHX_U32, 1, ids.data(), n_));
        check(sphx_body_upload(body_, "SortedID", SPHX_U32, 1, ids.data(), n_));
        if (vol > 0)
        {
            upload("VolumetricMeasure", std::vector<double>(n_, vol), 1);
            upload("Density", std::vector<double>(n_, rho0_), 1);
            upload("Mass", std::vector<double>(n_, rho0_ * vol), 1); // base_material.cpp:37-40
        }
        positions_ = pos;
    }
    void upload(const char *name, const std::vector<double> &v, int ncomp)
    {
        check(sphx_body_upload(body_, name, SPHX_F64, ncomp, v.data(), n_));
    }
    // prepareForOutput: device -> host copy of a variable (AoS, n x ncomp)
    std::vector<double> download(const char *name) const
    {
        void *p;
        sphx_dtype dt;
        int nc;
        check(sphx_body_device_ptr(body_, name, &p, &dt, &nc));
        std::vector<double> out(n_ * nc);
        check(sphx_body_download(body_, name, out.data(), n_));
        return out;
    }
    std::vector<Vecd> positions_; // generated positions (host copy used for shape normals)
};

class RealBody : public SPHBody
{
  public:
    sphx_mesh_desc mesh_{};
    sphx_cell_list cell_list_ = nullptr;
    template <typename... Args>
    RealBody(Args &&...args) : SPHBody(std::forward<Args>(args)...)
    {
        double lo[3] = {0, 0, 0}, up[3] = {0, 0, 0};
        for (int a = 0; a < Dimensions; ++a)
        {
            lo[a] = system_.bounds_.lower_[a];
            up[a] = system_.bounds_.upper_[a];
        }
        // SPHAdaptation::createCellLinkedList: grid spacing = cut-off radius, buffer 2
        check(sphx_mesh_from_bounds(Dimensions, lo, up, CutOffRadius(), 2, &mesh_));
    }
    ~RealBody() override { sphx_cell_list_destroy(cell_list_); }
    sphx_cell_list cellLinkedList()
    {
        if (!cell_list_)
            check(sphx_cell_list_create(system_.ctx_, &mesh_, n_ ? n_ : 1, &cell_list_));
        return cell_list_;
    }
    // RealBody::updateCellLinkedList (base_body.cpp:103-113)
    void updateCellLinkedList() { check(sphx_cell_list_update(cellLinkedList(), body_)); }
};

class FluidBody : public RealBody
{
  public:
    using RealBody::RealBody;
};
class SolidBody : public RealBody
{
  public:
    using RealBody::RealBody;
};
class ObserverBody : public SPHBody
{
  public:
    ObserverBody(SPHSystem &sys, const std::string &name) : SPHBody(sys, name) {}
};

// ------------------------------------------------------------------ relations
class BaseRelation
{
  public:
    sphx_relation rel_ = nullptr;
    SPHBody &body_;
    explicit BaseRelation(SPHBody &b) : body_(b) { b.relations_.push_back(this); }
    virtual ~BaseRelation() { sphx_relation_destroy(rel_); }
    BaseRelation(const BaseRelation &) = delete;
    SPHBody &getSPHBody() { return body_; }
    virtual void updateConfiguration() { check(sphx_relation_update(rel_)); }
};

class InnerRelation : public BaseRelation
{
  public:
    explicit InnerRelation(RealBody &b) : BaseRelation(b)
    {
        check(sphx_inner_relation_create(b.body_, b.cellLinkedList(), b.h_, &rel_));
    }
};

class ContactRelation : public BaseRelation
{
  public:
    RealBody *target_;
    ContactRelation(SPHBody &b, std::initializer_list<RealBody *> targets) : BaseRelation(b), target_(*targets.begin())
    {
        if (targets.size() != 1)
            throw SphxException(SPHX_ERR_INVALID_ARG, "one contact body per relation");
        Real h = std::max(b.h_, target_->h_); // NeighborBuilder::chooseKernel
        int depth = 1 + int(std::floor(b.CutOffRadius() * (1.0 / target_->mesh_.grid_spacing)));
        check(sphx_contact_relation_create(b.body_, target_->body_, target_->cellLinkedList(), h, depth,
                                           target_->rho0_, &rel_));
    }
};

class ComplexRelation
{
  public:
    InnerRelation &inner_;
    ContactRelation &contact_;
    ComplexRelation(InnerRelation &inner, ContactRelation &contact) : inner_(inner), contact_(contact) {}
    void updateConfiguration()
    {
        inner_.updateConfiguration();
        contact_.updateConfiguration();
    }
};

inline void SPHSystem::initializeSystemCellLinkedLists()
{
    for (SPHBody *b : bodies_)
        if (auto *rb = dynamic_cast<RealBody *>(b))
            rb->updateCellLinkedList();
}
inline void SPHSystem::initializeSystemConfigurations()
{
    for (SPHBody *b : bodies_)
        for (BaseRelation *r : b->relations_)
            r->updateConfiguration();
}

// ------------------------------------------------------------------ dynamics
namespace fluid_dynamics
{
struct Integration1stHalfWithWallRiemann
{
};
struct Integration2ndHalfWithWallRiemann
{
};
struct DensitySummationComplexFreeSurface
{
};
struct AcousticTimeStep
{
};
struct AdvectionTimeStep
{
};
struct Integration1stHalfInnerRiemann
{
};
struct Integration2ndHalfInnerNoRiemann
{
};
struct DensitySummationInner
{
};
struct ViscousForceInner
{
};
template <class LimiterType, class ParticleScope>
struct TransportVelocityCorrectionInner
{
};
struct AdvectionViscousTimeStep
{
};
} // namespace fluid_dynamics
struct TruncatedLinear
{
};
struct AllParticles
{
};
template <class GravityType>
struct GravityForce
{
};
struct NormalDirectionFromBodyShape
{
};

inline sphx_fluid_params fluidParams(SPHBody &b, Real U_ref = 0.0)
{
    // registerStateVariable of the fluid-step variables (fluid_integration.hpp:10-22)
    for (const char *v : {"Velocity", "Force", "ForcePrior"})
        check(sphx_body_register(b.body_, v, SPHX_F64, Dimensions));
    for (const char *v : {"Pressure", "DensityChangeRate", "DensitySummation"})
        check(sphx_body_register(b.body_, v, SPHX_F64, 1));
    sphx_fluid_params p{};
    p.rho0 = b.rho0_;
    p.c0 = b.c0_;
    p.h = b.h_;
    check(sphx_lattice_number_density(Dimensions, b.h_, b.system_.resolution_, &p.sigma0));
    p.limiter_slope = 3.0;
    p.acoustic_cfl = 0.6;
    p.advection_cfl = 0.25;
    p.U_ref = U_ref;
    return p;
}

template <class LocalDynamicsType, class ExecutionPolicy = execution::CudaDevicePolicy>
class Dynamics1Level
{
    static_assert(std::is_same<ExecutionPolicy, execution::CudaDevicePolicy>::value, "CUDA policy only");
    static constexpr bool first =
        std::is_same<LocalDynamicsType, fluid_dynamics::Integration1stHalfWithWallRiemann>::value ||
        std::is_same<LocalDynamicsType, fluid_dynamics::Integration1stHalfInnerRiemann>::value;
    static constexpr bool second =
        std::is_same<LocalDynamicsType, fluid_dynamics::Integration2ndHalfWithWallRiemann>::value ||
        std::is_same<LocalDynamicsType, fluid_dynamics::Integration2ndHalfInnerNoRiemann>::value;
    static_assert(first || second, "unsupported Dynamics1Level type");
    InnerRelation &inner_;
    ContactRelation *contact_;
    sphx_fluid_params p_;

  public:
    Dynamics1Level(InnerRelation &inner, ContactRelation &contact)
        : inner_(inner), contact_(&contact), p_(fluidParams(inner.getSPHBody())) {}
    // the inner-only forms (Integration1stHalfInnerRiemann, Integration2ndHalfInnerNoRiemann:
    // NoRiemannSolver is the acoustic solver with limiter slope 0, its pressure dissipation
    // vanishes)
    explicit Dynamics1Level(InnerRelation &inner)
        : inner_(inner), contact_(nullptr), p_(fluidParams(inner.getSPHBody()))
    {
        if (std::is_same<LocalDynamicsType, fluid_dynamics::Integration2ndHalfInnerNoRiemann>::value)
            p_.limiter_slope = 0.0;
    }
    void exec(Real dt = 0.0)
    {
        sphx_relation wall = contact_ ? contact_->rel_ : nullptr;
        if constexpr (first)
            check(sphx_integration_1st_half_with_wall_riemann(inner_.rel_, wall, &p_, dt));
        else
            check(sphx_integration_2nd_half_with_wall_riemann(inner_.rel_, wall, &p_, dt));
    }
};

template <class T>
struct IsTransportVelocityCorrection : std::false_type
{
};
template <class L, class S>
struct IsTransportVelocityCorrection<fluid_dynamics::TransportVelocityCorrectionInner<L, S>> : std::true_type
{
};

template <class LocalDynamicsType, class ExecutionPolicy = execution::CudaDevicePolicy>
class InteractionWithUpdate
{
    static constexpr bool complex =
        std::is_same<LocalDynamicsType, fluid_dynamics::DensitySummationComplexFreeSurface>::value;
    static constexpr bool inner_sum = std::is_same<LocalDynamicsType, fluid_dynamics::DensitySummationInner>::value;
    static constexpr bool viscous = std::is_same<LocalDynamicsType, fluid_dynamics::ViscousForceInner>::value;
    static constexpr bool tvc = IsTransportVelocityCorrection<LocalDynamicsType>::value;
    static_assert(complex || inner_sum || viscous || tvc, "unsupported interaction");
    InnerRelation &inner_;
    ContactRelation *contact_;
    sphx_fluid_params p_;
    Real coefficient_ = 0.2;

  public:
    InteractionWithUpdate(InnerRelation &inner, ContactRelation &contact)
        : inner_(inner), contact_(&contact), p_(fluidParams(inner.getSPHBody())) {}
    // inner forms; TransportVelocityCorrectionInner takes the correction coefficient (0.2)
    explicit InteractionWithUpdate(InnerRelation &inner, Real coefficient = 0.2)
        : inner_(inner), contact_(nullptr), p_(fluidParams(inner.getSPHBody())), coefficient_(coefficient)
    {
        if constexpr (viscous)
            check(sphx_relation_keep_distances(inner.rel_)); // the viscous force needs r_ij
    }
    void exec(Real = 0.0)
    {
        if constexpr (complex)
            check(sphx_density_summation_complex_free_surface(inner_.rel_, contact_ ? contact_->rel_ : nullptr,
                                                              &p_));
        else if constexpr (inner_sum)
            check(sphx_density_summation_inner(inner_.rel_, &p_));
        else if constexpr (viscous)
            check(sphx_viscous_force_inner(inner_.rel_, inner_.getSPHBody().mu_));
        else
            check(sphx_transport_velocity_correction_inner(inner_.rel_, coefficient_));
    }
};

template <class LocalDynamicsType, class ExecutionPolicy = execution::CudaDevicePolicy>
class ReduceDynamics
{
    SPHBody &body_;
    sphx_fluid_params p_;

  public:
    explicit ReduceDynamics(SPHBody &body, Real U_ref = 0.0) : body_(body), p_(fluidParams(body, U_ref))
    {
        // AdvectionViscousTimeStep: reference speed max(U_ref, mu / rho0 / h) (fluid_time_step.cpp:67-74)
        if (std::is_same<LocalDynamicsType, fluid_dynamics::AdvectionViscousTimeStep>::value)
            p_.U_ref = std::max(U_ref, body.mu_ / body.rho0_ / body.h_);
    }
    Real exec(Real = 0.0)
    {
        Real dt;
        if constexpr (std::is_same<LocalDynamicsType, fluid_dynamics::AcousticTimeStep>::value)
            check(sphx_acoustic_time_step(body_.body_, &p_, &dt));
        else
            check(sphx_advection_time_step(body_.body_, &p_, &dt));
        return dt;
    }
};

template <class T, class = void>
struct HasVelocityField : std::false_type
{
};
template <class T>
struct HasVelocityField<T, decltype(void(T::velocity(Vecd())))> : std::true_type
{
};

template <class LocalDynamicsType, class ExecutionPolicy = execution::CudaDevicePolicy>
class SimpleDynamics
{
    SPHBody &body_;
    Vecd g_;

  public:
    explicit SimpleDynamics(SPHBody &body) : body_(body) {}
    SimpleDynamics(SPHBody &body, const Gravity &g) : body_(body), g_(g.g_) {}
    void exec(Real = 0.0)
    {
        if constexpr (HasVelocityField<LocalDynamicsType>::value)
        {
            // an initial condition: Velocity from the current Position, on the host
            std::vector<double> x = body_.download("Position"), v(body_.n_ * Dimensions);
            for (size_t i = 0; i < body_.n_; ++i)
            {
                Vecd p;
                for (int a = 0; a < Dimensions; ++a)
                    p[a] = x[i * Dimensions + a];
                Vecd u = LocalDynamicsType::velocity(p);
                for (int a = 0; a < Dimensions; ++a)
                    v[i * Dimensions + a] = u[a];
            }
            body_.upload("Velocity", v, Dimensions);
        }
        else if constexpr (std::is_same<LocalDynamicsType, NormalDirectionFromBodyShape>::value)
        {
            std::vector<double> n(body_.n_ * Dimensions);
            for (size_t i = 0; i < body_.n_; ++i)
            {
                Vecd d = body_.shape_->findNormalDirection(body_.positions_[i]);
                for (int a = 0; a < Dimensions; ++a)
                    n[i * Dimensions + a] = d[a];
            }
            body_.upload("NormalDirection", n, Dimensions);
        }
        else
            check(sphx_gravity_force(body_.body_, g_.v));
    }
};

class ParticleSorting
{
    RealBody &body_;

  public:
    explicit ParticleSorting(RealBody &body) : body_(body) {}
    void exec(Real = 0.0) { check(sphx_particle_sorting(body_.body_, &body_.mesh_)); }
};

// ObservingAQuantity<Real> over an observer contact relation.
class ObservedQuantity
{
    ContactRelation &contact_;
    std::string name_;

  public:
    ObservedQuantity(const std::string &name, ContactRelation &contact) : contact_(contact), name_(name) {}
    std::vector<Real> exec()
    {
        std::vector<Real> out(contact_.getSPHBody().n_);
        if (!out.empty())
            check(sphx_observe_quantity(contact_.rel_, name_.c_str(), out.data()));
        return out;
    }
};

// ------------------------------------------------------------------ periodic boundaries
constexpr int xAxis = 0, yAxis = 1, zAxis = 2;

struct PeriodicAlongAxis
{
    Real lower_, upper_;
    int axis_;
    PeriodicAlongAxis(const BoundingBoxd &bounds, int axis)
        : lower_(bounds.lower_[axis]), upper_(bounds.upper_[axis]), axis_(axis) {}
};

// PeriodicConditionUsingCellLinkedList (domain_bounding.h:149-176): bounding_ wraps the
// positions; the images of update_cell_linked_list_ are inserted by every later update of
// the body's cell list once the axis is registered, so its exec() has nothing left to do.
class PeriodicConditionUsingCellLinkedList
{
  public:
    struct Bounding
    {
        RealBody &body_;
        PeriodicAlongAxis axis_;
        void exec(Real = 0.0) { check(sphx_periodic_bounding(body_.body_, axis_.axis_, axis_.lower_, axis_.upper_)); }
    } bounding_;
    struct UpdateCellLinkedList
    {
        void exec(Real = 0.0) {}
    } update_cell_linked_list_;
    PeriodicConditionUsingCellLinkedList(RealBody &body, PeriodicAlongAxis &periodic) : bounding_{body, periodic}
    {
        check(sphx_cell_list_set_periodic(body.cellLinkedList(), periodic.axis_, periodic.lower_, periodic.upper_,
                                          body.CutOffRadius()));
    }
};

class TotalKineticEnergy
{
    SPHBody &body_;

  public:
    explicit TotalKineticEnergy(SPHBody &body) : body_(body) {}
    Real exec()
    {
        Real e;
        double g[3] = {0, 0, 0};
        check(sphx_total_mechanical_energy(body_.body_, g, &e));
        return e;
    }
};

class MaximumSpeed
{
    SPHBody &body_;

  public:
    explicit MaximumSpeed(SPHBody &body) : body_(body) {}
    Real exec()
    {
        Real v;
        check(sphx_maximum_speed(body_.body_, &v));
        return v;
    }
};

// ------------------------------------------------------------------ CK call sites
// The computing-kernel forms of the tests_sycl drivers
// (tests/tests_sycl/3d_examples/test_3d_dambreak_sycl/dambreak.cpp:97-148):
// Inner<> / Contact<> relations, UpdateCellLinkedList / UpdateRelation / ParticleSortCK,
// StateDynamics, InteractionDynamicsCK and ReduceDynamicsCK templated on the execution
// policy, each exec() one call of the sphx_ck_* ABI.
template <typename... Parameters>
class Inner : public InnerRelation
{
  public:
    using InnerRelation::InnerRelation;
};
template <typename... Parameters>
class Contact : public ContactRelation
{
  public:
    using ContactRelation::ContactRelation;
};

template <class ExecutionPolicy, class BodyType>
class UpdateCellLinkedList
{
    RealBody &body_;

  public:
    explicit UpdateCellLinkedList(RealBody &body) : body_(body) {}
    void exec(Real = 0.0) { body_.updateCellLinkedList(); }
};

template <class ExecutionPolicy, class... RelationTypes>
class UpdateRelation
{
    std::vector<BaseRelation *> relations_;

  public:
    template <class... Relations>
    explicit UpdateRelation(Relations &...relations) : relations_{&relations...} {}
    void exec(Real = 0.0)
    {
        for (BaseRelation *r : relations_)
            r->updateConfiguration();
    }
};

// ParticleSortCK: Morton order of the cell-linked-list mesh; every registered variable is
// permuted (the CK state included), relations must be updated afterwards as the driver does
template <class ExecutionPolicy>
class ParticleSortCK
{
    RealBody &body_;

  public:
    explicit ParticleSortCK(RealBody &body) : body_(body) {}
    void exec(Real = 0.0) { check(sphx_particle_sorting(body_.body_, &body_.mesh_)); }
};

template <class GravityType>
struct GravityForceCK
{
};
struct NormalFromBodyShapeCK
{
};
struct LinearCorrectionMatrixComplex
{
};
struct FreeSurface
{
};
namespace fluid_dynamics
{
struct AdvectionStepSetup
{
};
struct UpdateParticlePosition
{
};
template <class... Relations>
struct CompressionSummation
{
};
template <class... Parameters> // <SPHBody, WeaklyCompressibleFluid, FreeSurface>
struct DensityRegularization
{
};
struct AcousticStep1stHalfWithWallRiemannCorrectionCK
{
};
struct AcousticStep2ndHalfWithWallRiemannCorrectionCK
{
};
struct FreeSurfaceIndicationComplexSpatialTemporalCK
{
};
struct AdvectionTimeStepCK
{
};
template <class FluidType>
struct AcousticTimeStepCK
{
};
} // namespace fluid_dynamics

template <class T>
struct IsCompressionSummation : std::false_type
{
};
template <class... R>
struct IsCompressionSummation<fluid_dynamics::CompressionSummation<R...>> : std::true_type
{
};
template <class T>
struct IsDensityRegularization : std::false_type
{
};
template <class... P>
struct IsDensityRegularization<fluid_dynamics::DensityRegularization<P...>> : std::true_type
{
};
template <class T>
struct IsAcousticTimeStepCK : std::false_type
{
};
template <class F>
struct IsAcousticTimeStepCK<fluid_dynamics::AcousticTimeStepCK<F>> : std::true_type
{
};

// BaseDynamics<ReturnType>: what containers, triggers and the time stepper hold
template <typename ReturnType>
class BaseDynamics
{
  public:
    virtual ~BaseDynamics() = default;
    virtual ReturnType exec(Real dt = 0.0) = 0;
};

// DynamicsArgs(relation, parameter): a relation with its constructor argument
struct DynamicsArgs
{
    InnerRelation &inner_;
    Real value_;
    DynamicsArgs(InnerRelation &inner, Real value) : inner_(inner), value_(value) {}
};

template <class ExecutionPolicy, class DynamicsType>
class StateDynamics
{
    SPHBody &body_;
    Vecd g_;

  public:
    explicit StateDynamics(SPHBody &body) : body_(body) {}
    StateDynamics(SPHBody &body, const Gravity &g) : body_(body), g_(g.g_) {}
    void exec(Real = 0.0)
    {
        if constexpr (std::is_same<DynamicsType, GravityForceCK<Gravity>>::value)
            check(sphx_gravity_force(body_.body_, g_.v));
        else if constexpr (std::is_same<DynamicsType, NormalFromBodyShapeCK>::value)
            SimpleDynamics<NormalDirectionFromBodyShape>(body_).exec();
        else if constexpr (std::is_same<DynamicsType, fluid_dynamics::AdvectionStepSetup>::value)
            check(sphx_ck_advection_step_setup(body_.body_));
        else if constexpr (std::is_same<DynamicsType, fluid_dynamics::UpdateParticlePosition>::value)
            check(sphx_ck_update_particle_position(body_.body_));
        else
        {
            static_assert(IsDensityRegularization<DynamicsType>::value, "unsupported state dynamics");
            check(sphx_ck_free_surface_regularization(body_.body_, body_.rho0_));
        }
    }
};

template <class ExecutionPolicy, class DynamicsType>
class InteractionDynamicsCK
{
    InnerRelation &inner_;
    ContactRelation &contact_;
    sphx_fluid_params p_;
    Real alpha_ = 0.5;

  public:
    InteractionDynamicsCK(InnerRelation &inner, ContactRelation &contact)
        : inner_(inner), contact_(contact), p_(fluidParams(inner.getSPHBody())) {}
    InteractionDynamicsCK(DynamicsArgs args, ContactRelation &contact)
        : inner_(args.inner_), contact_(contact), p_(fluidParams(args.inner_.getSPHBody())), alpha_(args.value_) {}
    void exec(Real dt = 0.0)
    {
        if constexpr (std::is_same<DynamicsType, LinearCorrectionMatrixComplex>::value)
            check(sphx_ck_linear_correction_matrix(inner_.rel_, contact_.rel_, alpha_));
        else if constexpr (std::is_same<DynamicsType,
                                        fluid_dynamics::AcousticStep1stHalfWithWallRiemannCorrectionCK>::value)
            check(sphx_ck_acoustic_step_1st_half(inner_.rel_, contact_.rel_, &p_, dt));
        else if constexpr (std::is_same<DynamicsType,
                                        fluid_dynamics::AcousticStep2ndHalfWithWallRiemannCorrectionCK>::value)
            check(sphx_ck_acoustic_step_2nd_half(inner_.rel_, contact_.rel_, &p_, dt));
        else if constexpr (std::is_same<DynamicsType,
                                        fluid_dynamics::FreeSurfaceIndicationComplexSpatialTemporalCK>::value)
            check(sphx_ck_free_surface_indication(inner_.rel_, contact_.rel_));
        else
        {
            static_assert(IsCompressionSummation<DynamicsType>::value, "unsupported interaction dynamics");
            check(sphx_ck_compression_summation(inner_.rel_, contact_.rel_));
        }
    }
};

template <class ExecutionPolicy, class DynamicsType>
class ReduceDynamicsCK : public BaseDynamics<Real>
{
    SPHBody &body_;
    sphx_fluid_params p_;

  public:
    explicit ReduceDynamicsCK(SPHBody &body, Real U_ref = 0.0) : body_(body), p_(fluidParams(body, U_ref)) {}
    Real exec(Real = 0.0) override
    {
        Real dt;
        if constexpr (IsAcousticTimeStepCK<DynamicsType>::value)
            check(sphx_ck_acoustic_time_step(body_.body_, &p_, &dt));
        else
        {
            static_assert(std::is_same<DynamicsType, fluid_dynamics::AdvectionTimeStepCK>::value,
                          "unsupported reduce dynamics");
            check(sphx_ck_advection_time_step(body_.body_, &p_, &dt));
        }
        return dt;
    }
};

// ObservedQuantityRecording<MainExecutionPolicy, Real>(name, observer contact) of the CK
// drivers: the tabulated-kernel interpolation with the current volumes, returned.
class ObservedQuantityCK
{
    ContactRelation &contact_;
    std::string name_;

  public:
    ObservedQuantityCK(const std::string &name, ContactRelation &contact) : contact_(contact), name_(name) {}
    std::vector<Real> exec()
    {
        std::vector<Real> out(contact_.getSPHBody().n_);
        if (!out.empty())
            check(sphx_ck_observe_quantity(contact_.rel_, name_.c_str(), out.data()));
        return out;
    }
};

class TotalMechanicalEnergy
{
    SPHBody &body_;
    Gravity g_;

  public:
    TotalMechanicalEnergy(SPHBody &body, const Gravity &g) : body_(body), g_(g) {}
    Real exec()
    {
        Real e;
        check(sphx_total_mechanical_energy(body_.body_, g_.g_.v, &e));
        return e;
    }
};
} // namespace SPH

#include "sph_solver_cuda.h"
