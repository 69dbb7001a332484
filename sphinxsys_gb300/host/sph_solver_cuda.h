/**
 * Particle-method containers, time stepper, state/restart output and the dynamic-time-
 * warping regression test of the CK drivers, on the CUDA execution policy.
 *
 * Mirrors the interfaces a driver such as
 * tests/tests_sycl/2d_examples/test_2d_dambreak_sycl/dambreak_sycl.cpp calls:
 *   SPHSolver / TimeStepper / TriggerByInterval   src/shared/shared_ck/particle_dynamics/sph_solver.h:57-200
 *   ParticleMethodContainer (add...Dynamics)      src/shared/shared_ck/particle_dynamics/particle_method_container.h:205-530
 *   addPostContactInteraction / addPostStateDynamics  src/shared/shared_ck/particle_dynamics/interaction_algorithms_ck.h:100-125
 *   BodyStatesRecordingToVtpCK                    src/shared/io_system/io_vtk.cpp:165-248 (file layout)
 *   RestartIOCK                                   src/shared/io_system/io_base.cpp:67-110 (file layout)
 *   RegressionTestDynamicTimeWarping              src/shared/regression_test/dynamic_time_warping_method.hpp:17-190
 * Every dynamics object a container creates is one call of the sphx_* ABI; the container
 * only owns the objects.  Included by sphinxsys_cuda.h.
 */
#pragma once

#include <cerrno>
#include <chrono>
#include <cstdio>
#include <fstream>
#include <iomanip>
#include <iostream>
#include <sstream>
#include <sys/stat.h>
#include <sys/types.h>

namespace SPH
{
namespace execution
{
struct ParallelPolicy
{
};
} // namespace execution
// par_ck: the policy of the CK particle methods (here the CUDA device); par_host: host
// methods (execution_policy.h:79-82)
inline constexpr execution::CudaDevicePolicy par_ck{};
inline constexpr execution::ParallelPolicy par_host{};

// TickCount / TimeInterval: the wall-clock statistics of the drivers
class TimeInterval
{
    double seconds_ = 0.0;

  public:
    TimeInterval() = default;
    explicit TimeInterval(double seconds) : seconds_(seconds) {}
    TimeInterval &operator+=(const TimeInterval &o)
    {
        seconds_ += o.seconds_;
        return *this;
    }
    TimeInterval operator-(const TimeInterval &o) const { return TimeInterval(seconds_ - o.seconds_); }
    double seconds() const { return seconds_; }
};
class TickCount
{
    std::chrono::steady_clock::time_point t_;

  public:
    static TickCount now()
    {
        TickCount t;
        t.t_ = std::chrono::steady_clock::now();
        return t;
    }
    TimeInterval operator-(const TickCount &o) const
    {
        return TimeInterval(std::chrono::duration<double>(t_ - o.t_).count());
    }
};

// control parameters of the CK interaction groups
struct OneLevel
{
};
struct WithUpdate
{
};
struct Wall
{
};
struct AcousticRiemannSolverCK
{
};
struct LinearCorrectionCK
{
};
template <typename... Parameters>
struct LinearCorrectionMatrix
{
};
template <typename... Parameters>
class TotalMechanicalEnergyCK
{
};
template <typename... Parameters>
class RegressionTestDynamicTimeWarping
{
};
template <typename... Parameters>
class BodyStatesRecordingToVtpCK;
template <typename... Parameters>
class RestartIOCK;
namespace fluid_dynamics
{
template <typename... Parameters>
struct AcousticStep1stHalf
{
};
template <typename... Parameters>
struct AcousticStep2ndHalf
{
};
} // namespace fluid_dynamics

template <template <typename...> class A, template <typename...> class B>
struct IsSameTemplate : std::false_type
{
};
template <template <typename...> class A>
struct IsSameTemplate<A, A> : std::true_type
{
};

// ------------------------------------------------------------------ interaction groups
// addInteractionDynamics<InteractionType, ControlParameters...>(inner[, parameter]) with
// .addPostContactInteraction<...>(wall contact) and .addPostStateDynamics<...>(body): the
// inner and contact parts run as one fused kernel of the sphx_ck_* ABI, which needs the
// wall contact; a post state dynamics (DensityRegularization after CompressionSummation)
// is fused into the same kernel.
template <class ExecutionPolicy, template <typename...> class InteractionType>
class InteractionGroupCK : public BaseDynamics<void>
{
    InnerRelation &inner_;
    ContactRelation *contact_ = nullptr;
    SPHBody *post_state_ = nullptr;
    sphx_fluid_params p_;
    Real parameter_;

  public:
    explicit InteractionGroupCK(InnerRelation &inner, Real parameter = 0.5)
        : inner_(inner), p_(fluidParams(inner.getSPHBody())), parameter_(parameter) {}
    template <typename... ContactParameters>
    InteractionGroupCK &addPostContactInteraction(ContactRelation &contact)
    {
        contact_ = &contact;
        return *this;
    }
    template <template <typename...> class UpdateType, typename... ControlParameters>
    InteractionGroupCK &addPostStateDynamics(SPHBody &body)
    {
        static_assert(IsSameTemplate<UpdateType, fluid_dynamics::DensityRegularization>::value &&
                          IsSameTemplate<InteractionType, fluid_dynamics::CompressionSummation>::value,
                      "post state dynamics: DensityRegularization after CompressionSummation");
        post_state_ = &body;
        return *this;
    }
    void exec(Real dt = 0.0) override
    {
        if (!contact_)
            throw SphxException(SPHX_ERR_INVALID_ARG, "the CK interactions of this policy need their wall contact "
                                                      "(addPostContactInteraction)");
        if constexpr (IsSameTemplate<InteractionType, LinearCorrectionMatrix>::value)
            check(sphx_ck_linear_correction_matrix(inner_.rel_, contact_->rel_, parameter_));
        else if constexpr (IsSameTemplate<InteractionType, fluid_dynamics::AcousticStep1stHalf>::value)
            check(sphx_ck_acoustic_step_1st_half(inner_.rel_, contact_->rel_, &p_, dt));
        else if constexpr (IsSameTemplate<InteractionType, fluid_dynamics::AcousticStep2ndHalf>::value)
            check(sphx_ck_acoustic_step_2nd_half(inner_.rel_, contact_->rel_, &p_, dt));
        else
        {
            static_assert(IsSameTemplate<InteractionType, fluid_dynamics::CompressionSummation>::value,
                          "unsupported interaction dynamics");
            if (post_state_)
                check(sphx_ck_density_regularization(inner_.rel_, contact_->rel_, &p_));
            else
                check(sphx_ck_compression_summation(inner_.rel_, contact_->rel_));
        }
    }
};

// ------------------------------------------------------------------ output folders
inline void makeFolder(const std::string &path)
{
    if (mkdir(path.c_str(), 0755) != 0 && errno != EEXIST)
        throw SphxException(SPHX_ERR_INVALID_ARG, "cannot create folder " + path);
}

// padValueWithZeros (io_base.h:72-77)
inline std::string padValueWithZeros(long long value, size_t width = 10)
{
    std::string s = std::to_string(value);
    return s.size() < width ? std::string(width - s.size(), '0') + s : s;
}

// a registered variable: type, components and the host copy (AoS) as doubles
struct HostVariable
{
    bool found = false;
    bool is_u32 = false;
    int ncomp = 0;
    std::vector<double> values;
};
inline HostVariable downloadVariable(const SPHBody &body, const std::string &name)
{
    HostVariable v;
    void *p;
    sphx_dtype dt;
    int nc;
    if (body.body_ == nullptr || sphx_body_device_ptr(body.body_, name.c_str(), &p, &dt, &nc) != SPHX_OK)
        return v;
    v.found = true;
    v.is_u32 = dt == SPHX_U32;
    v.ncomp = nc;
    size_t count = body.n_ * size_t(nc);
    if (v.is_u32)
    {
        std::vector<uint32_t> raw(count);
        if (count)
            check(sphx_body_download(body.body_, name.c_str(), raw.data(), body.n_));
        v.values.assign(raw.begin(), raw.end());
    }
    else
    {
        v.values.resize(count);
        if (count)
            check(sphx_body_download(body.body_, name.c_str(), v.values.data(), body.n_));
    }
    return v;
}

// ------------------------------------------------------------------ state files
// BodyStatesRecordingToVtpCK(sph_system): one VTK XML PolyData file per real body and
// output, <output>/<Body>_<sequence>.vtp, with positions, SortedParticle_ID and every
// variable added with addToWrite (io_vtk.cpp:165-248 layout, ascii).
template <>
class BodyStatesRecordingToVtpCK<>
{
    SPHSystem &sys_;
    std::vector<std::pair<SPHBody *, std::string>> to_write_;

    static void writeArray(std::ofstream &out, const std::string &name, const HostVariable &v, size_t n, int dim)
    {
        if (v.is_u32)
        {
            out << "    <DataArray Name=\"" << name << "\" type=\"Int32\" format=\"ascii\">\n    ";
            for (double x : v.values)
                out << static_cast<long long>(x) << " ";
        }
        else
        {
            int comps = v.ncomp == 1 ? 1 : (v.ncomp <= 3 ? 3 : 9);
            out << "    <DataArray Name=\"" << name << "\" type=\"Float32\"";
            if (comps > 1)
                out << "  NumberOfComponents=\"" << comps << "\"";
            out << " format=\"ascii\">\n    ";
            char buf[64];
            for (size_t i = 0; i < n; ++i)
                for (int c = 0; c < comps; ++c)
                {
                    double x = 0.0;
                    if (comps == 1)
                        x = v.values[i];
                    else if (comps == 3)
                        x = c < v.ncomp ? v.values[i * v.ncomp + c] : 0.0;
                    else // dim x dim matrix, written column by column as a 3 x 3 one
                    {
                        int col = c / 3, row = c % 3;
                        if (row < dim && col < dim)
                            x = v.values[i * v.ncomp + row * dim + col];
                    }
                    snprintf(buf, sizeof(buf), "%.9f ", x);
                    out << buf;
                }
        }
        out << "\n    </DataArray>\n";
    }

  public:
    explicit BodyStatesRecordingToVtpCK(SPHSystem &sys) : sys_(sys) {}
    template <typename T>
    void addToWrite(SPHBody &body, const std::string &name)
    {
        to_write_.emplace_back(&body, name);
    }
    // sequence: the physical time in microseconds, or ite_ + the iteration (io_base.cpp:14-54)
    void writeToFile() { write(padValueWithZeros(static_cast<long long>(sys_.physical_time_ * 1.0e6))); }
    void writeToFile(size_t iteration) { write("ite_" + padValueWithZeros(static_cast<long long>(iteration))); }
    void write(const std::string &sequence)
    {
        if (!sys_.StateRecording())
            return;
        makeFolder(sys_.output_folder_);
        for (SPHBody *b : sys_.bodies_)
        {
            if (dynamic_cast<RealBody *>(b) == nullptr || b->n_ == 0)
                continue;
            const size_t n = b->n_;
            std::ofstream out(sys_.output_folder_ + "/" + b->name_ + "_" + sequence + ".vtp");
            out << "<?xml version=\"1.0\"?>\n<VTKFile type=\"PolyData\" version=\"1.0\" byte_order=\"LittleEndian\">\n"
                << " <PolyData>\n<FieldData>\n<DataArray type=\"Float64\"  Name=\"TimeValue\" NumberOfTuples=\"1\" "
                   "format=\"ascii\">\n";
            char buf[64];
            snprintf(buf, sizeof(buf), "%.9f", sys_.physical_time_);
            out << buf << "\n </DataArray>\n</FieldData>\n";
            out << "  <Piece Name =\"" << b->name_ << "\" NumberOfPoints=\"" << n << "\" NumberOfVerts=\"" << n
                << "\">\n   <Points>\n";
            HostVariable pos = downloadVariable(*b, "Position");
            writeArray(out, "Position", pos, n, Dimensions);
            out << "   </Points>\n   <PointData  Vectors=\"vector\">\n";
            out << "    <DataArray Name=\"SortedParticle_ID\" type=\"Int32\" format=\"ascii\">\n    ";
            for (size_t i = 0; i < n; ++i)
                out << i << " ";
            out << "\n    </DataArray>\n";
            for (auto &w : to_write_)
                if (w.first == b)
                {
                    HostVariable v = downloadVariable(*b, w.second);
                    if (!v.found)
                        throw SphxException(SPHX_ERR_NOT_FOUND, "variable " + w.second + " of " + b->name_ +
                                                                    " is not registered");
                    writeArray(out, w.second, v, n, Dimensions);
                }
            out << "   </PointData>\n   <Verts>\n    <DataArray type=\"Int32\"  Name=\"connectivity\"  "
                   "format=\"ascii\">\n    ";
            for (size_t i = 0; i < n; ++i)
                out << i << " ";
            out << "\n    </DataArray>\n    <DataArray type=\"Int32\"  Name=\"offsets\"  format=\"ascii\">\n    ";
            for (size_t i = 0; i < n; ++i)
                out << i + 1 << " ";
            out << "\n    </DataArray>\n   </Verts>\n  </Piece>\n </PolyData>\n</VTKFile>\n";
        }
    }
};

// RestartIOCK(sph_system): <restart>/Restart_<10-digit step>.xml with a restart_data root
// (restart_time attribute), one body element per real body and one particle element per
// particle whose attributes are the body's evolving variables, 17 significant digits
// (io_base.cpp:67-110 layout).  Matrices are not written: the set-up after a restart
// recomputes them.
template <>
class RestartIOCK<>
{
    SPHSystem &sys_;

    static const std::vector<std::string> &fluidVariables()
    {
        static const std::vector<std::string> v = {
            "Position", "Velocity", "Force", "ForcePrior", "Density", "Pressure", "DensityChangeRate", "Mass",
            "VolumetricMeasure", "Compression", "CompressionRate", "Displacement", "VolumetricMeasureRef"};
        return v;
    }
    static const std::vector<std::string> &solidVariables()
    {
        static const std::vector<std::string> v = {"Position", "NormalDirection", "Mass", "VolumetricMeasure",
                                                   "Density"};
        return v;
    }
    std::string path(size_t step) const
    {
        return sys_.restart_folder_ + "/Restart_" + padValueWithZeros(static_cast<long long>(step)) + ".xml";
    }

  public:
    explicit RestartIOCK(SPHSystem &sys) : sys_(sys) {}
    void writeToFile(size_t step)
    {
        makeFolder(sys_.restart_folder_);
        std::ofstream out(path(step));
        char buf[64];
        snprintf(buf, sizeof(buf), "%.17g", sys_.physical_time_);
        out << "<restart_data restart_time=\"" << buf << "\">\n";
        for (SPHBody *b : sys_.bodies_)
        {
            if (dynamic_cast<RealBody *>(b) == nullptr || b->n_ == 0)
                continue;
            std::vector<std::pair<std::string, HostVariable>> vars;
            for (const std::string &nm : b->is_fluid_ ? fluidVariables() : solidVariables())
            {
                HostVariable v = downloadVariable(*b, nm);
                if (v.found && !v.is_u32)
                    vars.emplace_back(nm, std::move(v));
            }
            out << "    <body name=\"" << b->name_ << "\">\n";
            for (size_t i = 0; i < b->n_; ++i)
            {
                out << "        <particle";
                for (auto &nv : vars)
                {
                    out << " " << nv.first << "=\"";
                    for (int c = 0; c < nv.second.ncomp; ++c)
                    {
                        snprintf(buf, sizeof(buf), "%.17g", nv.second.values[i * nv.second.ncomp + c]);
                        out << (c ? ", " : "") << buf;
                    }
                    out << "\"";
                }
                out << " />\n";
            }
            out << "    </body>\n";
        }
        out << "</restart_data>\n";
    }
    // Loads every body of the file (same particle counts) and sets the physical time to
    // the restart time; cell lists and relations are rebuilt by the driver afterwards.
    Real readRestartFiles(size_t step)
    {
        std::ifstream in(path(step));
        if (!in)
            throw SphxException(SPHX_ERR_NOT_FOUND, "restart file " + path(step) + " is missing");
        std::stringstream ss;
        ss << in.rdbuf();
        const std::string text = ss.str();
        auto attribute = [](const std::string &tag, const std::string &name, std::string &value) {
            size_t p = tag.find(" " + name + "=\"");
            if (p == std::string::npos)
                return false;
            p += name.size() + 3;
            value = tag.substr(p, tag.find('"', p) - p);
            return true;
        };
        size_t root = text.find("<restart_data");
        std::string value;
        if (root == std::string::npos || !attribute(text.substr(root, text.find('>', root) - root), "restart_time", value))
            throw SphxException(SPHX_ERR_INVALID_ARG, "restart file " + path(step) + " has no restart_time");
        Real restart_time = std::stod(value);
        for (SPHBody *b : sys_.bodies_)
        {
            size_t pos = text.find("<body name=\"" + b->name_ + "\"");
            if (pos == std::string::npos || dynamic_cast<RealBody *>(b) == nullptr)
                continue;
            size_t end = text.find("</body>", pos);
            std::vector<std::string> names;
            std::vector<std::vector<double>> columns;
            std::vector<int> ncomp;
            size_t count = 0;
            for (size_t q = text.find("<particle", pos); q != std::string::npos && q < end;
                 q = text.find("<particle", q + 1))
            {
                std::string tag = text.substr(q, text.find("/>", q) - q);
                if (count == 0) // the attribute names of the first particle
                    for (size_t a = tag.find(' '); a != std::string::npos; a = tag.find(' ', tag.find('"', tag.find('"', a) + 1)))
                    {
                        size_t eq = tag.find('=', a);
                        if (eq == std::string::npos)
                            break;
                        names.push_back(tag.substr(a + 1, eq - a - 1));
                    }
                if (count == 0)
                {
                    columns.assign(names.size(), {});
                    ncomp.assign(names.size(), 0);
                }
                for (size_t k = 0; k < names.size(); ++k)
                {
                    if (!attribute(tag, names[k], value))
                        throw SphxException(SPHX_ERR_INVALID_ARG, "restart particle without " + names[k]);
                    std::stringstream vs(value);
                    std::string item;
                    int c = 0;
                    while (std::getline(vs, item, ','))
                    {
                        columns[k].push_back(std::stod(item));
                        ++c;
                    }
                    ncomp[k] = c;
                }
                ++count;
            }
            if (count != b->n_)
                throw SphxException(SPHX_ERR_INVALID_ARG, "restart body " + b->name_ + ": " + std::to_string(count) +
                                                              " particles for " + std::to_string(b->n_));
            for (size_t k = 0; k < names.size(); ++k)
                check(sphx_body_upload(b->body_, names[k].c_str(), SPHX_F64, ncomp[k], columns[k].data(), b->n_));
        }
        sys_.physical_time_ = restart_time;
        return restart_time;
    }
};

// ------------------------------------------------------------------ regression tests
// The dynamic-time-warping distance of two series (dynamic_time_warping_method.hpp:17-55):
// the local-distance table starts at zero, the band is +/- max(5, length difference), and
// cells outside the band keep their zero.
inline Real dtwDistance(const std::vector<Real> &a, const std::vector<Real> &b)
{
    const int la = int(a.size()), lb = int(b.size());
    if (la == 0 || lb == 0 || lb > 1.2 * la || lb < 0.8 * la)
        throw SphxException(SPHX_ERR_INVALID_ARG, "regression series lengths differ by more than 20 %");
    std::vector<std::vector<Real>> d(la, std::vector<Real>(lb, 0.0));
    d[0][0] = std::fabs(a[0] - b[0]);
    for (int i = 1; i < la; ++i)
        d[i][0] = d[i - 1][0] + std::fabs(a[i] - b[0]);
    for (int j = 1; j < lb; ++j)
        d[0][j] = d[0][j - 1] + std::fabs(a[0] - b[j]);
    const int window = std::max(5, std::abs(la - lb));
    for (int i = 1; i < la; ++i)
        for (int j = std::max(1, i - window); j < std::min(lb, i + window); ++j)
            d[i][j] = std::fabs(a[i] - b[j]) + std::min(d[i - 1][j], std::min(d[i][j - 1], d[i - 1][j - 1]));
    return d[la - 1][lb - 1];
}

namespace regression_io
{
inline std::vector<Real> numberedAttributes(const std::string &tag, const std::string &prefix)
{
    std::vector<Real> out;
    for (size_t k = 0;; ++k)
    {
        std::string key = " " + prefix + std::to_string(k) + "=\"";
        size_t p = tag.find(key);
        if (p == std::string::npos)
            return out;
        p += key.size();
        out.push_back(std::stod(tag.substr(p, tag.find('"', p) - p)));
    }
}
inline bool readFile(const std::string &path, std::string &text)
{
    std::ifstream in(path);
    if (!in)
        return false;
    std::stringstream ss;
    ss << in.rdbuf();
    text = ss.str();
    return true;
}
} // namespace regression_io

// The test of RegressionTestDynamicTimeWarping::testResult (dynamic_time_warping_method.h:
// 105-125, .hpp:73-87 and 164-190) for a series of snapshots [output][observation]: reads
// <input>/<identifier>_<quantity>_runtimes.dat (converged flag, number of runs), the stored
// maximum distances of _dtwdistance.xml (attributes <quantity>_<k>) and every stored
// _Run_<n>_result.xml (elements Particle_<k> with attributes snapshot_<s>); a run fails
// when dtw(stored, current) exceeds 1.01 times the stored maximum.  Returns false, after
// the reference's messages, when a file is missing or a distance is beyond the limit.
inline bool testDTWRegression(const std::string &input_folder, const std::string &identifier,
                              const std::string &quantity, const std::vector<std::vector<Real>> &snapshots)
{
    using namespace regression_io;
    const std::string base = input_folder + "/" + identifier + "_" + quantity;
    std::string text;
    if (!readFile(base + "_runtimes.dat", text))
    {
        printf("Error: %s_runtimes.dat is missing for regression test!\n", base.c_str());
        return false;
    }
    std::stringstream rs(text);
    std::string converged;
    int number_of_run = 0;
    rs >> converged >> number_of_run;
    const size_t observations = snapshots.empty() ? 0 : snapshots[0].size();
    std::vector<Real> stored_max(observations, 0.0);
    if (number_of_run > 1)
    {
        if (!readFile(base + "_dtwdistance.xml", text))
        {
            printf("Error: %s_dtwdistance.xml is missing for regression test!\n", base.c_str());
            return false;
        }
        std::vector<Real> d = numberedAttributes(text, quantity + "_");
        for (size_t k = 0; k < observations && k < d.size(); ++k)
            stored_max[k] = d[k];
    }
    for (int run = 0; run < number_of_run; ++run)
    {
        if (!readFile(base + "_Run_" + std::to_string(run) + "_result.xml", text))
            continue; // not preserved, not compared
        for (size_t k = 0; k < observations; ++k)
        {
            size_t p = text.find("<Particle_" + std::to_string(k) + " ");
            if (p == std::string::npos)
            {
                printf("Error: stored run %d of %s has no observation %zu\n", run, quantity.c_str(), k);
                return false;
            }
            std::vector<Real> stored = numberedAttributes(text.substr(p, text.find("/>", p) - p), "snapshot_");
            std::vector<Real> current(snapshots.size());
            for (size_t s = 0; s < snapshots.size(); ++s)
                current[s] = snapshots[s][k];
            Real distance = dtwDistance(stored, current);
            printf("DTW distance of %s[%zu] to stored run %d: %.17g (stored maximum %.17g)\n", quantity.c_str(), k,
                   run, distance, stored_max[k]);
            if (distance > 1.01 * stored_max[k])
            {
                printf("The maximum distance of %s[%zu] is %.17g, and the current distance is %.17g.\n",
                       quantity.c_str(), k, stored_max[k], distance);
                printf("The DTW distance of %s between current result and this previous local result is beyond "
                       "exception!\n",
                       quantity.c_str());
                return false;
            }
        }
    }
    printf("The result of %s is correct based on the dynamic time warping regression test!\n", quantity.c_str());
    return true;
}

// A recorded quantity (one value per observation point and output): writeToFile(iteration)
// records it and appends a line to <output>/<identifier>_<quantity>.dat; testResult() runs
// testDTWRegression on the series and exits with status 1 on failure, as the reference does.
class RegressionSeriesDTW
{
  protected:
    SPHSystem &sys_;
    std::string identifier_, quantity_;
    std::vector<std::vector<Real>> snapshots_; // [output][observation]

    void record(const std::vector<Real> &values)
    {
        makeFolder(sys_.output_folder_);
        const std::string path = sys_.output_folder_ + "/" + identifier_ + "_" + quantity_ + ".dat";
        std::ofstream out(path, snapshots_.empty() ? std::ios::trunc : std::ios::app);
        char buf[64];
        if (snapshots_.empty())
        {
            out << "run_time";
            for (size_t k = 0; k < values.size(); ++k)
                out << "   " << quantity_ << "[" << k << "]";
            out << "\n";
        }
        snprintf(buf, sizeof(buf), "%.9f", sys_.physical_time_);
        out << buf;
        for (Real v : values)
        {
            snprintf(buf, sizeof(buf), "%.17g", v);
            out << "   " << buf;
        }
        out << "\n";
        snapshots_.push_back(values);
    }

  public:
    RegressionSeriesDTW(SPHSystem &sys, const std::string &identifier, const std::string &quantity)
        : sys_(sys), identifier_(identifier), quantity_(quantity) {}
    const std::vector<std::vector<Real>> &snapshots() const { return snapshots_; }
    void testResult()
    {
        if (!testDTWRegression(sys_.input_folder_, identifier_, quantity_, snapshots_))
            exit(1);
    }
    // Building or extending the stored database is left to the reference build.
    void generateDataBase(Real, const std::string & = "false")
    {
        throw SphxException(SPHX_ERR_INVALID_ARG, "generating regression databases is not supported by this policy");
    }
};

// addReduceRegression<RegressionTestDynamicTimeWarping, TotalMechanicalEnergyCK>(body, gravity)
class ReducedQuantityRegressionCK : public RegressionSeriesDTW
{
    TotalMechanicalEnergy energy_;

  public:
    ReducedQuantityRegressionCK(SPHBody &body, const Gravity &g)
        : RegressionSeriesDTW(body.system_, body.name_, "TotalMechanicalEnergy"), energy_(body, g) {}
    void writeToFile(size_t = 0) { record({energy_.exec()}); }
};

// addObserveRegression<RegressionTestDynamicTimeWarping, Real>(observer contact, name)
class ObservedQuantityRegressionCK : public RegressionSeriesDTW
{
    ObservedQuantityCK observe_;

  public:
    ObservedQuantityRegressionCK(ContactRelation &contact, const std::string &name)
        : RegressionSeriesDTW(contact.getSPHBody().system_, contact.getSPHBody().name_, name), observe_(name, contact) {}
    void writeToFile(size_t = 0) { record(observe_.exec()); }
};

// The regression recorders of the classic drivers (tests/3d_examples/test_3d_dambreak/
// dambreak.cpp:86-87): RegressionTestDynamicTimeWarping<ReducedQuantityRecording<
// TotalMechanicalEnergy>>(body, gravity) and RegressionTestDynamicTimeWarping<
// ObservedQuantityRecording<Real>>(name, observer contact), with the state recorder's
// classic name.
template <class ReduceType>
class ReducedQuantityRecording
{
};
template <class DataType>
class ObservedQuantityRecording
{
};
template <>
class RegressionTestDynamicTimeWarping<ReducedQuantityRecording<TotalMechanicalEnergy>> : public RegressionSeriesDTW
{
    TotalMechanicalEnergy energy_;

  public:
    RegressionTestDynamicTimeWarping(SPHBody &body, const Gravity &g)
        : RegressionSeriesDTW(body.system_, body.name_, "TotalMechanicalEnergy"), energy_(body, g) {}
    void writeToFile(size_t = 0) { record({energy_.exec()}); }
};
template <>
class RegressionTestDynamicTimeWarping<ObservedQuantityRecording<Real>> : public RegressionSeriesDTW
{
    ObservedQuantity observe_;

  public:
    RegressionTestDynamicTimeWarping(const std::string &name, ContactRelation &contact)
        : RegressionSeriesDTW(contact.getSPHBody().system_, contact.getSPHBody().name_, name),
          observe_(name, contact) {}
    void writeToFile(size_t = 0) { record(observe_.exec()); }
};
class BodyStatesRecordingToVtp : public BodyStatesRecordingToVtpCK<>
{
  public:
    using BodyStatesRecordingToVtpCK<>::BodyStatesRecordingToVtpCK;
};

// ------------------------------------------------------------------ containers
class BaseMethodContainer
{
  protected:
    std::vector<std::shared_ptr<void>> kept_;
    template <class T, typename... Args>
    T &keep(Args &&...args)
    {
        auto p = std::make_shared<T>(std::forward<Args>(args)...);
        kept_.push_back(p);
        return *p;
    }

  public:
    virtual ~BaseMethodContainer() = default;
};

template <class ExecutionPolicy>
class ParticleMethodContainer : public BaseMethodContainer
{
  public:
    explicit ParticleMethodContainer(const ExecutionPolicy &) {}

    auto &addCellLinkedListDynamics(RealBody &body) { return keep<UpdateCellLinkedList<ExecutionPolicy, RealBody>>(body); }
    template <class FirstRelation, typename... OtherRelations>
    auto &addRelationDynamics(FirstRelation &first, OtherRelations &...others)
    {
        return keep<UpdateRelation<ExecutionPolicy, FirstRelation, OtherRelations...>>(first, others...);
    }
    auto &addSortDynamics(RealBody &body) { return keep<ParticleSortCK<ExecutionPolicy>>(body); }
    template <class UpdateType, typename... Args>
    auto &addStateDynamics(SPHBody &body, Args &&...args)
    {
        return keep<StateDynamics<ExecutionPolicy, UpdateType>>(body, std::forward<Args>(args)...);
    }
    template <class ReduceType, typename... Args>
    auto &addReduceDynamics(SPHBody &body, Args &&...args)
    {
        return keep<ReduceDynamicsCK<ExecutionPolicy, ReduceType>>(body, std::forward<Args>(args)...);
    }
    template <template <typename...> class InteractionType, typename... ControlParameters, typename... Args>
    auto &addInteractionDynamics(InnerRelation &inner, Args &&...args)
    {
        return keep<InteractionGroupCK<ExecutionPolicy, InteractionType>>(inner, std::forward<Args>(args)...);
    }
    template <template <typename...> class RecorderType>
    auto &addBodyStateRecorder(SPHSystem &sys)
    {
        return keep<RecorderType<>>(sys);
    }
    template <template <typename...> class IOType>
    auto &addIODynamics(SPHSystem &sys)
    {
        return keep<IOType<>>(sys);
    }
    template <template <typename...> class RegressionType, template <typename...> class LocalReduceMethodType>
    auto &addReduceRegression(SPHBody &body, const Gravity &g)
    {
        static_assert(IsSameTemplate<RegressionType, RegressionTestDynamicTimeWarping>::value &&
                          IsSameTemplate<LocalReduceMethodType, TotalMechanicalEnergyCK>::value,
                      "reduce regression: dynamic time warping of the total mechanical energy");
        return keep<ReducedQuantityRegressionCK>(body, g);
    }
    template <template <typename...> class RegressionType, typename VariableType>
    auto &addObserveRegression(ContactRelation &contact, const std::string &name)
    {
        static_assert(IsSameTemplate<RegressionType, RegressionTestDynamicTimeWarping>::value &&
                          std::is_same<VariableType, Real>::value,
                      "observe regression: dynamic time warping of a Real quantity");
        return keep<ObservedQuantityRegressionCK>(contact, name);
    }
};

// TimeStepper (sph_solver.cpp:40-190): the physical time, the global time-step size and
// the interval triggers, each advanced by incrementPhysicalTime.
class TimeStepper
{
  public:
    class TriggerByInterval
    {
        Real present_time_ = 0.0, interval_;

      public:
        explicit TriggerByInterval(Real initial_interval) : interval_(initial_interval) {}
        // fires once the time since it last fired exceeds the interval, then takes the next
        // interval from the evaluator (sph_solver.cpp:53-62)
        bool operator()(BaseDynamics<Real> &interval_evaluator)
        {
            if (present_time_ > interval_)
            {
                present_time_ = 0.0;
                interval_ = interval_evaluator.exec();
                return true;
            }
            return false;
        }
        bool operator()()
        {
            if (present_time_ > interval_)
            {
                present_time_ = 0.0;
                return true;
            }
            return false;
        }
        Real getInterval() const { return interval_; }
        void incrementPresentTime(Real dt) { present_time_ += dt; }
    };
    class TriggerByPhysicalTime
    {
        SPHSystem &sys_;
        Real trigger_time_;

      public:
        TriggerByPhysicalTime(SPHSystem &sys, Real trigger_time) : sys_(sys), trigger_time_(trigger_time) {}
        bool operator()() { return sys_.physical_time_ > trigger_time_; }
    };

    explicit TimeStepper(SPHSystem &sys) : sys_(sys) {}
    TriggerByInterval &addTriggerByInterval(Real initial_interval)
    {
        intervals_.push_back(std::make_unique<TriggerByInterval>(initial_interval));
        return *intervals_.back();
    }
    TriggerByPhysicalTime &addTriggerByPhysicalTime(Real trigger_time)
    {
        physical_times_.push_back(std::make_unique<TriggerByPhysicalTime>(sys_, trigger_time));
        return *physical_times_.back();
    }
    Real incrementPhysicalTime(Real dt)
    {
        global_dt_ = dt;
        sys_.physical_time_ += dt;
        for (auto &t : intervals_)
            t->incrementPresentTime(dt);
        return dt;
    }
    Real incrementPhysicalTime(BaseDynamics<Real> &step_evaluator) { return incrementPhysicalTime(step_evaluator.exec()); }
    bool isEndTime(Real end_time) const { return sys_.physical_time_ >= end_time; }
    void setPhysicalTime(Real t) { sys_.physical_time_ = t; }
    Real getPhysicalTime() const { return sys_.physical_time_; }
    Real getGlobalTimeStepSize() const { return global_dt_; }

  private:
    SPHSystem &sys_;
    Real global_dt_ = 0.0;
    std::vector<std::unique_ptr<TriggerByInterval>> intervals_;
    std::vector<std::unique_ptr<TriggerByPhysicalTime>> physical_times_;
};

class SPHSolver
{
    SPHSystem &sys_;
    TimeStepper time_stepper_;
    std::vector<std::unique_ptr<BaseMethodContainer>> containers_;

  public:
    explicit SPHSolver(SPHSystem &sys) : sys_(sys), time_stepper_(sys) {}
    template <typename ExecutionPolicy>
    auto &addParticleMethodContainer(const ExecutionPolicy &policy)
    {
        auto c = std::make_unique<ParticleMethodContainer<ExecutionPolicy>>(policy);
        auto &ref = *c;
        containers_.push_back(std::move(c));
        return ref;
    }
    TimeStepper &getTimeStepper() { return time_stepper_; }
};
} // namespace SPH
