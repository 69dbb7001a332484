// Weakly-compressible fluid dynamics on the device (FP64 drop-in of the classic path).
//
// Reference (src/shared/particle_dynamics/fluid_dynamics/):
//   DensitySummationComplexFreeSurface   density_summation.cpp:74-82,124-144, .hpp:28-32
//   Integration1stHalfWithWallRiemann    fluid_integration.hpp:49-113
//   Integration2ndHalfWithWallRiemann    fluid_integration.hpp:166-231
//   AcousticTimeStep / AdvectionTimeStep fluid_time_step.cpp:21-31,54-65
//   AcousticRiemannSolver                src/shared/materials/riemann_solver.h:55-124
//   WeaklyCompressibleFluid EOS          src/shared/materials/weakly_compressible_fluid.cpp:17-20
//
// Fusion: Dynamics1Level runs initialization, interaction and update as three passes
// (dynamics_algorithms.h:336-352).  Here the 1st half is two launches (density/pressure
// initialisation, then interaction + wall contact + velocity update + the position
// half-step) and the 2nd half is one launch (position half-step + interaction + wall
// contact + density update): every fused update only touches the particle's own
// variables, which no other particle reads in that interaction.
#include <algorithm>

#include "sphx_device.cuh"
#include "sphx_internal.cuh"

using namespace sphx;

namespace
{
constexpr unsigned kBlock = 128;

// Acoustic Riemann solver constants for a fluid interacting with itself or a wall.
struct Riemann
{
    double inv_rho0c0_ave, rho0c0_geo_ave, inv_c0_ave, slope;
};

Riemann make_riemann(const sphx_fluid_params &p)
{
    double Z = p.rho0 * p.c0;
    double inv_sum = 1.0 / (Z + Z);
    Riemann r;
    r.inv_rho0c0_ave = (Z + Z) / (Z * Z + Z * Z);
    r.rho0c0_geo_ave = 2.0 * Z * Z * inv_sum;
    r.inv_c0_ave = 0.5 * (p.rho0 + p.rho0) * r.inv_rho0c0_ave;
    r.slope = p.limiter_slope;
    return r;
}

__device__ __forceinline__ double dissipative_p_jump(const Riemann &rs, double u)
{
    return rs.rho0c0_geo_ave * u * fmin(rs.slope * (rs.inv_c0_ave * fmax(u, 0.0)), 1.0);
}

struct Neighbors
{
    const uint32_t *count, *J;
    const double *DW, *E, *R;
    size_t stride; // cap * n_src
    unsigned cap;  // slots per particle; loops never read past it
    uint32_t limit; // target particles the entries index (tested by the checked build)
};

// Entry j indexes a target particle (always true unless built with SPHX_CHECK).
__device__ __forceinline__ bool entry_ok(const Neighbors &nb, uint32_t j)
{
    return SPHX_CHECKED(j < nb.limit, kCheckListEntry, j);
}

Neighbors neighbors_of(sphx_relation r)
{
    Neighbors nb;
    nb.count = r->count;
    nb.J = r->j;
    nb.DW = r->dW;
    nb.E = r->e;
    nb.R = r->r;
    nb.stride = size_t(r->cap) * r->n_src;
    nb.cap = unsigned(r->cap);
    nb.limit = uint32_t(r->tgt ? r->tgt->n : 0);
    return nb;
}

struct FluidVars
{
    double *pos, *vel, *force;
    const double *force_prior;
    double *rho, *p, *drho_dt;
    const double *mass, *Vol;
    double *rho_sum;
};

struct WallVars
{
    const double *Vol, *acc, *vel_ave, *n;
    size_t n_wall;
};

// ---------------------------------------------------------------- density summation
__global__ void k_density_summation(size_t n, const double *__restrict__ sigma_inner,
                                    const double *__restrict__ sigma_wall, const double *__restrict__ mass,
                                    double rho0, double inv_sigma0, double *__restrict__ rho_sum,
                                    double *__restrict__ rho, int free_surface)
{
    size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    double rs = sigma_inner[i] * rho0 * inv_sigma0;
    if (sigma_wall)
        rs += sigma_wall[i] * rho0 * rho0 * inv_sigma0 / mass[i];
    rho_sum[i] = rs;
    // FreeSurface update SMAX(rho_sum, rho0) or the plain update rho = rho_sum; Vol unchanged
    rho[i] = free_surface ? fmax(rs, rho0) : rs;
}

// ---------------------------------------------------------------- 1st half
__global__ void k_init_1st(size_t n, double *__restrict__ rho, const double *__restrict__ drho_dt,
                           double *__restrict__ p, double p0, double rho0, double dt)
{
    size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    double r = rho[i] + drho_dt[i] * dt * 0.5;
    rho[i] = r;
    p[i] = p0 * (r / rho0 - 1.0);
}

template <int D>
__global__ void __launch_bounds__(kBlock)
    k_interact_1st(size_t n, FluidVars f, Neighbors in, Neighbors wn, WallVars w, Riemann rs, double dt)
{
    size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    const double p_i = f.p[i], rho_i = f.rho[i], Vol_i = f.Vol[i], m_i = f.mass[i];
    double force[3] = {0, 0, 0};
    double rho_dissipation = 0;
    const unsigned cnt = min(in.count[i], in.cap);
    for (unsigned s = 0; s < cnt; ++s)
    {
        size_t slot = size_t(s) * n + i;
        uint32_t j = in.J[slot];
        if (!entry_ok(in, j))
            continue;
        double dWV = in.DW[slot] * f.Vol[j];
        double p_j = f.p[j];
        double sc = (p_i + p_j) * dWV;
#pragma unroll
        for (int d = 0; d < D; ++d)
            force[d] -= sc * in.E[d * in.stride + slot];
        rho_dissipation += ((p_i - p_j) * rs.inv_rho0c0_ave) * dWV;
    }
    double F[3];
#pragma unroll
    for (int d = 0; d < D; ++d)
        F[d] = f.force[d * n + i] + force[d] * Vol_i;
    double drho = rho_dissipation * rho_i;
    if (wn.count)
    {
        double fp_m[3];
#pragma unroll
        for (int d = 0; d < D; ++d)
            fp_m[d] = f.force_prior[d * n + i] / m_i;
        double wforce[3] = {0, 0, 0};
        double wrho = 0;
        const unsigned wc = min(wn.count[i], wn.cap);
        for (unsigned s = 0; s < wc; ++s)
        {
            size_t slot = size_t(s) * n + i;
            uint32_t j = wn.J[slot];
            if (!entry_ok(wn, j))
                continue;
            double dWV = wn.DW[slot] * w.Vol[j];
            double r_ij = wn.R[slot];
            double e[3];
            double face = 0;
#pragma unroll
            for (int d = 0; d < D; ++d)
            {
                e[d] = wn.E[d * wn.stride + slot];
                face += (fp_m[d] - w.acc[d * w.n_wall + j]) * (-e[d]);
            }
            double p_j_in_wall = p_i + rho_i * r_ij * fmax(0.0, face);
            double sc = (p_i + p_j_in_wall) * dWV;
#pragma unroll
            for (int d = 0; d < D; ++d)
                wforce[d] -= sc * e[d];
            wrho += ((p_i - p_j_in_wall) * rs.inv_rho0c0_ave) * dWV;
        }
#pragma unroll
        for (int d = 0; d < D; ++d)
            F[d] += wforce[d] * Vol_i;
        drho += wrho * rho_i;
    }
    f.drho_dt[i] = drho;
#pragma unroll
    for (int d = 0; d < D; ++d)
    {
        f.force[d * n + i] = F[d];
        double v = f.vel[d * n + i];
        f.pos[d * n + i] += v * dt * 0.5; // initialization: x += v dt/2 with the old velocity
        f.vel[d * n + i] = v + (f.force_prior[d * n + i] + F[d]) / m_i * dt;
    }
}

// ---------------------------------------------------------------- 2nd half
template <int D>
__global__ void __launch_bounds__(kBlock)
    k_interact_2nd(size_t n, FluidVars f, Neighbors in, Neighbors wn, WallVars w, Riemann rs, double dt)
{
    size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    double v_i[3] = {0, 0, 0};
#pragma unroll
    for (int d = 0; d < D; ++d)
        v_i[d] = f.vel[d * n + i];
    const double rho_i = f.rho[i], Vol_i = f.Vol[i];
    double density_change_rate = 0;
    double p_dissipation[3] = {0, 0, 0};
    const unsigned cnt = min(in.count[i], in.cap);
    for (unsigned s = 0; s < cnt; ++s)
    {
        size_t slot = size_t(s) * n + i;
        uint32_t j = in.J[slot];
        if (!entry_ok(in, j))
            continue;
        double dWV = in.DW[slot] * f.Vol[j];
        double e[3];
        double u_jump = 0;
#pragma unroll
        for (int d = 0; d < D; ++d)
        {
            e[d] = in.E[d * in.stride + slot];
            u_jump += (v_i[d] - f.vel[d * n + j]) * e[d];
        }
        density_change_rate += u_jump * dWV;
        double sc = dissipative_p_jump(rs, u_jump) * dWV;
#pragma unroll
        for (int d = 0; d < D; ++d)
            p_dissipation[d] += sc * e[d];
    }
    double drho = f.drho_dt[i] + density_change_rate * rho_i;
    double F[3];
#pragma unroll
    for (int d = 0; d < D; ++d)
        F[d] = p_dissipation[d] * Vol_i;
    if (wn.count)
    {
        double wrate = 0;
        double wdiss[3] = {0, 0, 0};
        const unsigned wc = min(wn.count[i], wn.cap);
        for (unsigned s = 0; s < wc; ++s)
        {
            size_t slot = size_t(s) * n + i;
            uint32_t j = wn.J[slot];
            if (!entry_ok(wn, j))
                continue;
            double dWV = wn.DW[slot] * w.Vol[j];
            double e[3], nj[3], va[3];
            double en = 0;
#pragma unroll
            for (int d = 0; d < D; ++d)
            {
                e[d] = wn.E[d * wn.stride + slot];
                nj[d] = w.n[d * w.n_wall + j];
                va[d] = w.vel_ave[d * w.n_wall + j];
                en += e[d] * nj[d];
            }
            double sgn = en < 0.0 ? -1.0 : (en > 0.0 ? 1.0 : 0.0);
            double dv_e = 0, dv_n = 0;
#pragma unroll
            for (int d = 0; d < D; ++d)
            {
                double n_star = sgn * nj[d];
                double vin_wall = 2.0 * va[d] - v_i[d];
                dv_e += (v_i[d] - vin_wall) * e[d];
                dv_n += (v_i[d] - va[d]) * n_star;
            }
            wrate += dv_e * dWV;
            double u_jump = 2.0 * dv_n;
            double sc = dissipative_p_jump(rs, u_jump) * dWV;
#pragma unroll
            for (int d = 0; d < D; ++d)
                wdiss[d] += sc * (sgn * nj[d]);
        }
        drho += wrate * rho_i;
#pragma unroll
        for (int d = 0; d < D; ++d)
            F[d] += wdiss[d] * Vol_i;
    }
    f.drho_dt[i] = drho;
    f.rho[i] = rho_i + drho * dt * 0.5;
#pragma unroll
    for (int d = 0; d < D; ++d)
    {
        f.force[d * n + i] = F[d];
        f.pos[d * n + i] += v_i[d] * dt * 0.5; // initialization of the 2nd half
    }
}

// ---------------------------------------------------------------- reductions
// Max reductions write the order-preserving bits of non-negative doubles; the warp and
// block maxima are exact, so the result does not depend on the launch order.
__device__ __forceinline__ void block_max_to(unsigned long long *slot, double v)
{
    unsigned long long b = ordered_bits(v);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
    {
        unsigned long long y = __shfl_down_sync(0xffffffffu, b, o);
        b = y > b ? y : b;
    }
    __shared__ unsigned long long sm[32];
    unsigned lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    if (lane == 0)
        sm[warp] = b;
    __syncthreads();
    if (warp == 0)
    {
        b = lane < (blockDim.x >> 5) ? sm[lane] : 0ull;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1)
        {
            unsigned long long y = __shfl_down_sync(0xffffffffu, b, o);
            b = y > b ? y : b;
        }
        if (lane == 0)
            atomicMax(slot, b);
    }
}

template <int D>
__global__ void k_acoustic_max(size_t n, const double *__restrict__ vel, double c0, unsigned long long *slot)
{
    double m = -1.0e300;
    for (size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += size_t(gridDim.x) * blockDim.x)
    {
        double s = vel[i] * vel[i] + vel[n + i] * vel[n + i];
        if (D == 3)
            s = s + vel[2 * n + i] * vel[2 * n + i];
        m = fmax(m, c0 + sqrt(s));
    }
    block_max_to(slot, m);
}

template <int D>
__global__ void k_advection_max(size_t n, const double *__restrict__ vel, const double *__restrict__ force,
                                const double *__restrict__ fprior, const double *__restrict__ mass, double h_min,
                                unsigned long long *slot)
{
    double m = -1.0e300;
    for (size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += size_t(gridDim.x) * blockDim.x)
    {
        double v2 = 0, f2 = 0;
#pragma unroll
        for (int d = 0; d < D; ++d)
        {
            double v = vel[d * n + i];
            double ft = force[d * n + i] + fprior[d * n + i];
            v2 += v * v;
            f2 += ft * ft;
        }
        double acc = 4.0 * h_min * sqrt(f2) / mass[i];
        m = fmax(m, fmax(v2, acc));
    }
    block_max_to(slot, m);
}

__global__ void k_gravity(size_t n, int dim, const double *__restrict__ mass, double g0, double g1, double g2,
                          double *__restrict__ fprior, double *__restrict__ prev)
{
    size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    double g[3] = {g0, g1, g2};
    for (int d = 0; d < dim; ++d)
    {
        double cur = mass[i] * g[d];
        fprior[d * n + i] += cur - prev[d * n + i];
        prev[d * n + i] = cur;
    }
}

// Interpolation at observer points: one warp per observer, fixed-order combine.
__global__ void k_observe(size_t n_obs, size_t n_tgt, unsigned cap, const uint32_t *__restrict__ count, const uint32_t *__restrict__ J,
                          const double *__restrict__ W, const double *__restrict__ Vol, const double *__restrict__ q,
                          double *__restrict__ out)
{
    size_t i = blockIdx.x;
    if (i >= n_obs || threadIdx.x != 0)
        return;
    double num = 0, ttl = 0;
    const unsigned cnt = min(count[i], cap);
    for (unsigned s = 0; s < cnt; ++s)
    {
        size_t slot = size_t(s) * n_obs + i;
        const uint32_t j = J[slot];
        if (!SPHX_CHECKED(j < n_tgt, kCheckListEntry, j))
            continue;
        double w = W[slot] * Vol[j];
        num += w * q[j];
        ttl += w;
    }
    out[i] = num / (ttl + kTinyReal);
}

// Deterministic block partial sums of the mechanical energy.
template <int D>
__global__ void k_energy_partials(size_t n, const double *__restrict__ pos, const double *__restrict__ vel,
                                  const double *__restrict__ mass, double g0, double g1, double g2,
                                  double *__restrict__ partials)
{
    double g[3] = {g0, g1, g2};
    double s = 0;
    for (size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += size_t(gridDim.x) * blockDim.x)
    {
        double v2 = 0, gx = 0;
#pragma unroll
        for (int d = 0; d < D; ++d)
        {
            double v = vel[d * n + i];
            v2 += v * v;
            gx += g[d] * (-pos[d * n + i]);
        }
        s += 0.5 * mass[i] * v2 + mass[i] * gx;
    }
    __shared__ double sm[kBlock];
    sm[threadIdx.x] = s;
    __syncthreads();
    for (unsigned o = blockDim.x / 2; o > 0; o >>= 1)
    {
        if (threadIdx.x < o)
            sm[threadIdx.x] += sm[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0)
        partials[blockIdx.x] = sm[0];
}

__global__ void k_sum_partials(unsigned np, const double *__restrict__ partials, double *__restrict__ out)
{
    if (threadIdx.x == 0 && blockIdx.x == 0)
    {
        double s = 0;
        for (unsigned k = 0; k < np; ++k)
            s += partials[k];
        *out = s;
    }
}

template <int D>
__global__ void k_upper_front(size_t n, const double *__restrict__ pos, int axis, double l0, double l1, double l2,
                              double u0, double u1, double u2, unsigned long long *slot)
{
    double lo[3] = {l0, l1, l2}, up[3] = {u0, u1, u2};
    double m = -1.0e300;
    for (size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += size_t(gridDim.x) * blockDim.x)
    {
        bool in = true;
#pragma unroll
        for (int d = 0; d < D; ++d)
        {
            double x = pos[d * n + i];
            in = in && !(x < lo[d] || x > up[d]);
        }
        if (in)
            m = fmax(m, pos[axis * n + i]);
    }
    block_max_to(slot, m);
}

int fluid_vars(sphx_body b, FluidVars &f)
{
    Field *pos, *vel, *force, *fp, *rho, *p, *drho, *mass, *Vol, *rs;
    int D = b->dim;
    SPHX_TRY(b->need("Position", SPHX_F64, D, &pos));
    SPHX_TRY(b->require("Velocity", SPHX_F64, D, &vel));
    SPHX_TRY(b->require("Force", SPHX_F64, D, &force));
    SPHX_TRY(b->require("ForcePrior", SPHX_F64, D, &fp));
    SPHX_TRY(b->need("Density", SPHX_F64, 1, &rho));
    SPHX_TRY(b->require("Pressure", SPHX_F64, 1, &p));
    SPHX_TRY(b->require("DensityChangeRate", SPHX_F64, 1, &drho));
    SPHX_TRY(b->need("Mass", SPHX_F64, 1, &mass));
    SPHX_TRY(b->need("VolumetricMeasure", SPHX_F64, 1, &Vol));
    SPHX_TRY(b->require("DensitySummation", SPHX_F64, 1, &rs));
    f.pos = static_cast<double *>(pos->dev);
    f.vel = static_cast<double *>(vel->dev);
    f.force = static_cast<double *>(force->dev);
    f.force_prior = static_cast<const double *>(fp->dev);
    f.rho = static_cast<double *>(rho->dev);
    f.p = static_cast<double *>(p->dev);
    f.drho_dt = static_cast<double *>(drho->dev);
    f.mass = static_cast<const double *>(mass->dev);
    f.Vol = static_cast<const double *>(Vol->dev);
    f.rho_sum = static_cast<double *>(rs->dev);
    return SPHX_OK;
}

int wall_vars(sphx_body w, WallVars &v)
{
    Field *Vol, *acc, *vel, *n;
    int D = w->dim;
    SPHX_TRY(w->need("VolumetricMeasure", SPHX_F64, 1, &Vol));
    SPHX_TRY(w->require("Acceleration", SPHX_F64, D, &acc));
    SPHX_TRY(w->require("Velocity", SPHX_F64, D, &vel));
    SPHX_TRY(w->need("NormalDirection", SPHX_F64, D, &n));
    v.Vol = static_cast<const double *>(Vol->dev);
    v.acc = static_cast<const double *>(acc->dev);
    v.vel_ave = static_cast<const double *>(vel->dev);
    v.n = static_cast<const double *>(n->dev);
    v.n_wall = w->n;
    return SPHX_OK;
}

int check_pair(sphx_relation inner, sphx_relation wall, const sphx_fluid_params *p)
{
    if (!inner || !p || !inner->inner)
        return fail(SPHX_ERR_INVALID_ARG, "an inner relation and fluid parameters are required");
    if (wall && (wall->inner || wall->src != inner->src))
        return fail(SPHX_ERR_INVALID_ARG, "the wall relation must be a contact relation of the same fluid body");
    if (inner->n_src != inner->src->n || (wall && wall->n_src != wall->src->n))
        return fail(SPHX_ERR_INVALID_ARG, "relation not updated for the current particle count");
    if (!(p->rho0 > 0) || !(p->c0 > 0))
        return fail(SPHX_ERR_INVALID_ARG, "rho0 and c0 must be positive");
    return SPHX_OK;
}

int read_max(sphx_ctx ctx, double *out)
{
    SPHX_CUDA(cudaMemcpyAsync(ctx->h_red, ctx->d_red, sizeof(unsigned long long), cudaMemcpyDeviceToHost,
                              ctx->stream));
    SPHX_CUDA(cudaStreamSynchronize(ctx->stream));
    *out = from_ordered_bits(ctx->h_red[0]);
    return SPHX_OK;
}

// ViscousForce<Inner<>, FixedViscosity, NoKernelCorrection> (viscous_dynamics.hpp:25-53) and
// the ForcePrior update (force_prior.hpp:22-26): the configuration-time r, e, dW of the inner
// relation, e . (2 e) for the (absent) kernel correction.
template <int D>
__global__ void __launch_bounds__(kBlock) k_viscous_inner(size_t n, Neighbors in, const double *__restrict__ vel,
                                                          const double *__restrict__ Vol, double mu, double h,
                                                          double *__restrict__ viscous, double *__restrict__ prev,
                                                          double *__restrict__ force_prior)
{
    size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    double f[3] = {0, 0, 0}, vi[3] = {0, 0, 0};
#pragma unroll
    for (int a = 0; a < D; ++a)
        vi[a] = vel[a * n + i];
    const unsigned cnt = min(in.count[i], in.cap);
    for (unsigned s = 0; s < cnt; ++s)
    {
        size_t slot = size_t(s) * n + i;
        uint32_t j = in.J[slot];
        if (!entry_ok(in, j))
            continue;
        double e[3] = {0, 0, 0};
#pragma unroll
        for (int a = 0; a < D; ++a)
            e[a] = in.E[a * in.stride + slot];
        double ee = 0;
#pragma unroll
        for (int a = 0; a < D; ++a)
            ee += e[a] * (2.0 * e[a]);
        double denom = in.R[slot] + 0.01 * h;
        double dWV_factor = in.DW[slot];
#pragma unroll
        for (int a = 0; a < D; ++a)
        {
            double vd = (vi[a] - vel[a * n + j]) / denom;
            f[a] += ee * mu * vd * dWV_factor * Vol[j];
        }
    }
    const double Vol_i = Vol[i];
#pragma unroll
    for (int a = 0; a < D; ++a)
    {
        double v = f[a] * Vol_i;
        force_prior[a * n + i] += v - prev[a * n + i];
        prev[a * n + i] = v;
        viscous[a * n + i] = v;
    }
}

// TransportVelocityCorrection<Inner<SPHAdaptation, TruncatedLinear>> (transport_velocity_correction
// .hpp:32-66): kernel-gradient integral from the configuration-time dW, e, then the position
// shift with the limiter min(100 h^2 |.|^2, 1); interaction and update fused (the update
// moves only the particle's own position, which no neighbour term reads).
template <int D>
__global__ void __launch_bounds__(kBlock) k_tvc_inner(size_t n, Neighbors in, const double *__restrict__ Vol,
                                                      double h2, double scaling, double *__restrict__ pos)
{
    size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    double inc[3] = {0, 0, 0};
    const unsigned cnt = min(in.count[i], in.cap);
    for (unsigned s = 0; s < cnt; ++s)
    {
        size_t slot = size_t(s) * n + i;
        uint32_t j = in.J[slot];
        if (!entry_ok(in, j))
            continue;
        double w = (1.0 + 1.0) * in.DW[slot] * Vol[j];
#pragma unroll
        for (int a = 0; a < D; ++a)
            inc[a] -= w * in.E[a * in.stride + slot];
    }
    double sq = inc[0] * inc[0] + inc[1] * inc[1];
    if (D == 3)
        sq = sq + inc[2] * inc[2];
    double lim = fmin(100.0 * (h2 * sq), 1.0);
#pragma unroll
    for (int a = 0; a < D; ++a)
        pos[a * n + i] += scaling * lim * inc[a] * 1.0 * 1.0;
}

unsigned reduce_grid(sphx_ctx ctx, size_t n)
{
    unsigned g = grid_for(n, kBlock);
    unsigned cap = unsigned(std::max(1, ctx->num_sms)) * 8u;
    return std::max(1u, std::min(g, cap));
}
} // namespace

extern "C" int sphx_density_summation_complex_free_surface(sphx_relation inner, sphx_relation wall,
                                                           const sphx_fluid_params *p)
{
    SPHX_TRY(check_pair(inner, wall, p));
    if (!(p->sigma0 > 0))
        return fail(SPHX_ERR_INVALID_ARG, "sigma0 must be positive");
    sphx_body b = inner->src;
    FluidVars f;
    SPHX_TRY(fluid_vars(b, f));
    size_t n = b->n;
    if (n == 0)
        return SPHX_OK;
    sphx_ctx ctx = b->ctx;
    k_density_summation<<<grid_for(n, 256), 256, 0, ctx->stream>>>(n, inner->wsum, wall ? wall->wsum : nullptr,
                                                                   f.mass, p->rho0, 1.0 / p->sigma0, f.rho_sum,
                                                                   f.rho, 1);
    SPHX_LAUNCHED(ctx);
    return SPHX_OK;
}

extern "C" int sphx_integration_1st_half_with_wall_riemann(sphx_relation inner, sphx_relation wall,
                                                           const sphx_fluid_params *p, double dt)
{
    SPHX_TRY(check_pair(inner, wall, p));
    sphx_body b = inner->src;
    FluidVars f;
    SPHX_TRY(fluid_vars(b, f));
    WallVars w{};
    if (wall)
        SPHX_TRY(wall_vars(wall->tgt, w));
    size_t n = b->n;
    if (n == 0)
        return SPHX_OK;
    sphx_ctx ctx = b->ctx;
    double p0 = p->rho0 * p->c0 * p->c0;
    k_init_1st<<<grid_for(n, 256), 256, 0, ctx->stream>>>(n, f.rho, f.drho_dt, f.p, p0, p->rho0, dt);
    SPHX_LAUNCHED(ctx);
    Neighbors in = neighbors_of(inner);
    Neighbors wn{};
    if (wall)
        wn = neighbors_of(wall);
    Riemann rs = make_riemann(*p);
    if (b->dim == 2)
        k_interact_1st<2><<<grid_for(n, kBlock), kBlock, 0, ctx->stream>>>(n, f, in, wn, w, rs, dt);
    else
        k_interact_1st<3><<<grid_for(n, kBlock), kBlock, 0, ctx->stream>>>(n, f, in, wn, w, rs, dt);
    SPHX_LAUNCHED(ctx);
    return SPHX_OK;
}

extern "C" int sphx_integration_2nd_half_with_wall_riemann(sphx_relation inner, sphx_relation wall,
                                                           const sphx_fluid_params *p, double dt)
{
    SPHX_TRY(check_pair(inner, wall, p));
    sphx_body b = inner->src;
    FluidVars f;
    SPHX_TRY(fluid_vars(b, f));
    WallVars w{};
    if (wall)
        SPHX_TRY(wall_vars(wall->tgt, w));
    size_t n = b->n;
    if (n == 0)
        return SPHX_OK;
    sphx_ctx ctx = b->ctx;
    Neighbors in = neighbors_of(inner);
    Neighbors wn{};
    if (wall)
        wn = neighbors_of(wall);
    Riemann rs = make_riemann(*p);
    if (b->dim == 2)
        k_interact_2nd<2><<<grid_for(n, kBlock), kBlock, 0, ctx->stream>>>(n, f, in, wn, w, rs, dt);
    else
        k_interact_2nd<3><<<grid_for(n, kBlock), kBlock, 0, ctx->stream>>>(n, f, in, wn, w, rs, dt);
    SPHX_LAUNCHED(ctx);
    return SPHX_OK;
}

extern "C" int sphx_acoustic_time_step(sphx_body b, const sphx_fluid_params *p, double *dt)
{
    if (!b || !p || !dt)
        return fail(SPHX_ERR_INVALID_ARG, "null argument");
    Field *vel;
    SPHX_TRY(b->require("Velocity", SPHX_F64, b->dim, &vel));
    sphx_ctx ctx = b->ctx;
    size_t n = b->n;
    SPHX_CUDA(cudaMemsetAsync(ctx->d_red, 0, sizeof(unsigned long long), ctx->stream));
    if (n > 0)
    {
        unsigned g = reduce_grid(ctx, n);
        if (b->dim == 2)
            k_acoustic_max<2><<<g, kBlock, 0, ctx->stream>>>(n, static_cast<const double *>(vel->dev), p->c0,
                                                             ctx->d_red);
        else
            k_acoustic_max<3><<<g, kBlock, 0, ctx->stream>>>(n, static_cast<const double *>(vel->dev), p->c0,
                                                             ctx->d_red);
        SPHX_LAUNCHED(ctx);
    }
    double m;
    SPHX_TRY(read_max(ctx, &m));
    if (n == 0)
        m = -1.79769313486231570815e308; // ReduceMax initial value MinReal
    *dt = p->acoustic_cfl * p->h / (m + kTinyReal);
    return SPHX_OK;
}

extern "C" int sphx_advection_time_step(sphx_body b, const sphx_fluid_params *p, double *dt)
{
    if (!b || !p || !dt)
        return fail(SPHX_ERR_INVALID_ARG, "null argument");
    FluidVars f;
    SPHX_TRY(fluid_vars(b, f));
    sphx_ctx ctx = b->ctx;
    size_t n = b->n;
    SPHX_CUDA(cudaMemsetAsync(ctx->d_red, 0, sizeof(unsigned long long), ctx->stream));
    if (n > 0)
    {
        unsigned g = reduce_grid(ctx, n);
        if (b->dim == 2)
            k_advection_max<2><<<g, kBlock, 0, ctx->stream>>>(n, f.vel, f.force, f.force_prior, f.mass, p->h,
                                                              ctx->d_red);
        else
            k_advection_max<3><<<g, kBlock, 0, ctx->stream>>>(n, f.vel, f.force, f.force_prior, f.mass, p->h,
                                                              ctx->d_red);
        SPHX_LAUNCHED(ctx);
    }
    double m;
    SPHX_TRY(read_max(ctx, &m));
    double speed_max = n > 0 ? sqrt(m) : 0.0;
    *dt = p->advection_cfl * p->h / (std::max(speed_max, p->U_ref) + kTinyReal);
    return SPHX_OK;
}

extern "C" int sphx_gravity_force(sphx_body b, const double *g)
{
    if (!b || !g)
        return fail(SPHX_ERR_INVALID_ARG, "null argument");
    Field *mass, *fp, *prev;
    SPHX_TRY(b->need("Mass", SPHX_F64, 1, &mass));
    SPHX_TRY(b->require("ForcePrior", SPHX_F64, b->dim, &fp));
    SPHX_TRY(b->require("PreviousGravityForce", SPHX_F64, b->dim, &prev));
    if (b->n == 0)
        return SPHX_OK;
    k_gravity<<<grid_for(b->n, 256), 256, 0, b->ctx->stream>>>(
        b->n, b->dim, static_cast<const double *>(mass->dev), g[0], g[1], b->dim == 3 ? g[2] : 0.0,
        static_cast<double *>(fp->dev), static_cast<double *>(prev->dev));
    SPHX_LAUNCHED(b->ctx);
    return SPHX_OK;
}

extern "C" int sphx_observe_quantity(sphx_relation rel, const char *name, double *out)
{
    if (!rel || !name || !out || rel->inner || !rel->W)
        return fail(SPHX_ERR_INVALID_ARG, "observation needs a contact relation from observer points");
    sphx_body tgt = rel->tgt;
    Field *Vol, *q;
    SPHX_TRY(tgt->need("VolumetricMeasure", SPHX_F64, 1, &Vol));
    SPHX_TRY(tgt->need(name, SPHX_F64, 1, &q));
    size_t n = rel->src->n;
    if (n == 0)
        return SPHX_OK;
    if (rel->n_src != n)
        return fail(SPHX_ERR_INVALID_ARG, "observer relation not updated");
    sphx_ctx ctx = rel->ctx;
    SPHX_TRY(ctx->ensure_scratch(n * sizeof(double)));
    double *d_out = static_cast<double *>(ctx->d_scratch);
    k_observe<<<unsigned(n), 32, 0, ctx->stream>>>(n, tgt->n, unsigned(rel->cap), rel->count, rel->j, rel->W,
                                                   static_cast<const double *>(Vol->dev),
                                                   static_cast<const double *>(q->dev), d_out);
    SPHX_LAUNCHED(ctx);
    SPHX_CUDA(cudaMemcpyAsync(out, d_out, n * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    SPHX_CUDA(cudaStreamSynchronize(ctx->stream));
    return SPHX_OK;
}

extern "C" int sphx_total_mechanical_energy(sphx_body b, const double *g, double *energy)
{
    if (!b || !g || !energy)
        return fail(SPHX_ERR_INVALID_ARG, "null argument");
    Field *pos, *vel, *mass;
    SPHX_TRY(b->need("Position", SPHX_F64, b->dim, &pos));
    SPHX_TRY(b->require("Velocity", SPHX_F64, b->dim, &vel));
    SPHX_TRY(b->need("Mass", SPHX_F64, 1, &mass));
    sphx_ctx ctx = b->ctx;
    size_t n = b->n;
    unsigned np = reduce_grid(ctx, std::max<size_t>(n, 1));
    SPHX_TRY(ctx->ensure_scratch((np + 1) * sizeof(double)));
    double *part = static_cast<double *>(ctx->d_scratch);
    double g2 = b->dim == 3 ? g[2] : 0.0;
    if (b->dim == 2)
        k_energy_partials<2><<<np, kBlock, 0, ctx->stream>>>(n, static_cast<const double *>(pos->dev),
                                                             static_cast<const double *>(vel->dev),
                                                             static_cast<const double *>(mass->dev), g[0], g[1], g2,
                                                             part);
    else
        k_energy_partials<3><<<np, kBlock, 0, ctx->stream>>>(n, static_cast<const double *>(pos->dev),
                                                             static_cast<const double *>(vel->dev),
                                                             static_cast<const double *>(mass->dev), g[0], g[1], g2,
                                                             part);
    SPHX_LAUNCHED(ctx);
    k_sum_partials<<<1, 32, 0, ctx->stream>>>(np, part, part + np);
    SPHX_LAUNCHED(ctx);
    SPHX_CUDA(cudaMemcpyAsync(energy, part + np, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    SPHX_CUDA(cudaStreamSynchronize(ctx->stream));
    return SPHX_OK;
}

extern "C" int sphx_density_summation_inner(sphx_relation inner, const sphx_fluid_params *p)
{
    SPHX_TRY(check_pair(inner, nullptr, p));
    sphx_body b = inner->src;
    FluidVars f;
    SPHX_TRY(fluid_vars(b, f));
    size_t n = b->n;
    if (n == 0)
        return SPHX_OK;
    sphx_ctx ctx = b->ctx;
    k_density_summation<<<grid_for(n, 256), 256, 0, ctx->stream>>>(n, inner->wsum, nullptr, f.mass, p->rho0,
                                                                   1.0 / p->sigma0, f.rho_sum, f.rho, 0);
    SPHX_LAUNCHED(ctx);
    return SPHX_OK;
}

extern "C" int sphx_viscous_force_inner(sphx_relation inner, double mu)
{
    if (!inner || !inner->inner)
        return fail(SPHX_ERR_INVALID_ARG, "an inner relation is required");
    if (!inner->r)
        return fail(SPHX_ERR_INVALID_ARG, "the inner relation keeps no distances: call "
                                          "sphx_relation_keep_distances before its update");
    sphx_body b = inner->src;
    if (inner->n_src != b->n)
        return fail(SPHX_ERR_INVALID_ARG, "relation not updated for the current particle count");
    const int D = b->dim;
    Field *vel, *Vol, *fp, *visc, *prev;
    SPHX_TRY(b->require("Velocity", SPHX_F64, D, &vel));
    SPHX_TRY(b->need("VolumetricMeasure", SPHX_F64, 1, &Vol));
    SPHX_TRY(b->require("ForcePrior", SPHX_F64, D, &fp));
    SPHX_TRY(b->require("ViscousForce", SPHX_F64, D, &visc));
    SPHX_TRY(b->require("PreviousViscousForce", SPHX_F64, D, &prev));
    size_t n = b->n;
    if (n == 0)
        return SPHX_OK;
    sphx_ctx ctx = b->ctx;
    Neighbors in = neighbors_of(inner);
    auto d = [](Field *f) { return static_cast<double *>(f->dev); };
    if (D == 2)
        k_viscous_inner<2><<<grid_for(n, kBlock), kBlock, 0, ctx->stream>>>(n, in, d(vel), d(Vol), mu, inner->h,
                                                                            d(visc), d(prev), d(fp));
    else
        k_viscous_inner<3><<<grid_for(n, kBlock), kBlock, 0, ctx->stream>>>(n, in, d(vel), d(Vol), mu, inner->h,
                                                                            d(visc), d(prev), d(fp));
    SPHX_LAUNCHED(ctx);
    return SPHX_OK;
}

extern "C" int sphx_transport_velocity_correction_inner(sphx_relation inner, double coefficient)
{
    if (!inner || !inner->inner)
        return fail(SPHX_ERR_INVALID_ARG, "an inner relation is required");
    sphx_body b = inner->src;
    if (inner->n_src != b->n)
        return fail(SPHX_ERR_INVALID_ARG, "relation not updated for the current particle count");
    const int D = b->dim;
    Field *pos, *Vol;
    SPHX_TRY(b->need("Position", SPHX_F64, D, &pos));
    SPHX_TRY(b->need("VolumetricMeasure", SPHX_F64, 1, &Vol));
    size_t n = b->n;
    if (n == 0)
        return SPHX_OK;
    sphx_ctx ctx = b->ctx;
    double h2 = inner->h * inner->h;
    Neighbors in = neighbors_of(inner);
    double *p = static_cast<double *>(pos->dev);
    const double *V = static_cast<const double *>(Vol->dev);
    if (D == 2)
        k_tvc_inner<2><<<grid_for(n, kBlock), kBlock, 0, ctx->stream>>>(n, in, V, h2, coefficient * h2, p);
    else
        k_tvc_inner<3><<<grid_for(n, kBlock), kBlock, 0, ctx->stream>>>(n, in, V, h2, coefficient * h2, p);
    SPHX_LAUNCHED(ctx);
    return SPHX_OK;
}

extern "C" int sphx_maximum_speed(sphx_body b, double *out)
{
    if (!b || !out)
        return fail(SPHX_ERR_INVALID_ARG, "null argument");
    Field *vel;
    SPHX_TRY(b->require("Velocity", SPHX_F64, b->dim, &vel));
    sphx_ctx ctx = b->ctx;
    size_t n = b->n;
    SPHX_CUDA(cudaMemsetAsync(ctx->d_red, 0, sizeof(unsigned long long), ctx->stream));
    if (n > 0)
    {
        unsigned g = reduce_grid(ctx, n);
        if (b->dim == 2)
            k_acoustic_max<2><<<g, kBlock, 0, ctx->stream>>>(n, static_cast<const double *>(vel->dev), 0.0,
                                                             ctx->d_red);
        else
            k_acoustic_max<3><<<g, kBlock, 0, ctx->stream>>>(n, static_cast<const double *>(vel->dev), 0.0,
                                                             ctx->d_red);
        SPHX_LAUNCHED(ctx);
    }
    double m = 0;
    SPHX_TRY(read_max(ctx, &m));
    *out = n > 0 ? m : 0.0;
    return SPHX_OK;
}

extern "C" int sphx_upper_front_in_axis_direction(sphx_body b, int axis, const double *lo, const double *up,
                                                  double *front)
{
    if (!b || !lo || !up || !front || axis < 0 || axis >= b->dim)
        return fail(SPHX_ERR_INVALID_ARG, "invalid upper-front arguments");
    Field *pos;
    SPHX_TRY(b->need("Position", SPHX_F64, b->dim, &pos));
    sphx_ctx ctx = b->ctx;
    size_t n = b->n;
    SPHX_CUDA(cudaMemsetAsync(ctx->d_red, 0, sizeof(unsigned long long), ctx->stream));
    if (n > 0)
    {
        unsigned g = reduce_grid(ctx, n);
        double l2 = b->dim == 3 ? lo[2] : 0.0, u2 = b->dim == 3 ? up[2] : 0.0;
        if (b->dim == 2)
            k_upper_front<2><<<g, kBlock, 0, ctx->stream>>>(n, static_cast<const double *>(pos->dev), axis, lo[0],
                                                            lo[1], l2, up[0], up[1], u2, ctx->d_red);
        else
            k_upper_front<3><<<g, kBlock, 0, ctx->stream>>>(n, static_cast<const double *>(pos->dev), axis, lo[0],
                                                            lo[1], l2, up[0], up[1], u2, ctx->d_red);
        SPHX_LAUNCHED(ctx);
    }
    SPHX_TRY(read_max(ctx, front));
    return SPHX_OK;
}
