// CK numerics of the fluid step on the device (FP64 drop-in of the particle methods the
// tests_sycl dam-break drivers instantiate, tests/tests_sycl/2d_examples/
// test_2d_dambreak_sycl/dambreak_sycl.cpp:97-123):
//
//   KernelTabulatedCK + Neighbor<SPHAdaptation, SPHAdaptation>  kernel_tabulated_ck.h:37-62,
//                                         kernel_tabulated_ck.cpp:5-25, neighbor_method.hpp:66-142
//   LinearCorrectionMatrix<Inner<WithUpdate>> + <Contact>        kernel_correction_ck.hpp:25-80
//   AcousticStep1stHalf / 2ndHalf <Inner<OneLevel, AcousticRiemannSolverCK, LinearCorrectionCK>>
//     + <Contact<Wall, ...>>                acoustic_step_1st_half.hpp, acoustic_step_2nd_half.hpp
//   RiemannSolver AverageP / AverageV / DissipativePJump / DissipativeUJump
//                                                                 riemann_solver_ck.hpp:14-50
//   CompressionSummation + DensityRegularization<FreeSurface>     density_regularization.hpp:40-118
//   AdvectionStepSetup / UpdateParticlePosition                   fluid_time_step_ck.h:145-176
//   AcousticTimeStepCK / AdvectionTimeStepCK                      fluid_time_step_ck.hpp:25-57,
//                                                                 fluid_time_step_ck.cpp:16-20
//
// Pair geometry comes from the current Position, which the CK loop moves once per
// advection step (UpdateParticlePosition); the neighbour index lists are the relations'
// (the cut-off test of the configuration).  Every sum runs in list order, so results match
// the oracle's restatement to rounding.  Fusion: the 1st half is two launches
// (compression / density / pressure / displacement initialisation, then interaction + wall
// + velocity update), the 2nd half one launch (displacement, interaction, wall, compression
// update): each fused update touches only the particle's own variables, which no other
// particle reads in that interaction.
#include <algorithm>
#include <cmath>
#include <string>
#include <vector>

#include "sphx_device.cuh"
#include "sphx_internal.cuh"

using namespace sphx;

namespace
{
constexpr unsigned kBlock = 128;
constexpr int kTab = 24; // kernel_resolution_ 20 + 4

// Tabulated Wendland C2 of one smoothing length.
struct TabK
{
    double inv_h, inv_hW, inv_hdW, dim_factor, dq, d0, d1, d2, d3;
    double w[kTab], dw[kTab];
};

TabK make_tab(int D, double h)
{
    TabK t{};
    const double Pi = M_PI;
    double kinv_h = 1.0 / h;
    double fW2 = kinv_h * kinv_h * 7.0 / (4.0 * Pi), fW3 = kinv_h * kinv_h * kinv_h * 21.0 / (16.0 * Pi);
    t.dim_factor = D == 2 ? fW2 * h * h : fW3 * h * h * h; // Kernel::DimensionFactor2D/3D
    t.dq = 2.0 / 20.0;
    for (int i = 0; i < kTab; ++i)
    {
        double q = double(i - 1) * t.dq;
        t.w[i] = std::pow(1.0 - 0.5 * q, 4) * (1.0 + 2.0 * q); // KernelWendlandC2::W_1D
        t.dw[i] = 0.625 * std::pow(q - 2.0, 3) * q;            // KernelWendlandC2::dW_1D
    }
    t.d0 = (-1.0 * t.dq) * (-2.0 * t.dq) * (-3.0 * t.dq);
    t.d1 = t.dq * (-1.0 * t.dq) * (-2.0 * t.dq);
    t.d2 = (2.0 * t.dq) * t.dq * (-1.0 * t.dq);
    t.d3 = (3.0 * t.dq) * (2.0 * t.dq) * t.dq;
    t.inv_h = 1.0 / h;
    double h2 = t.inv_h * t.inv_h, h3 = h2 * t.inv_h, h4 = h3 * t.inv_h;
    t.inv_hW = D == 2 ? h2 : h3;
    t.inv_hdW = D == 2 ? h3 : h4;
    return t;
}

__device__ __forceinline__ double cubic(const TabK &t, const double *data, double q)
{
    int location = int(floor(q / t.dq));
    int i = location + 1;
    double f1 = q - double(location) * t.dq, f0 = f1 + t.dq, f2 = f1 - t.dq, f3 = f1 - 2 * t.dq;
    return (f1 * f2 * f3) / t.d0 * data[i - 1] + (f0 * f2 * f3) / t.d1 * data[i] +
           (f0 * f1 * f3) / t.d2 * data[i + 1] + (f0 * f1 * f2) / t.d3 * data[i + 2];
}
__device__ __forceinline__ double tW(const TabK &t, double r) { return t.inv_hW * t.dim_factor * cubic(t, t.w, r * t.inv_h); }
__device__ __forceinline__ double tdW(const TabK &t, double r)
{
    return t.inv_hdW * t.dim_factor * cubic(t, t.dw, r * t.inv_h);
}
__device__ __forceinline__ double tW0(const TabK &t) { return t.inv_hW * t.dim_factor * cubic(t, t.w, 0.0); }

struct Lists
{
    const uint32_t *count, *J;
    size_t n_src;
    unsigned cap;
    uint32_t limit; // target particles the entries index (tested by the checked build)
};

// Entry j indexes a target particle (always true unless built with SPHX_CHECK).
__device__ __forceinline__ bool entry_ok(const Lists &l, uint32_t j)
{
    return SPHX_CHECKED(j < l.limit, kCheckListEntry, j);
}

Lists lists_of(sphx_relation r)
{
    Lists l{};
    if (!r)
        return l;
    l.count = r->count;
    l.J = r->j;
    l.n_src = r->n_src;
    l.cap = unsigned(r->cap);
    l.limit = uint32_t(r->tgt ? r->tgt->n : 0);
    return l;
}

// x_i - x_j, |x_i - x_j| ((dx^2 + dy^2) + dz^2) and its normalisation (Eigen normalized())
template <int D>
__device__ __forceinline__ double geometry(const double *pos_i, size_t ni, size_t i, const double *pos_j, size_t nj,
                                           size_t j, double *r, double *e)
{
    for (int a = 0; a < D; ++a)
        r[a] = pos_i[a * ni + i] - pos_j[a * nj + j];
    double n2 = __dadd_rn(__dmul_rn(r[0], r[0]), __dmul_rn(r[1], r[1]));
    if (D == 3)
        n2 = __dadd_rn(n2, __dmul_rn(r[2], r[2]));
    double len = sqrt(n2);
    for (int a = 0; a < D; ++a)
        e[a] = n2 > 0 ? r[a] / len : r[a];
    return len;
}

template <int D>
__device__ __forceinline__ double dot(const double *a, const double *b)
{
    double s = a[0] * b[0] + a[1] * b[1];
    if (D == 3)
        s = s + a[2] * b[2];
    return s;
}

// y = B x for the row-major D x D matrix of particle i (SoA: element (a, b) at B[(a D + b) n + i])
template <int D>
__device__ __forceinline__ void matvec(const double *B, size_t n, size_t i, const double *x, double *y)
{
    for (int a = 0; a < D; ++a)
    {
        double s = 0;
        for (int b = 0; b < D; ++b)
            s += B[(a * D + b) * n + i] * x[b];
        y[a] = s;
    }
}

struct CKFluid
{
    double *pos, *vel, *force, *rho, *p, *Vol;
    const double *force_prior, *mass;
    double *compression, *rate, *dpos, *B, *Vol_ref, *csum;
};

struct CKWall
{
    const double *pos, *Vol, *Vol_ref, *acc, *vel_ave, *n;
    size_t nw;
};

struct CKParams
{
    double rho0, p0, Z, inv_Zsum, inv_rho0c0_ave, rho0c0_geo_ave, inv_c0_ave, slope;
};

CKParams make_ck_params(const sphx_fluid_params &p)
{
    CKParams c{};
    c.rho0 = p.rho0;
    c.p0 = p.rho0 * p.c0 * p.c0;
    double Z = p.rho0 * p.c0;
    c.Z = Z;
    c.inv_Zsum = 1.0 / (Z + Z);
    c.inv_rho0c0_ave = (Z + Z) / (std::pow(Z, 2.0) + std::pow(Z, 2.0));
    c.rho0c0_geo_ave = 2.0 * Z * Z * c.inv_Zsum;
    c.inv_c0_ave = 0.5 * (p.rho0 + p.rho0) * c.inv_rho0c0_ave;
    c.slope = p.limiter_slope;
    return c;
}

__device__ __forceinline__ double p_jump(const CKParams &c, double u)
{
    return c.rho0c0_geo_ave * u * fmin(c.slope * (c.inv_c0_ave * fmax(u, 0.0)), 1.0);
}

// ---------------------------------------------------------------- kernels
// CompressionSummation<Inner, Contact> and, with REGULARIZE, the post-state
// DensityRegularization<FreeSurface> in the same pass.
template <int D, bool REGULARIZE>
__device__ __forceinline__ void ck_summation(size_t n, const CKFluid &f, const CKWall &w, const Lists &in,
                                             const Lists &wl, const TabK &t, double rho0)
{
    size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    double sum = tW0(t) * f.Vol_ref[i];
    double r[3], e[3];
    unsigned c = min(in.count[i], in.cap);
    for (unsigned s = 0; s < c; ++s)
    {
        uint32_t j = in.J[size_t(s) * n + i];
        if (!entry_ok(in, j))
            continue;
        double len = geometry<D>(f.pos, n, i, f.pos, n, j, r, e);
        sum += tW(t, len) * f.Vol_ref[j];
    }
    if (wl.J)
    {
        c = min(wl.count[i], wl.cap);
        for (unsigned s = 0; s < c; ++s)
        {
            uint32_t j = wl.J[size_t(s) * n + i];
            if (!entry_ok(wl, j))
                continue;
            double len = geometry<D>(f.pos, n, i, w.pos, w.nw, j, r, e);
            sum += tW(t, len) * w.Vol_ref[j];
        }
    }
    f.csum[i] = sum;
    if (REGULARIZE)
    {
        double comp = fmax(sum, 1.0);
        f.compression[i] = comp;
        f.rho[i] = comp * rho0;
    }
}

template <int D>
__global__ void k_ck_regularization(size_t n, CKFluid f, CKWall w, Lists in, Lists wl, TabK t, double rho0)
{
    ck_summation<D, true>(n, f, w, in, wl, t, rho0);
}

template <int D>
__global__ void k_ck_compression_summation(size_t n, CKFluid f, CKWall w, Lists in, Lists wl, TabK t, double rho0)
{
    ck_summation<D, false>(n, f, w, in, wl, t, rho0);
}

// DensityRegularization<SPHBody, WeaklyCompressibleFluid, FreeSurface> alone
// (density_regularization.h:164-180): compression = max(CompressionSummation, 1).
template <int D>
__global__ void k_ck_free_surface_regularization(size_t n, CKFluid f, double rho0)
{
    size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    double comp = fmax(f.csum[i], 1.0);
    f.compression[i] = comp;
    f.rho[i] = comp * rho0;
}

template <int D>
__global__ void k_ck_setup(size_t n, CKFluid f)
{
    size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    f.Vol[i] = f.mass[i] / f.rho[i];
    for (int a = 0; a < D; ++a)
        f.dpos[a * n + i] = 0.0;
}

template <int D>
__global__ void k_ck_update_position(size_t n, CKFluid f)
{
    size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    for (int a = 0; a < D; ++a)
        f.pos[a * n + i] += f.dpos[a * n + i];
}

template <int D>
__device__ __forceinline__ double det(const double *M)
{
    if (D == 2)
        return M[0] * M[3] - M[1] * M[2];
    return M[0] * (M[4] * M[8] - M[5] * M[7]) - M[1] * (M[3] * M[8] - M[5] * M[6]) +
           M[2] * (M[3] * M[7] - M[4] * M[6]);
}
template <int D>
__device__ __forceinline__ void inverse(const double *A, double *R)
{
    double d = det<D>(A);
    if (D == 2)
    {
        R[0] = A[3] / d;
        R[1] = -A[1] / d;
        R[2] = -A[2] / d;
        R[3] = A[0] / d;
        return;
    }
    R[0] = (A[4] * A[8] - A[5] * A[7]) / d;
    R[1] = (A[2] * A[7] - A[1] * A[8]) / d;
    R[2] = (A[1] * A[5] - A[2] * A[4]) / d;
    R[3] = (A[5] * A[6] - A[3] * A[8]) / d;
    R[4] = (A[0] * A[8] - A[2] * A[6]) / d;
    R[5] = (A[2] * A[3] - A[0] * A[5]) / d;
    R[6] = (A[3] * A[7] - A[4] * A[6]) / d;
    R[7] = (A[1] * A[6] - A[0] * A[7]) / d;
    R[8] = (A[0] * A[4] - A[1] * A[3]) / d;
}

template <int D>
__global__ void k_ck_correction(size_t n, CKFluid f, CKWall w, Lists in, Lists wl, TabK t, double alpha)
{
    size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    double B[D * D];
    for (int k = 0; k < D * D; ++k)
        B[k] = 0.0;
    double r[3], e[3];
    auto add = [&](double len, double Vj) {
        double dW = tdW(t, len);
        for (int a = 0; a < D; ++a)
            for (int b = 0; b < D; ++b)
                B[a * D + b] -= r[a] * (dW * e[b] * Vj);
    };
    unsigned c = min(in.count[i], in.cap);
    for (unsigned s = 0; s < c; ++s)
    {
        uint32_t j = in.J[size_t(s) * n + i];
        if (!entry_ok(in, j))
            continue;
        add(geometry<D>(f.pos, n, i, f.pos, n, j, r, e), f.Vol[j]);
    }
    if (wl.J)
    {
        c = min(wl.count[i], wl.cap);
        for (unsigned s = 0; s < c; ++s)
        {
            uint32_t j = wl.J[size_t(s) * n + i];
            if (!entry_ok(wl, j))
                continue;
            add(geometry<D>(f.pos, n, i, w.pos, w.nw, j, r, e), w.Vol[j]);
        }
    }
    double determinant = det<D>(B);
    double det_sqr = fmax(alpha - determinant, 0.0);
    // inverseTikhonov (vector_functions.h:199-203): (B^T B + eps I)^-1 B^T, eps = SqrtEps
    double BtB[D * D], Inv[D * D];
    for (int a = 0; a < D; ++a)
        for (int b = 0; b < D; ++b)
        {
            double sum = 0;
            for (int k = 0; k < D; ++k)
                sum += B[k * D + a] * B[k * D + b];
            BtB[a * D + b] = sum + (a == b ? 1.0e-8 : 0.0);
        }
    inverse<D>(BtB, Inv);
    double weight = determinant / (determinant + det_sqr);
    for (int a = 0; a < D; ++a)
        for (int b = 0; b < D; ++b)
        {
            double sum = 0;
            for (int k = 0; k < D; ++k)
                sum += Inv[a * D + k] * B[b * D + k];
            f.B[(a * D + b) * n + i] = weight * sum + (1.0 - weight) * (a == b ? 1.0 : 0.0);
        }
}

template <int D>
__global__ void k_ck_init1(size_t n, CKFluid f, CKParams k, double dt)
{
    size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    double comp = f.compression[i] + 0.5 * dt * f.rate[i];
    f.compression[i] = comp;
    double rho = comp * k.rho0;
    f.rho[i] = rho;
    f.p[i] = k.p0 * (rho / k.rho0 - 1.0);
    for (int a = 0; a < D; ++a)
        f.dpos[a * n + i] += f.vel[a * n + i] * dt * 0.5;
}

template <int D>
__global__ void __launch_bounds__(kBlock) k_ck_interact1(size_t n, CKFluid f, CKWall w, Lists in, Lists wl, TabK t,
                                                         CKParams k, double dt)
{
    size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    const double p_i = f.p[i];
    double fs[3] = {0, 0, 0}, dis = 0;
    double r[3], e[3], bi[3], bj[3];
    unsigned c = min(in.count[i], in.cap);
    for (unsigned s = 0; s < c; ++s)
    {
        uint32_t j = in.J[size_t(s) * n + i];
        if (!entry_ok(in, j))
            continue;
        double len = geometry<D>(f.pos, n, i, f.pos, n, j, r, e);
        double dWV = tdW(t, len) * f.Vol[j];
        matvec<D>(f.B, n, j, e, bj);
        matvec<D>(f.B, n, i, e, bi);
        const double p_j = f.p[j];
        for (int a = 0; a < D; ++a)
            fs[a] -= k.inv_Zsum * (p_i * k.Z * bj[a] + p_j * k.Z * bi[a]) * 2.0 * dWV;
        dis += (p_i - p_j) * k.inv_rho0c0_ave * dWV;
    }
    const double Vol_i = f.Vol[i], comp_i = f.compression[i];
    for (int a = 0; a < D; ++a)
        f.force[a * n + i] += fs[a] * Vol_i;
    double rate = dis * comp_i;
    if (wl.J)
    {
        double wf[3] = {0, 0, 0}, wdis = 0;
        const double rho_i = f.rho[i], m_i = f.mass[i];
        c = min(wl.count[i], wl.cap);
        for (unsigned s = 0; s < c; ++s)
        {
            uint32_t j = wl.J[size_t(s) * n + i];
            if (!entry_ok(wl, j))
                continue;
            double len = geometry<D>(f.pos, n, i, w.pos, w.nw, j, r, e);
            double dWV = tdW(t, len) * w.Vol[j];
            double acc[3];
            for (int a = 0; a < D; ++a)
                acc[a] = -(f.force_prior[a * n + i] / m_i - w.acc[a * w.nw + j]);
            double face = dot<D>(acc, e);
            double p_wall = p_i + rho_i * len * fmax(0.0, face);
            matvec<D>(f.B, n, i, e, bi);
            for (int a = 0; a < D; ++a)
                wf[a] -= (p_i + p_wall) * bi[a] * dWV;
            wdis += (p_i - p_wall) * k.inv_rho0c0_ave * dWV;
        }
        for (int a = 0; a < D; ++a)
            f.force[a * n + i] += wf[a] * Vol_i;
        rate += wdis * comp_i;
    }
    f.rate[i] = rate;
    const double m_i = f.mass[i];
    for (int a = 0; a < D; ++a)
        f.vel[a * n + i] += (f.force_prior[a * n + i] + f.force[a * n + i]) / m_i * dt;
}

template <int D>
__global__ void __launch_bounds__(kBlock) k_ck_second(size_t n, CKFluid f, CKWall w, Lists in, Lists wl, TabK t,
                                                      CKParams k, double dt)
{
    size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    double v_i[3] = {0, 0, 0};
    for (int a = 0; a < D; ++a)
    {
        v_i[a] = f.vel[a * n + i];
        f.dpos[a * n + i] += v_i[a] * dt * 0.5;
    }
    double div = 0, pd[3] = {0, 0, 0};
    double r[3], e[3], be[3];
    unsigned c = min(in.count[i], in.cap);
    for (unsigned s = 0; s < c; ++s)
    {
        uint32_t j = in.J[size_t(s) * n + i];
        if (!entry_ok(in, j))
            continue;
        double len = geometry<D>(f.pos, n, i, f.pos, n, j, r, e);
        double dWV = tdW(t, len) * f.Vol[j];
        matvec<D>(f.B, n, i, e, be);
        double dv[3], du[3];
        for (int a = 0; a < D; ++a)
        {
            double v_j = f.vel[a * n + j];
            double v_ave = (v_i[a] * k.Z + v_j * k.Z) * k.inv_Zsum;
            dv[a] = v_i[a] - v_ave;
            du[a] = v_i[a] - v_j;
        }
        div += 2.0 * dot<D>(dv, be) * dWV;
        double pj = p_jump(k, dot<D>(du, e)) * dWV;
        for (int a = 0; a < D; ++a)
            pd[a] += pj * e[a];
    }
    const double comp_i = f.compression[i], Vol_i = f.Vol[i];
    double rate = f.rate[i] + div * comp_i;
    double F[3];
    for (int a = 0; a < D; ++a)
        F[a] = pd[a] * Vol_i;
    if (wl.J)
    {
        double wdiv = 0, wd[3] = {0, 0, 0};
        c = min(wl.count[i], wl.cap);
        for (unsigned s = 0; s < c; ++s)
        {
            uint32_t j = wl.J[size_t(s) * n + i];
            if (!entry_ok(wl, j))
                continue;
            double len = geometry<D>(f.pos, n, i, w.pos, w.nw, j, r, e);
            double dWV = tdW(t, len) * w.Vol[j];
            double vel_diff[3], nj[3];
            matvec<D>(f.B, n, i, e, be);
            for (int a = 0; a < D; ++a)
            {
                vel_diff[a] = 2.0 * (v_i[a] - w.vel_ave[a * w.nw + j]);
                nj[a] = w.n[a * w.nw + j];
            }
            wdiv += dot<D>(vel_diff, be) * dWV;
            double en = dot<D>(e, nj);
            double sgn = en > 0 ? 1.0 : (en < 0 ? -1.0 : 0.0);
            double ns[3];
            for (int a = 0; a < D; ++a)
                ns[a] = sgn * nj[a];
            double pj = p_jump(k, dot<D>(vel_diff, ns)) * dWV;
            for (int a = 0; a < D; ++a)
                wd[a] += pj * ns[a];
        }
        rate += wdiv * comp_i;
        for (int a = 0; a < D; ++a)
            F[a] += wd[a] * Vol_i;
    }
    f.rate[i] = rate;
    for (int a = 0; a < D; ++a)
        f.force[a * n + i] = F[a];
    double comp = comp_i + 0.5 * dt * rate;
    f.compression[i] = comp;
    f.rho[i] = comp * k.rho0;
}

__device__ __forceinline__ void block_max(unsigned long long *slot, double v)
{
    unsigned long long b = ordered_bits(v);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
    {
        unsigned long long y = __shfl_down_sync(0xffffffffu, b, o);
        b = y > b ? y : b;
    }
    if ((threadIdx.x & 31u) == 0)
        atomicMax(slot, b);
}

// FreeSurfaceIndicationCK<Inner<WithUpdate>, Contact<>> (surface_indication_ck.hpp:49-150):
// position divergence -sum dW V r over the inner neighbours with the spatial-temporal rule
// (a particle below the threshold that was not a surface particle and has no previous
// surface particle among its neighbours is lifted to twice the threshold), the wall
// neighbours added, then the indicator: 0 above the threshold unless a neighbour closer
// than h lies below it; the previous indicator takes the new value.
template <int D>
__global__ void k_ck_indication_inner(size_t n, CKFluid f, Lists in, TabK t, const int *__restrict__ prev,
                                      double *__restrict__ pos_div, double thr)
{
    size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    double pd = 0.0, r[3], e[3];
    const unsigned c = min(in.count[i], in.cap);
    for (unsigned s = 0; s < c; ++s)
    {
        uint32_t j = in.J[size_t(s) * n + i];
        if (!entry_ok(in, j))
            continue;
        double len = geometry<D>(f.pos, n, i, f.pos, n, j, r, e);
        pd -= tdW(t, len) * f.Vol[j] * len;
    }
    if (pd < thr && prev[i] != 1)
    {
        bool near_previous = false;
        for (unsigned s = 0; s < c && !near_previous; ++s)
            near_previous = prev[in.J[size_t(s) * n + i]] == 1;
        if (!near_previous)
            pd = 2.0 * thr;
    }
    pos_div[i] = pd;
}

template <int D>
__global__ void k_ck_indication_contact(size_t n, CKFluid f, CKWall w, Lists wl, TabK t, double *__restrict__ pos_div)
{
    size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    double pd = 0.0, r[3], e[3];
    const unsigned c = min(wl.count[i], wl.cap);
    for (unsigned s = 0; s < c; ++s)
    {
        uint32_t j = wl.J[size_t(s) * n + i];
        if (!entry_ok(wl, j))
            continue;
        double len = geometry<D>(f.pos, n, i, w.pos, w.nw, j, r, e);
        pd -= tdW(t, len) * w.Vol[j] * len;
    }
    pos_div[i] += pd;
}

template <int D>
__global__ void k_ck_indication_update(size_t n, CKFluid f, Lists in, const double *__restrict__ pos_div,
                                       int *__restrict__ indicator, int *__restrict__ prev, double thr, double h)
{
    size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    int v = 1;
    if (pos_div[i] > thr)
    {
        bool very_near = false;
        double r[3], e[3];
        const unsigned c = min(in.count[i], in.cap);
        for (unsigned s = 0; s < c && !very_near; ++s)
        {
            uint32_t j = in.J[size_t(s) * n + i];
            if (!entry_ok(in, j))
                continue;
            double len = geometry<D>(f.pos, n, i, f.pos, n, j, r, e);
            very_near = pos_div[j] < thr && len < h;
        }
        if (!very_near)
            v = 0;
    }
    indicator[i] = v;
    prev[i] = v;
}

template <int D>
__global__ void k_ck_acoustic_max(size_t n, CKFluid f, double c0, double h_min, unsigned long long *slot)
{
    double m = 0.0;
    for (size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += size_t(gridDim.x) * blockDim.x)
    {
        double F[3], v[3];
        for (int a = 0; a < D; ++a)
        {
            F[a] = f.force[a * n + i] + f.force_prior[a * n + i];
            v[a] = f.vel[a * n + i];
        }
        double acc_scale = sqrt(4.0 * h_min * sqrt(dot<D>(F, F)) / f.mass[i]);
        m = fmax(m, fmax(c0 + sqrt(dot<D>(v, v)), acc_scale));
    }
    block_max(slot, m);
}

template <int D>
__global__ void k_ck_advection_max(size_t n, CKFluid f, unsigned long long *slot)
{
    double m = 0.0;
    for (size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += size_t(gridDim.x) * blockDim.x)
    {
        double v[3];
        for (int a = 0; a < D; ++a)
            v[a] = f.vel[a * n + i];
        m = fmax(m, dot<D>(v, v));
    }
    block_max(slot, m);
}

template <int D>
__global__ void k_ck_observe(size_t n_obs, const double *__restrict__ opos, Lists ol, const double *__restrict__ fpos,
                             size_t nf, const double *__restrict__ Vol, const double *__restrict__ q, TabK t,
                             double *__restrict__ out)
{
    size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n_obs)
        return;
    double num = 0, ttl = 0, r[3], e[3];
    unsigned c = min(ol.count[i], ol.cap);
    for (unsigned s = 0; s < c; ++s)
    {
        uint32_t j = ol.J[size_t(s) * n_obs + i];
        double wj = tW(t, geometry<D>(opos, n_obs, i, fpos, nf, j, r, e)) * Vol[j];
        num += wj * q[j];
        ttl += wj;
    }
    out[i] = num / (ttl + kTinyReal);
}

// ---------------------------------------------------------------- host helpers
double *f64(Field *f) { return static_cast<double *>(f->dev); }

// A CK state variable, created on first use with its registration value: Compression and
// CompressionSummation 1, LinearCorrectionMatrix the identity, VolumetricMeasureRef a copy of
// VolumetricMeasure (registerStateVariableFrom), the rest zero.
int ck_field(sphx_body b, const char *name, int ncomp, Field **out)
{
    bool fresh = b->find(name) == nullptr;
    SPHX_TRY(b->require(name, SPHX_F64, ncomp, out));
    if (!fresh || b->n == 0)
        return SPHX_OK;
    sphx_ctx ctx = b->ctx;
    size_t n = b->n;
    std::string s(name);
    if (s == "Compression" || s == "CompressionSummation" || s == "LinearCorrectionMatrix")
    {
        std::vector<double> h(size_t(ncomp) * n, 0.0);
        if (s == "LinearCorrectionMatrix")
        {
            int D = b->dim;
            for (int a = 0; a < D; ++a)
                std::fill(h.begin() + size_t(a * D + a) * n, h.begin() + size_t(a * D + a + 1) * n, 1.0);
        }
        else
            std::fill(h.begin(), h.end(), 1.0);
        SPHX_CUDA(cudaMemcpyAsync((*out)->dev, h.data(), h.size() * sizeof(double), cudaMemcpyHostToDevice,
                                  ctx->stream));
        SPHX_CUDA(cudaStreamSynchronize(ctx->stream));
    }
    else if (s == "VolumetricMeasureRef")
    {
        Field *Vol;
        SPHX_TRY(b->need("VolumetricMeasure", SPHX_F64, 1, &Vol));
        SPHX_CUDA(cudaMemcpyAsync((*out)->dev, Vol->dev, n * sizeof(double), cudaMemcpyDeviceToDevice, ctx->stream));
    }
    return SPHX_OK;
}

int ck_fluid(sphx_body b, CKFluid &f)
{
    const int D = b->dim;
    Field *pos, *vel, *force, *fp, *rho, *p, *Vol, *mass, *comp, *rate, *dpos, *B, *vref, *csum;
    SPHX_TRY(b->need("Position", SPHX_F64, D, &pos));
    SPHX_TRY(b->require("Velocity", SPHX_F64, D, &vel));
    SPHX_TRY(b->require("Force", SPHX_F64, D, &force));
    SPHX_TRY(b->require("ForcePrior", SPHX_F64, D, &fp));
    SPHX_TRY(b->need("Density", SPHX_F64, 1, &rho));
    SPHX_TRY(b->require("Pressure", SPHX_F64, 1, &p));
    SPHX_TRY(b->need("VolumetricMeasure", SPHX_F64, 1, &Vol));
    SPHX_TRY(b->need("Mass", SPHX_F64, 1, &mass));
    SPHX_TRY(ck_field(b, "Compression", 1, &comp));
    SPHX_TRY(ck_field(b, "CompressionRate", 1, &rate));
    SPHX_TRY(ck_field(b, "Displacement", D, &dpos));
    SPHX_TRY(ck_field(b, "LinearCorrectionMatrix", D * D, &B));
    SPHX_TRY(ck_field(b, "VolumetricMeasureRef", 1, &vref));
    SPHX_TRY(ck_field(b, "CompressionSummation", 1, &csum));
    f.pos = f64(pos);
    f.vel = f64(vel);
    f.force = f64(force);
    f.force_prior = f64(fp);
    f.rho = f64(rho);
    f.p = f64(p);
    f.Vol = f64(Vol);
    f.mass = f64(mass);
    f.compression = f64(comp);
    f.rate = f64(rate);
    f.dpos = f64(dpos);
    f.B = f64(B);
    f.Vol_ref = f64(vref);
    f.csum = f64(csum);
    return SPHX_OK;
}

int ck_wall(sphx_relation wall, CKWall &w)
{
    w = CKWall{};
    if (!wall)
        return SPHX_OK;
    sphx_body b = wall->tgt;
    const int D = b->dim;
    Field *pos, *Vol, *vref, *acc, *vel, *n;
    SPHX_TRY(b->need("Position", SPHX_F64, D, &pos));
    SPHX_TRY(b->need("VolumetricMeasure", SPHX_F64, 1, &Vol));
    SPHX_TRY(ck_field(b, "VolumetricMeasureRef", 1, &vref));
    SPHX_TRY(b->require("Acceleration", SPHX_F64, D, &acc));
    SPHX_TRY(b->require("Velocity", SPHX_F64, D, &vel));
    SPHX_TRY(b->need("NormalDirection", SPHX_F64, D, &n));
    w.pos = f64(pos);
    w.Vol = f64(Vol);
    w.Vol_ref = f64(vref);
    w.acc = f64(acc);
    w.vel_ave = f64(vel);
    w.n = f64(n);
    w.nw = b->n;
    return SPHX_OK;
}

int ck_check(sphx_relation inner, sphx_relation wall)
{
    if (!inner || !inner->inner)
        return fail(SPHX_ERR_INVALID_ARG, "an inner relation is required");
    if (wall && (wall->inner || wall->src != inner->src))
        return fail(SPHX_ERR_INVALID_ARG, "the wall relation must be a contact relation of the same fluid body");
    if (inner->n_src != inner->src->n || (wall && wall->n_src != wall->src->n))
        return fail(SPHX_ERR_INVALID_ARG, "relation not updated for the current particle count");
    return SPHX_OK;
}

unsigned red_grid(sphx_ctx ctx, size_t n)
{
    unsigned g = grid_for(n, kBlock);
    unsigned cap = unsigned(std::max(1, ctx->num_sms)) * 8u;
    return std::max(1u, std::min(g, cap));
}

int read_max(sphx_ctx ctx, double *out)
{
    SPHX_CUDA(cudaMemcpyAsync(ctx->h_red, ctx->d_red, sizeof(unsigned long long), cudaMemcpyDeviceToHost,
                              ctx->stream));
    SPHX_CUDA(cudaStreamSynchronize(ctx->stream));
    *out = from_ordered_bits(ctx->h_red[0]);
    return SPHX_OK;
}

} // namespace

#define CK_DISPATCH(b, KERNEL, GRID, ...)                                                                              \
    do                                                                                                                 \
    {                                                                                                                  \
        if ((b)->dim == 2)                                                                                             \
            KERNEL<2><<<GRID, kBlock, 0, (b)->ctx->stream>>>(__VA_ARGS__);                                             \
        else                                                                                                           \
            KERNEL<3><<<GRID, kBlock, 0, (b)->ctx->stream>>>(__VA_ARGS__);                                             \
        SPHX_LAUNCHED((b)->ctx);                                                                                       \
    } while (0)

extern "C" int sphx_ck_density_regularization(sphx_relation inner, sphx_relation wall, const sphx_fluid_params *p)
{
    SPHX_TRY(ck_check(inner, wall));
    if (!p)
        return fail(SPHX_ERR_INVALID_ARG, "null parameters");
    sphx_body b = inner->src;
    CKFluid f;
    CKWall w;
    SPHX_TRY(ck_fluid(b, f));
    SPHX_TRY(ck_wall(wall, w));
    size_t n = b->n;
    if (n == 0)
        return SPHX_OK;
    CK_DISPATCH(b, k_ck_regularization, grid_for(n, kBlock), n, f, w, lists_of(inner), lists_of(wall),
                make_tab(b->dim, inner->h), p->rho0);
    return SPHX_OK;
}

extern "C" int sphx_ck_compression_summation(sphx_relation inner, sphx_relation wall)
{
    SPHX_TRY(ck_check(inner, wall));
    sphx_body b = inner->src;
    CKFluid f;
    CKWall w;
    SPHX_TRY(ck_fluid(b, f));
    SPHX_TRY(ck_wall(wall, w));
    size_t n = b->n;
    if (n == 0)
        return SPHX_OK;
    CK_DISPATCH(b, k_ck_compression_summation, grid_for(n, kBlock), n, f, w, lists_of(inner), lists_of(wall),
                make_tab(b->dim, inner->h), 0.0);
    return SPHX_OK;
}

extern "C" int sphx_ck_free_surface_regularization(sphx_body b, double rho0)
{
    if (!b)
        return fail(SPHX_ERR_INVALID_ARG, "null body");
    CKFluid f;
    SPHX_TRY(ck_fluid(b, f));
    if (b->n == 0)
        return SPHX_OK;
    CK_DISPATCH(b, k_ck_free_surface_regularization, grid_for(b->n, kBlock), b->n, f, rho0);
    return SPHX_OK;
}

extern "C" int sphx_ck_advection_step_setup(sphx_body b)
{
    if (!b)
        return fail(SPHX_ERR_INVALID_ARG, "null body");
    CKFluid f;
    SPHX_TRY(ck_fluid(b, f));
    if (b->n == 0)
        return SPHX_OK;
    CK_DISPATCH(b, k_ck_setup, grid_for(b->n, kBlock), b->n, f);
    return SPHX_OK;
}

extern "C" int sphx_ck_update_particle_position(sphx_body b)
{
    if (!b)
        return fail(SPHX_ERR_INVALID_ARG, "null body");
    CKFluid f;
    SPHX_TRY(ck_fluid(b, f));
    if (b->n == 0)
        return SPHX_OK;
    CK_DISPATCH(b, k_ck_update_position, grid_for(b->n, kBlock), b->n, f);
    return SPHX_OK;
}

extern "C" int sphx_ck_linear_correction_matrix(sphx_relation inner, sphx_relation wall, double alpha)
{
    SPHX_TRY(ck_check(inner, wall));
    sphx_body b = inner->src;
    CKFluid f;
    CKWall w;
    SPHX_TRY(ck_fluid(b, f));
    SPHX_TRY(ck_wall(wall, w));
    size_t n = b->n;
    if (n == 0)
        return SPHX_OK;
    CK_DISPATCH(b, k_ck_correction, grid_for(n, kBlock), n, f, w, lists_of(inner), lists_of(wall),
                make_tab(b->dim, inner->h), alpha);
    return SPHX_OK;
}

extern "C" int sphx_ck_free_surface_indication(sphx_relation inner, sphx_relation wall)
{
    SPHX_TRY(ck_check(inner, wall));
    sphx_body b = inner->src;
    CKFluid f;
    CKWall w;
    SPHX_TRY(ck_fluid(b, f));
    SPHX_TRY(ck_wall(wall, w));
    Field *pd, *ind, *prev;
    SPHX_TRY(b->require("PositionDivergence", SPHX_F64, 1, &pd));
    SPHX_TRY(b->require("Indicator", SPHX_I32, 1, &ind));
    const bool fresh = b->find("PreviousSurfaceIndicator") == nullptr;
    SPHX_TRY(b->require("PreviousSurfaceIndicator", SPHX_I32, 1, &prev));
    size_t n = b->n;
    if (n == 0)
        return SPHX_OK;
    sphx_ctx ctx = b->ctx;
    if (fresh) // registerStateVariable<int>("PreviousSurfaceIndicator", 1)
    {
        std::vector<int> ones(n, 1);
        SPHX_CUDA(cudaMemcpyAsync(prev->dev, ones.data(), n * sizeof(int), cudaMemcpyHostToDevice, ctx->stream));
        SPHX_CUDA(cudaStreamSynchronize(ctx->stream));
    }
    const double thr = 0.75 * b->dim;
    TabK t = make_tab(b->dim, inner->h);
    double *pos_div = f64(pd);
    int *indicator = static_cast<int *>(ind->dev), *previous = static_cast<int *>(prev->dev);
    CK_DISPATCH(b, k_ck_indication_inner, grid_for(n, kBlock), n, f, lists_of(inner), t, previous, pos_div, thr);
    if (wall)
        CK_DISPATCH(b, k_ck_indication_contact, grid_for(n, kBlock), n, f, w, lists_of(wall), t, pos_div);
    CK_DISPATCH(b, k_ck_indication_update, grid_for(n, kBlock), n, f, lists_of(inner), pos_div, indicator, previous,
                thr, inner->h);
    return SPHX_OK;
}

extern "C" int sphx_ck_acoustic_step_1st_half(sphx_relation inner, sphx_relation wall, const sphx_fluid_params *p,
                                              double dt)
{
    SPHX_TRY(ck_check(inner, wall));
    if (!p)
        return fail(SPHX_ERR_INVALID_ARG, "null parameters");
    sphx_body b = inner->src;
    CKFluid f;
    CKWall w;
    SPHX_TRY(ck_fluid(b, f));
    SPHX_TRY(ck_wall(wall, w));
    size_t n = b->n;
    if (n == 0)
        return SPHX_OK;
    CKParams k = make_ck_params(*p);
    CK_DISPATCH(b, k_ck_init1, grid_for(n, kBlock), n, f, k, dt);
    CK_DISPATCH(b, k_ck_interact1, grid_for(n, kBlock), n, f, w, lists_of(inner), lists_of(wall),
                make_tab(b->dim, inner->h), k, dt);
    return SPHX_OK;
}

extern "C" int sphx_ck_acoustic_step_2nd_half(sphx_relation inner, sphx_relation wall, const sphx_fluid_params *p,
                                              double dt)
{
    SPHX_TRY(ck_check(inner, wall));
    if (!p)
        return fail(SPHX_ERR_INVALID_ARG, "null parameters");
    sphx_body b = inner->src;
    CKFluid f;
    CKWall w;
    SPHX_TRY(ck_fluid(b, f));
    SPHX_TRY(ck_wall(wall, w));
    size_t n = b->n;
    if (n == 0)
        return SPHX_OK;
    CK_DISPATCH(b, k_ck_second, grid_for(n, kBlock), n, f, w, lists_of(inner), lists_of(wall),
                make_tab(b->dim, inner->h), make_ck_params(*p), dt);
    return SPHX_OK;
}

extern "C" int sphx_ck_acoustic_time_step(sphx_body b, const sphx_fluid_params *p, double *dt)
{
    if (!b || !p || !dt)
        return fail(SPHX_ERR_INVALID_ARG, "null argument");
    CKFluid f;
    SPHX_TRY(ck_fluid(b, f));
    sphx_ctx ctx = b->ctx;
    SPHX_CUDA(cudaMemsetAsync(ctx->d_red, 0, sizeof(unsigned long long), ctx->stream));
    if (b->n > 0)
        CK_DISPATCH(b, k_ck_acoustic_max, red_grid(ctx, b->n), b->n, f, p->c0, p->h, ctx->d_red);
    double m = 0;
    SPHX_TRY(read_max(ctx, &m));
    if (b->n == 0)
        m = 0.0;
    *dt = p->acoustic_cfl * p->h / (m + kTinyReal);
    return SPHX_OK;
}

extern "C" int sphx_ck_advection_time_step(sphx_body b, const sphx_fluid_params *p, double *dt)
{
    if (!b || !p || !dt)
        return fail(SPHX_ERR_INVALID_ARG, "null argument");
    CKFluid f;
    SPHX_TRY(ck_fluid(b, f));
    sphx_ctx ctx = b->ctx;
    SPHX_CUDA(cudaMemsetAsync(ctx->d_red, 0, sizeof(unsigned long long), ctx->stream));
    if (b->n > 0)
        CK_DISPATCH(b, k_ck_advection_max, red_grid(ctx, b->n), b->n, f, ctx->d_red);
    double m = 0;
    SPHX_TRY(read_max(ctx, &m));
    if (b->n == 0)
        m = 0.0;
    *dt = p->advection_cfl * p->h / (std::max(std::sqrt(m), p->U_ref) + kTinyReal);
    return SPHX_OK;
}

extern "C" int sphx_ck_observe_quantity(sphx_relation observer_contact, const char *name, double *out)
{
    if (!observer_contact || !name || !out || observer_contact->inner)
        return fail(SPHX_ERR_INVALID_ARG, "an observer contact relation, a name and an output are required");
    sphx_body ob = observer_contact->src, fb = observer_contact->tgt;
    if (observer_contact->n_src != ob->n)
        return fail(SPHX_ERR_INVALID_ARG, "relation not updated for the current particle count");
    const int D = ob->dim;
    Field *opos, *fpos, *Vol, *q;
    SPHX_TRY(ob->need("Position", SPHX_F64, D, &opos));
    SPHX_TRY(fb->need("Position", SPHX_F64, D, &fpos));
    SPHX_TRY(fb->need("VolumetricMeasure", SPHX_F64, 1, &Vol));
    SPHX_TRY(fb->need(name, SPHX_F64, 1, &q));
    size_t n = ob->n;
    if (n == 0)
        return SPHX_OK;
    sphx_ctx ctx = ob->ctx;
    SPHX_TRY(ctx->ensure_scratch(n * sizeof(double)));
    double *d_out = static_cast<double *>(ctx->d_scratch);
    CK_DISPATCH(ob, k_ck_observe, grid_for(n, kBlock), n, f64(opos), lists_of(observer_contact), f64(fpos), fb->n,
                f64(Vol), f64(q), make_tab(D, observer_contact->h), d_out);
    SPHX_CUDA(cudaMemcpyAsync(out, d_out, n * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    SPHX_CUDA(cudaStreamSynchronize(ctx->stream));
    return SPHX_OK;
}
