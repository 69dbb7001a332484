// Mixed-precision fused dam-break solver (sphx_mp_*).
//
// Same step sequence as the classic FP64 path (Dambreak.cpp:166-220): advection dt,
// DensitySummationComplexFreeSurface (density_summation.cpp:74-82,124-144),
// Integration1stHalfWithWallRiemann / Integration2ndHalfWithWallRiemann
// (fluid_integration.hpp:49-113,166-231), acoustic / advection time steps
// (fluid_time_step.cpp:21-31,54-65) and the configuration update.
//
// Layout (cell order, re-sorted at every configuration update):
//   geo0   float4  {offset from the cell's lower corner at the last configuration
//                   update (x, y, z), packed integer cell coordinates (15 bits per axis
//                   in 2D, 10 in 3D)}
//   dyn    float4  {velocity (x, y, z), pressure}
//   off    float3  current offset from the same cell corner (SoA)
//   force  float3 (SoA); drho = rho - rho0, drho_dt, drho_sum (density summation) float
//   id     uint32  index of the particle in the FP64 body it came from
// A neighbour's data is one 16-byte load: geo0 for the kernel geometry (both sweeps),
// dyn for its pressure (1st half) or velocity (2nd half).  Pair arithmetic is FP32 with
// compensated sums (plain partial sums over groups of 8 neighbours, Kahan-added); the
// position half-steps, the time-step reductions and the conservation sums are FP64.
// Neighbour index lists (ELL, slot-major) are rebuilt at each configuration update
// together with the density summation's sums; the kernel geometry (W, dW, e) is
// recomputed per pair from geo0, as the reference keeps the configuration-time kernel
// values for the whole advection step.
#include <algorithm>
#include <cmath>
#include <vector>

#include "mp_common.cuh"
#include "sphx_device.cuh"
#include "sphx_internal.cuh"

using namespace sphx;
using namespace sphx::mpc;

namespace
{
struct MPConst
{
    MeshDev m;
    MPParams p;
    double gd[3];
    double acoustic_cfl, advection_cfl, U_ref;
    int periodic;        // periodic flow in the box [lo, up] (sphx_mp_create_periodic)
    double lo[3], up[3];
    double inv_gs;       // 1 / sub-cell spacing
};
using MPFluid = MPState;
using MPLists = MPNeighbors;
struct MPWall : MPWallData
{
    size_t nw;
};

// ---------------------------------------------------------------- (re)hash + sort
// From FP64 positions: component d of particle i at pos[d * comp_stride + i * row_stride]
// (the body's SoA layout, or host rows).
template <int D>
__global__ void k_mp_from_fp64(size_t n, const double *__restrict__ pos, size_t comp_stride, size_t row_stride,
                               MPConst k, uint32_t *__restrict__ ncell, float *__restrict__ noff,
                               uint32_t *__restrict__ key, uint32_t *__restrict__ rank, uint32_t *__restrict__ count)
{
    size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    const MeshDev &m = k.m;
    double x[3] = {0, 0, 0};
#pragma unroll
    for (int d = 0; d < D; ++d)
    {
        x[d] = pos[d * comp_stride + i * row_stride];
        if (k.periodic)
        {
            const double L = k.up[d] - k.lo[d];
            if (x[d] < k.lo[d])
                x[d] += L;
            if (x[d] > k.up[d])
                x[d] -= L;
        }
    }
    int c[3] = {0, 0, 0};
    sub_cell_index<D>(m, k.inv_gs, x, c);
#pragma unroll
    for (int d = 0; d < D; ++d)
        noff[d * n + i] = float(x[d] - cell_corner(m, d, c[d]));
    ncell[i] = pack_cell<D>(c);
    uint32_t lc = linear_cell<D>(m, c);
    key[i] = lc;
    rank[i] = atomicAdd(&count[lc], 1u);
}

// FP64 reconstruction of a position from its (cell, offset) pair.  A periodic flow wraps
// it into its box, as PeriodicBounding does at the end of the advection step
// (domain_bounding.h:103-113); between the position update and the next re-hash the
// offset may still point outside the box.
__device__ __forceinline__ double reconstruct(const MPConst &k, int d, int cell, float offset)
{
    double x = cell_corner(k.m, d, cell) + double(offset);
    if (k.periodic)
    {
        const double L = k.up[d] - k.lo[d];
        if (x < k.lo[d])
            x += L;
        if (x > k.up[d])
            x -= L;
    }
    return x;
}

template <int D>
__global__ void k_mp_rehash(size_t n, const float4 *__restrict__ geo0, const float *__restrict__ off, MPConst k,
                            uint32_t *__restrict__ ncell, float *__restrict__ noff, uint32_t *__restrict__ key,
                            uint32_t *__restrict__ rank, uint32_t *__restrict__ count)
{
    size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    const MeshDev &m = k.m;
    int c0[3];
    unpack_cell<D>(__float_as_uint(geo0[i].w), c0);
    float o[3] = {0.f, 0.f, 0.f}, no[3];
#pragma unroll
    for (int d = 0; d < D; ++d)
        o[d] = off[d * n + i];
    int c[3] = {0, 0, 0};
    rehash_relative<D>(m, k.inv_gs, k.periodic != 0, c0, o, c, no);
#pragma unroll
    for (int d = 0; d < D; ++d)
        noff[d * n + i] = no[d];
    ncell[i] = pack_cell<D>(c);
    uint32_t lc = linear_cell<D>(m, c);
    key[i] = lc;
    rank[i] = atomicAdd(&count[lc], 1u);
}

__global__ void k_mp_scatter(size_t n, const uint32_t *__restrict__ key, const uint32_t *__restrict__ rank,
                             const uint32_t *__restrict__ offset, uint32_t *__restrict__ perm)
{
    size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i < n)
        perm[offset[key[i]] + rank[i]] = uint32_t(i);
}

__global__ void k_mp_sort_segments(size_t nseg, const uint32_t *__restrict__ offset, uint32_t *__restrict__ idx)
{
    size_t c = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (c >= nseg)
        return;
    uint32_t b = offset[c], e = offset[c + 1];
    for (uint32_t k = b + 1; k < e; ++k)
    {
        uint32_t v = idx[k];
        uint32_t q = k;
        while (q > b && idx[q - 1] > v)
        {
            idx[q] = idx[q - 1];
            --q;
        }
        idx[q] = v;
    }
}

__global__ void k_mp_set_total(uint32_t *offset, size_t ncells, uint32_t total) { offset[ncells] = total; }

// Gathers the state into the new cell order.
template <int D>
__global__ void k_mp_gather(size_t n, const uint32_t *__restrict__ perm, const uint32_t *__restrict__ ncell,
                            const float *__restrict__ noff, MPFluid src, MPFluid dst)
{
    size_t k = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (k >= n)
        return;
    uint32_t i = perm[k];
    float o[3] = {0.f, 0.f, 0.f};
#pragma unroll
    for (int d = 0; d < D; ++d)
    {
        o[d] = noff[d * n + i];
        dst.off[d * n + k] = o[d];
        dst.force[d * n + k] = src.force[d * n + i];
    }
    dst.geo0[k] = make_float4(o[0], o[1], o[2], __uint_as_float(ncell[i]));
    dst.dyn[k] = src.dyn[i];
    dst.drho[k] = src.drho[i];
    dst.drho_dt[k] = src.drho_dt[i];
    dst.id[k] = src.id[i];
    if (src.fprior)
#pragma unroll
        for (int d = 0; d < D; ++d)
            dst.fprior[d * n + k] = src.fprior[d * n + i];
}

// ---------------------------------------------------------------- configuration + density sums
template <int D>
__global__ void k_mp_build(size_t n, MPConst k, MPFluid f, const uint32_t *__restrict__ f_offset, MPWall w,
               const uint32_t *__restrict__ w_offset, MPLists in, MPLists wl, unsigned int *max_counts)
{
    size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i < n)
        build_particle<D>(i, n, k.p, Visit{k.m, 0u, f_offset, w_offset}, f, w, in, wl, max_counts);
}

template <int D>
__global__ void k_mp_build_periodic(size_t n, MPConst k, MPFluid f, const uint32_t *__restrict__ f_offset, MPLists in,
                                    unsigned int *max_counts)
{
    size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i < n)
        build_particle_periodic<D>(i, n, k.p, k.m, f_offset, f, in, max_counts);
}

// Start of a periodic-flow advection step: rho = rho_sum (DensitySummationInner) and the
// transport-velocity shift of the positions.
template <int D>
__global__ void k_mp_density_periodic(size_t n, MPFluid f)
{
    size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    f.drho[i] = f.drho_sum[i];
#pragma unroll
    for (int d = 0; d < D; ++d)
        f.off[d * n + i] = f.off[d * n + i] + f.shift[d * n + i];
}

// DensitySummation update with the FreeSurface rule rho = max(rho_sum, rho0), at the
// start of the advection step as in the reference loop.
__global__ void k_mp_density(size_t n, const float *__restrict__ drho_sum, float *__restrict__ drho)
{
    size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i < n)
        drho[i] = fmaxf(drho_sum[i], 0.0f);
}

// ---------------------------------------------------------------- acoustic sub-step
__global__ void k_mp_init1(size_t n, float *__restrict__ drho, const float *__restrict__ drho_dt,
                           float4 *__restrict__ dyn, float p0_over_rho0, float half_dt)
{
    size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    float r = drho[i] + drho_dt[i] * half_dt;
    drho[i] = r;
    reinterpret_cast<float *>(dyn)[4 * i + 3] = p0_over_rho0 * r;
}

// at most 64 registers: 4 blocks of 256 threads per SM
template <int D, bool LISTS>
__global__ void __launch_bounds__(256, 4) k_mp_first(size_t n, MPConst k, MPFluid f, const uint32_t *__restrict__ f_offset, MPWall w,
               const uint32_t *__restrict__ w_offset, MPLists in, MPLists wl, double dt,
               unsigned long long *ac_slot)
{
    size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    double vmax = -1.0e300;
    if (i < n)
        vmax = first_particle<D, LISTS>(i, n, k.p, Visit{k.m, 0u, f_offset, w_offset}, dt, f, w, in, wl);
    warp_max_to(ac_slot, vmax);
}

template <int D, bool LISTS>
__global__ void k_mp_second(size_t n, MPConst k, MPFluid f, const uint32_t *__restrict__ f_offset, MPWall w,
                const uint32_t *__restrict__ w_offset, MPLists in, MPLists wl, double dt,
                unsigned long long *adv_slot)
{
    size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    double amax = -1.0e300;
    if (i < n)
        amax = second_particle<D, LISTS>(i, n, k.p, Visit{k.m, 0u, f_offset, w_offset}, dt, f, w, in, wl);
    warp_max_to(adv_slot, amax);
}

template <int D, bool LISTS>
__global__ void __launch_bounds__(256, 4) k_mp_first_periodic(size_t n, MPConst k, MPFluid f,
                                                               const uint32_t *__restrict__ f_offset, MPLists in,
                                                               double dt, unsigned long long *ac_slot)
{
    size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    double vmax = -1.0e300;
    if (i < n)
        vmax = first_particle_periodic<D, LISTS>(i, n, k.p, k.m, f_offset, dt, f, in);
    warp_max_to(ac_slot, vmax);
}

template <int D, bool LISTS, bool RIEMANN>
__global__ void k_mp_second_periodic(size_t n, MPConst k, MPFluid f, const uint32_t *__restrict__ f_offset,
                                     MPLists in, double dt, unsigned long long *adv_slot)
{
    size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    double amax = -1.0e300;
    if (i < n)
        amax = second_particle_periodic<D, LISTS, RIEMANN>(i, n, k.p, k.m, f_offset, dt, f, in);
    warp_max_to(adv_slot, amax);
}

template <int D>
__global__ void k_mp_initial_max(size_t n, MPConst k, MPFluid f, unsigned long long *ac_slot,
                                 unsigned long long *adv_slot)
{
    size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    double am = -1.0e300, vm = -1.0e300;
    if (i < n)
        initial_max<D>(i, n, k.p, k.gd, f, &vm, &am);
    warp_max_to(ac_slot, vm);
    warp_max_to(adv_slot, am);
}

// ---------------------------------------------------------------- FP64 body -> FP32 state
struct ImportArgs
{
    const double *vel, *force, *rho, *drho_dt, *fprior;
    double rho0, c0_sqr;
};

template <int D>
__global__ void k_mp_import(size_t n, ImportArgs a, MPFluid f)
{
    size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    float v[3] = {0.f, 0.f, 0.f};
#pragma unroll
    for (int d = 0; d < D; ++d)
    {
        v[d] = a.vel ? float(a.vel[d * n + i]) : 0.f;
        f.force[d * n + i] = a.force ? float(a.force[d * n + i]) : 0.f;
        if (f.fprior)
            f.fprior[d * n + i] = a.fprior ? float(a.fprior[d * n + i]) : 0.f;
    }
    float dr = float(a.rho[i] - a.rho0);
    f.drho[i] = dr;
    f.drho_dt[i] = a.drho_dt ? float(a.drho_dt[i]) : 0.f;
    f.dyn[i] = make_float4(v[0], v[1], v[2], float(a.c0_sqr) * dr);
    f.id[i] = uint32_t(i);
}

// Host-row import straight into cell order (sphx_mp_upload_host).  Slot k holds body
// particle perm[k]: first its geometry from the hashed positions, then, once the other
// rows have arrived, its state with the conversions of k_mp_import.
template <int D>
__global__ void k_mp_place_geometry(size_t n, const uint32_t *__restrict__ perm, const uint32_t *__restrict__ ncell,
                                    const float *__restrict__ noff, MPFluid dst)
{
    size_t k = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (k >= n)
        return;
    uint32_t i = perm[k];
    float o[3] = {0.f, 0.f, 0.f};
#pragma unroll
    for (int d = 0; d < D; ++d)
    {
        o[d] = noff[d * n + i];
        dst.off[d * n + k] = o[d];
    }
    dst.geo0[k] = make_float4(o[0], o[1], o[2], __uint_as_float(ncell[i]));
}

template <int D>
__global__ void k_mp_place_state(size_t n, const uint32_t *__restrict__ perm, const double *__restrict__ vel,
                                 const double *__restrict__ force, const double *__restrict__ rho,
                                 const double *__restrict__ drho_dt, double rho0, double c0_sqr, MPFluid dst)
{
    size_t k = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (k >= n)
        return;
    uint32_t i = perm[k];
    float v[3] = {0.f, 0.f, 0.f};
#pragma unroll
    for (int d = 0; d < D; ++d)
    {
        v[d] = float(vel[size_t(i) * D + d]);
        dst.force[d * n + k] = float(force[size_t(i) * D + d]);
    }
    float dr = float(rho[i] - rho0);
    dst.drho[k] = dr;
    dst.drho_dt[k] = float(drho_dt[i]);
    dst.dyn[k] = make_float4(v[0], v[1], v[2], float(c0_sqr) * dr);
    dst.id[k] = i;
}

// ---------------------------------------------------------------- outputs
__device__ __forceinline__ double position(const MPConst &k, const MPFluid &f, size_t n, size_t i, int d, const int *c)
{
    return reconstruct(k, d, c[d], f.off[d * n + i]);
}

template <int D>
__global__ void k_mp_download(size_t n, MPConst k, MPFluid f, double *__restrict__ pos, double *__restrict__ vel,
                              double *__restrict__ rho, double *__restrict__ p, double *__restrict__ force,
                              double *__restrict__ drho_dt, double *__restrict__ fprior)
{
    size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    uint32_t o = f.id[i];
    int c[3];
    unpack_cell<D>(__float_as_uint(f.geo0[i].w), c);
    float4 di = f.dyn[i];
    const float v[3] = {di.x, di.y, di.z};
#pragma unroll
    for (int d = 0; d < D; ++d)
    {
        pos[d * n + o] = position(k, f, n, i, d, c);
        vel[d * n + o] = v[d];
        force[d * n + o] = f.force[d * n + i];
        if (fprior && f.fprior)
            fprior[d * n + o] = f.fprior[d * n + i];
    }
    rho[o] = double(k.p.rho0) + double(f.drho[i]);
    p[o] = di.w; // pressure of the last 1st-half initialisation, as the FP64 body holds it
    drho_dt[o] = f.drho_dt[i];
}

// Host-row export (sphx_mp_download_host): position, velocity, density and pressure rows
// in the body's particle order, the values k_mp_download writes.
template <int D>
__global__ void k_mp_export_rows(size_t n, MPConst k, MPFluid f, double *__restrict__ pos, double *__restrict__ vel,
                                 double *__restrict__ rho, double *__restrict__ p)
{
    size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    uint32_t o = f.id[i];
    int c[3];
    unpack_cell<D>(__float_as_uint(f.geo0[i].w), c);
    float4 di = f.dyn[i];
    const float v[3] = {di.x, di.y, di.z};
#pragma unroll
    for (int d = 0; d < D; ++d)
    {
        pos[size_t(o) * D + d] = position(k, f, n, i, d, c);
        vel[size_t(o) * D + d] = v[d];
    }
    rho[o] = double(k.p.rho0) + double(f.drho[i]);
    p[o] = di.w;
}

template <int D>
__global__ void k_mp_conservation(size_t n, MPConst k, MPFluid f, double *__restrict__ partials)
{
    double s[5] = {0, 0, 0, 0, 0};
    for (size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += size_t(gridDim.x) * blockDim.x)
    {
        int c[3];
        unpack_cell<D>(__float_as_uint(f.geo0[i].w), c);
        float4 di = f.dyn[i];
        const float vv[3] = {di.x, di.y, di.z};
        double m = k.p.mass, v2 = 0, gx = 0;
        s[0] += m;
#pragma unroll
        for (int d = 0; d < D; ++d)
        {
            double v = vv[d];
            s[1 + d] += m * v;
            v2 += v * v;
            gx += k.gd[d] * (-position(k, f, n, i, d, c));
        }
        s[4] += 0.5 * m * v2 + m * gx;
    }
    __shared__ double sm[5][256];
    for (int q = 0; q < 5; ++q)
        sm[q][threadIdx.x] = s[q];
    __syncthreads();
    for (unsigned o = blockDim.x / 2; o > 0; o >>= 1)
    {
        if (threadIdx.x < o)
            for (int q = 0; q < 5; ++q)
                sm[q][threadIdx.x] += sm[q][threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0)
        for (int q = 0; q < 5; ++q)
            partials[blockIdx.x * 5 + q] = sm[q][0];
}

template <int D>
__global__ void k_mp_upper_front(size_t n, MPConst k, MPFluid f, int axis, double l0, double l1, double l2,
                                 double u0, double u1, double u2, unsigned long long *slot)
{
    double lo[3] = {l0, l1, l2}, up[3] = {u0, u1, u2};
    double m = -1.0e300;
    for (size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += size_t(gridDim.x) * blockDim.x)
    {
        int c[3];
        unpack_cell<D>(__float_as_uint(f.geo0[i].w), c);
        double x[3];
        bool in = true;
#pragma unroll
        for (int d = 0; d < D; ++d)
        {
            x[d] = position(k, f, n, i, d, c);
            in = in && !(x[d] < lo[d] || x[d] > up[d]);
        }
        if (in)
            m = fmax(m, x[axis]);
    }
    warp_max_to(slot, m);
}

template <int D>
__global__ void k_wall_load(size_t nw, const uint32_t *__restrict__ perm, const double *__restrict__ pos,
                            const double *__restrict__ nrm, MeshDev m, float4 *__restrict__ geo,
                            float4 *__restrict__ n_out)
{
    size_t k = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (k >= nw)
        return;
    uint32_t i = perm[k];
    double x[3] = {0, 0, 0};
#pragma unroll
    for (int d = 0; d < D; ++d)
        x[d] = pos[d * nw + i];
    int c[3] = {0, 0, 0};
    cell_index<D>(m, x, c);
    float o[3] = {0.f, 0.f, 0.f}, nn[3] = {0.f, 0.f, 0.f};
#pragma unroll
    for (int d = 0; d < D; ++d)
    {
        o[d] = float(x[d] - cell_corner(m, d, c[d]));
        nn[d] = float(nrm[d * nw + i]);
    }
    geo[k] = make_float4(o[0], o[1], o[2], __uint_as_float(pack_cell<D>(c)));
    n_out[k] = make_float4(nn[0], nn[1], nn[2], 0.f);
}

template <int D>
__global__ void k_wall_hash(size_t nw, const double *__restrict__ pos, MeshDev m, uint32_t *__restrict__ key,
                            uint32_t *__restrict__ rank, uint32_t *__restrict__ count)
{
    size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= nw)
        return;
    double x[3] = {0, 0, 0};
#pragma unroll
    for (int d = 0; d < D; ++d)
        x[d] = pos[d * nw + i];
    int c[3] = {0, 0, 0};
    cell_index<D>(m, x, c);
    uint32_t lc = linear_cell<D>(m, c);
    key[i] = lc;
    rank[i] = atomicAdd(&count[lc], 1u);
}

template <typename T>
T *dalloc(size_t n)
{
    T *p = nullptr;
    if (cudaMalloc(&p, std::max<size_t>(n, 1) * sizeof(T)) != cudaSuccess)
        return nullptr;
    return p;
}
} // namespace

struct sphx_mp_s
{
    sphx_ctx ctx = nullptr;
    int dim = 3;
    size_t n = 0, nw = 0, ncells = 0;
    MPConst k{};
    MPFluid a{}, b{}; // current state and re-sort target
    MPWall w{};
    uint32_t *f_offset = nullptr, *w_offset = nullptr, *count = nullptr;
    uint32_t *key = nullptr, *rank = nullptr, *perm = nullptr, *ncell = nullptr;
    float *noff = nullptr;
    MPLists in{}, wl{};
    unsigned long long *slots = nullptr; // 0 acoustic, 1 advection, 2 misc, 3 build counts
    unsigned long long *h_slots = nullptr;
    double physical_time = 0, acoustic_dt = 0;
    // positions moved since the last configuration update: the re-hash, re-sort and list
    // build run at the start of the next advection step, so that a caller who replaces
    // the state between steps (sphx_mp_upload) pays for one configuration, not two
    bool moved = false;
    // host-row transfers (sphx_mp_upload_host / sphx_mp_download_host): device staging
    // rows, a side stream for the copies that overlap the configuration, two events
    double *stage = nullptr;
    cudaStream_t side = nullptr;
    cudaEvent_t ev_pos = nullptr, ev_rest = nullptr;
    int block = 128, strategy = 0;
    // optional CUDA-event timing of the two sweep kernels (sphx_mp_set_profiling)
    bool profiling = false;
    std::vector<cudaEvent_t> ev_first, ev_second; // start/stop pairs
    double ms_first = 0, ms_second = 0;
    long n_first = 0, n_second = 0;
    std::vector<void *> owned;
    template <typename T>
    T *alloc(size_t cnt)
    {
        T *p = dalloc<T>(cnt);
        if (p)
            owned.push_back(p);
        return p;
    }
};

namespace
{
// The periodic 2nd half with or without the Riemann dissipation (limiter slope 0 is the
// reference's NoRiemannSolver).
template <int D, bool LISTS>
void launch_second_periodic(sphx_mp_s *mp, unsigned blk, double dt)
{
    const size_t n = mp->n;
    cudaStream_t s = mp->ctx->stream;
    if (mp->k.p.s_lim != 0.0f)
        k_mp_second_periodic<D, LISTS, true><<<grid_for(n, blk), blk, 0, s>>>(n, mp->k, mp->a, mp->f_offset, mp->in,
                                                                             dt, mp->slots + 1);
    else
        k_mp_second_periodic<D, LISTS, false><<<grid_for(n, blk), blk, 0, s>>>(n, mp->k, mp->a, mp->f_offset,
                                                                              mp->in, dt, mp->slots + 1);
}

int alloc_state(sphx_mp mp, MPFluid &s)
{
    size_t n = mp->n, D = size_t(mp->dim);
    s.geo0 = mp->alloc<float4>(n);
    s.dyn = mp->alloc<float4>(n);
    s.off = mp->alloc<float>(D * n);
    s.force = mp->alloc<float>(D * n);
    s.drho = mp->alloc<float>(n);
    s.drho_dt = mp->alloc<float>(n);
    s.drho_sum = mp->alloc<float>(n);
    s.id = mp->alloc<uint32_t>(n);
    if (!s.geo0 || !s.dyn || !s.off || !s.force || !s.drho || !s.drho_dt || !s.drho_sum || !s.id)
        return fail(SPHX_ERR_OUT_OF_MEMORY, "mixed-precision state allocation failed");
    if (mp->k.periodic)
    {
        s.fprior = mp->alloc<float>(D * n);
        s.shift = mp->alloc<float>(D * n);
        if (!s.fprior || !s.shift)
            return fail(SPHX_ERR_OUT_OF_MEMORY, "mixed-precision state allocation failed");
    }
    return SPHX_OK;
}

int alloc_lists(sphx_mp mp, MPLists &l, unsigned cap)
{
    if (l.J)
    {
        cudaFree(l.J);
        mp->owned.erase(std::remove(mp->owned.begin(), mp->owned.end(), (void *)l.J), mp->owned.end());
    }
    l.J = mp->alloc<uint32_t>(size_t(cap) * std::max<size_t>(mp->n, 1));
    if (!l.J)
        return fail(SPHX_ERR_OUT_OF_MEMORY, "neighbour list allocation failed (%u slots)", cap);
    l.cap = cap;
    return SPHX_OK;
}

// Counting sort of mp->key[0..n) into mp->perm (stable), cell offsets into `offset`.
int sort_keys(sphx_mp mp, size_t n, uint32_t *offset)
{
    sphx_ctx ctx = mp->ctx;
    cudaStream_t s = ctx->stream;
    SPHX_TRY(exclusive_scan(ctx, mp->count, offset, mp->ncells));
    k_mp_set_total<<<1, 1, 0, s>>>(offset, mp->ncells, uint32_t(n));
    SPHX_LAUNCHED(ctx);
    if (n == 0)
        return SPHX_OK;
    k_mp_scatter<<<grid_for(n, 256), 256, 0, s>>>(n, mp->key, mp->rank, offset, mp->perm);
    SPHX_LAUNCHED(ctx);
    k_mp_sort_segments<<<grid_for(mp->ncells, 256), 256, 0, s>>>(mp->ncells, offset, mp->perm);
    SPHX_LAUNCHED(ctx);
    return SPHX_OK;
}

template <int D>
int launch_build(sphx_mp mp)
{
    sphx_ctx ctx = mp->ctx;
    cudaStream_t s = ctx->stream;
    unsigned int *mc = reinterpret_cast<unsigned int *>(mp->slots + 3);
    for (int attempt = 0; attempt < 2; ++attempt)
    {
        SPHX_CUDA(cudaMemsetAsync(mc, 0, 2 * sizeof(unsigned int), s));
        if (mp->k.periodic)
            k_mp_build_periodic<D><<<grid_for(mp->n, 256), 256, 0, s>>>(mp->n, mp->k, mp->a, mp->f_offset, mp->in, mc);
        else
            k_mp_build<D><<<grid_for(mp->n, 256), 256, 0, s>>>(mp->n, mp->k, mp->a, mp->f_offset, mp->w,
                                                              mp->w_offset, mp->in, mp->wl, mc);
        SPHX_LAUNCHED(ctx);
        SPHX_CUDA(cudaMemcpyAsync(mp->h_slots + 3, mc, 2 * sizeof(unsigned int), cudaMemcpyDeviceToHost, s));
        SPHX_CUDA(cudaStreamSynchronize(s));
        const unsigned int *h = reinterpret_cast<const unsigned int *>(mp->h_slots + 3);
        bool grow = false;
        if (h[0] > mp->in.cap)
        {
            SPHX_TRY(alloc_lists(mp, mp->in, h[0] + h[0] / 4 + 4));
            grow = true;
        }
        if (h[1] > mp->wl.cap)
        {
            SPHX_TRY(alloc_lists(mp, mp->wl, h[1] + h[1] / 4 + 4));
            grow = true;
        }
        if (!grow)
            return SPHX_OK;
    }
    return fail(SPHX_ERR_CAPACITY, "mixed-precision neighbour lists overflowed after growing");
}

template <int D>
int configuration_update(sphx_mp mp, bool from_state)
{
    sphx_ctx ctx = mp->ctx;
    cudaStream_t s = ctx->stream;
    size_t n = mp->n;
    if (from_state)
    {
        SPHX_CUDA(cudaMemsetAsync(mp->count, 0, mp->ncells * sizeof(uint32_t), s));
        if (n > 0)
        {
            k_mp_rehash<D><<<grid_for(n, 256), 256, 0, s>>>(n, mp->a.geo0, mp->a.off, mp->k, mp->ncell, mp->noff,
                                                            mp->key, mp->rank, mp->count);
            SPHX_LAUNCHED(ctx);
        }
    }
    SPHX_TRY(sort_keys(mp, n, mp->f_offset));
    if (n > 0)
    {
        k_mp_gather<D><<<grid_for(n, 256), 256, 0, s>>>(n, mp->perm, mp->ncell, mp->noff, mp->a, mp->b);
        SPHX_LAUNCHED(ctx);
        std::swap(mp->a, mp->b);
        SPHX_TRY(launch_build<D>(mp));
    }
    return SPHX_OK;
}

int read_slot(sphx_mp mp, int slot, double *out)
{
    SPHX_CUDA(cudaMemcpyAsync(mp->h_slots + slot, mp->slots + slot, sizeof(unsigned long long),
                              cudaMemcpyDeviceToHost, mp->ctx->stream));
    SPHX_CUDA(cudaStreamSynchronize(mp->ctx->stream));
    *out = from_ordered_bits(mp->h_slots[slot]);
    return SPHX_OK;
}

// The configuration update deferred from the end of the last advection step.
int settle_configuration(sphx_mp mp)
{
    if (mp->moved)
    {
        SPHX_TRY(mp->dim == 2 ? configuration_update<2>(mp, true) : configuration_update<3>(mp, true));
        mp->moved = false;
    }
    return SPHX_OK;
}

template <int D>
int substep(sphx_mp mp, double dt)
{
    sphx_ctx ctx = mp->ctx;
    cudaStream_t s = ctx->stream;
    size_t n = mp->n;
    if (n == 0)
        return SPHX_OK;
    unsigned blk = unsigned(mp->block);
    k_mp_init1<<<grid_for(n, 256), 256, 0, s>>>(n, mp->a.drho, mp->a.drho_dt, mp->a.dyn, mp->k.p.p0_over_rho0,
                                                float(0.5 * dt));
    SPHX_LAUNCHED(ctx);
    SPHX_CUDA(cudaMemsetAsync(mp->slots, 0, 2 * sizeof(unsigned long long), s));
    cudaEvent_t e[4] = {nullptr, nullptr, nullptr, nullptr};
    if (mp->profiling)
        for (int q = 0; q < 4; ++q)
        {
            SPHX_CUDA(cudaEventCreate(&e[q]));
            (q < 2 ? mp->ev_first : mp->ev_second).push_back(e[q]);
        }
    if (e[0])
        SPHX_CUDA(cudaEventRecord(e[0], s));
    if (mp->k.periodic)
    {
        if (mp->strategy == 0)
            k_mp_first_periodic<D, true><<<grid_for(n, blk), blk, 0, s>>>(n, mp->k, mp->a, mp->f_offset, mp->in, dt,
                                                                         mp->slots);
        else
            k_mp_first_periodic<D, false><<<grid_for(n, blk), blk, 0, s>>>(n, mp->k, mp->a, mp->f_offset, mp->in, dt,
                                                                          mp->slots);
    }
    else if (mp->strategy == 0)
        k_mp_first<D, true><<<grid_for(n, blk), blk, 0, s>>>(n, mp->k, mp->a, mp->f_offset, mp->w, mp->w_offset,
                                                            mp->in, mp->wl, dt, mp->slots);
    else
        k_mp_first<D, false><<<grid_for(n, blk), blk, 0, s>>>(n, mp->k, mp->a, mp->f_offset, mp->w, mp->w_offset,
                                                             mp->in, mp->wl, dt, mp->slots);
    SPHX_LAUNCHED(ctx);
    if (e[1])
        SPHX_CUDA(cudaEventRecord(e[1], s));
    if (e[2])
        SPHX_CUDA(cudaEventRecord(e[2], s));
    if (mp->k.periodic)
    {
        if (mp->strategy == 0)
            launch_second_periodic<D, true>(mp, blk, dt);
        else
            launch_second_periodic<D, false>(mp, blk, dt);
    }
    else if (mp->strategy == 0)
        k_mp_second<D, true><<<grid_for(n, blk), blk, 0, s>>>(n, mp->k, mp->a, mp->f_offset, mp->w, mp->w_offset,
                                                             mp->in, mp->wl, dt, mp->slots + 1);
    else
        k_mp_second<D, false><<<grid_for(n, blk), blk, 0, s>>>(n, mp->k, mp->a, mp->f_offset, mp->w,
                                                              mp->w_offset, mp->in, mp->wl, dt, mp->slots + 1);
    SPHX_LAUNCHED(ctx);
    if (e[3])
        SPHX_CUDA(cudaEventRecord(e[3], s));
    return SPHX_OK;
}

template <int D>
int advection_step(sphx_mp mp, int loop_style, int *substeps, double *adv_dt)
{
    SPHX_TRY(settle_configuration(mp));
    double adv_max;
    SPHX_TRY(read_slot(mp, 1, &adv_max));
    double Dt = mp->k.advection_cfl * mp->k.p.h / (std::max(std::sqrt(adv_max), mp->k.U_ref) + kTinyReal);
    if (mp->n > 0)
    {
        if (mp->k.periodic)
            k_mp_density_periodic<D><<<grid_for(mp->n, 256), 256, 0, mp->ctx->stream>>>(mp->n, mp->a);
        else
            k_mp_density<<<grid_for(mp->n, 256), 256, 0, mp->ctx->stream>>>(mp->n, mp->a.drho_sum, mp->a.drho);
        SPHX_LAUNCHED(mp->ctx);
    }
    double relaxation = 0, dt = mp->acoustic_dt;
    int count = 0;
    while (relaxation < Dt)
    {
        double ac;
        if (loop_style == 0) // AcousticTimeStep before the relaxation (Dambreak.cpp:184)
        {
            SPHX_TRY(read_slot(mp, 0, &ac));
            dt = mp->k.acoustic_cfl * mp->k.p.h / (ac + kTinyReal);
            if (mp->k.periodic) // dt = SMIN(acoustic dt, Dt) (taylor_green.cpp:146)
                dt = std::min(dt, Dt);
        }
        SPHX_TRY(substep<D>(mp, dt));
        if (loop_style == 1) // after it (test_3d_dambreak/dambreak.cpp:197)
        {
            SPHX_TRY(read_slot(mp, 0, &ac));
            dt = mp->k.acoustic_cfl * mp->k.p.h / (ac + kTinyReal);
        }
        relaxation += dt;
        mp->physical_time += dt;
        ++count;
    }
    mp->acoustic_dt = dt;
    mp->moved = true;
    if (substeps)
        *substeps = count;
    if (adv_dt)
        *adv_dt = Dt;
    return SPHX_OK;
}

// Folds the recorded event pairs into the running totals and frees the events.
void collect_events(sphx_mp mp)
{
    auto fold = [](std::vector<cudaEvent_t> &ev, double &ms, long &cnt) {
        for (size_t q = 0; q + 1 < ev.size(); q += 2)
        {
            float t = 0.f;
            if (cudaEventElapsedTime(&t, ev[q], ev[q + 1]) == cudaSuccess)
            {
                ms += t;
                ++cnt;
            }
            cudaEventDestroy(ev[q]);
            cudaEventDestroy(ev[q + 1]);
        }
        ev.clear();
    };
    fold(mp->ev_first, mp->ms_first, mp->n_first);
    fold(mp->ev_second, mp->ms_second, mp->n_second);
}
} // namespace

namespace
{
// Loads the FP64 fluid body's state (any particle order) into the solver, re-sorts it into
// cell order, rebuilds the neighbour lists and density sums, and primes the time-step
// maxima: the set-up of sphx_mp_create and sphx_mp_upload.
int import_fluid(sphx_mp mp, sphx_body fb, double rho0, double c0)
{
    const int D = mp->dim;
    const size_t n = mp->n;
    const size_t nc = mp->ncells;
    sphx_ctx ctx = mp->ctx;
    cudaStream_t s = ctx->stream;
    SPHX_CUDA(cudaStreamSynchronize(s));
    // fluid: FP64 body state -> FP32 (body order) in `a`, then the first configuration
    Field *pos = fb->find("Position"), *vel = fb->find("Velocity"), *force = fb->find("Force"),
          *rho = fb->find("Density"), *drho = fb->find("DensityChangeRate"), *fprior = fb->find("ForcePrior");
    if (!pos || !rho)
        return fail(SPHX_ERR_NOT_FOUND, "fluid Position / Density missing");
    if (n > 0)
    {
        ImportArgs ia{(const double *)(vel ? vel->dev : nullptr), (const double *)(force ? force->dev : nullptr),
                      (const double *)rho->dev, (const double *)(drho ? drho->dev : nullptr),
                      (const double *)(fprior && fprior->dtype == SPHX_F64 && fprior->ncomp == D ? fprior->dev
                                                                                                 : nullptr),
                      rho0, c0 * c0};
        if (D == 2)
            k_mp_import<2><<<grid_for(n, 256), 256, 0, s>>>(n, ia, mp->a);
        else
            k_mp_import<3><<<grid_for(n, 256), 256, 0, s>>>(n, ia, mp->a);
        SPHX_LAUNCHED(ctx);
    }
    // maxima for the first time steps, from the imported state (the configuration below
    // only reorders it, except for the prior force a periodic flow recomputes there)
    if (cudaMemsetAsync(mp->slots, 0, 2 * sizeof(unsigned long long), s) != cudaSuccess)
        return fail(SPHX_ERR_CUDA, "memset failed");
    if (n > 0)
    {
        if (D == 2)
            k_mp_initial_max<2><<<grid_for(n, 256), 256, 0, s>>>(n, mp->k, mp->a, mp->slots, mp->slots + 1);
        else
            k_mp_initial_max<3><<<grid_for(n, 256), 256, 0, s>>>(n, mp->k, mp->a, mp->slots, mp->slots + 1);
        ctx->launches++;
    }
    if (cudaMemsetAsync(mp->count, 0, nc * sizeof(uint32_t), s) != cudaSuccess)
        return fail(SPHX_ERR_CUDA, "memset failed");
    if (n > 0)
    {
        if (D == 2)
            k_mp_from_fp64<2><<<grid_for(n, 256), 256, 0, s>>>(n, (const double *)pos->dev, n, 1, mp->k, mp->ncell,
                                                               mp->noff, mp->key, mp->rank, mp->count);
        else
            k_mp_from_fp64<3><<<grid_for(n, 256), 256, 0, s>>>(n, (const double *)pos->dev, n, 1, mp->k, mp->ncell,
                                                               mp->noff, mp->key, mp->rank, mp->count);
        ctx->launches++;
    }
    SPHX_TRY(D == 2 ? configuration_update<2>(mp, false) : configuration_update<3>(mp, false));
    mp->moved = false;
    return SPHX_OK;
}
} // namespace

extern "C" int sphx_mp_create(sphx_relation inner, sphx_relation wall, const sphx_fluid_params *p,
                              const double *gravity, sphx_mp *out)
{
    if (!inner || !wall || !p || !gravity || !out || !inner->inner || wall->inner || wall->src != inner->src)
        return fail(SPHX_ERR_INVALID_ARG, "sphx_mp_create needs an inner and a wall contact relation of one fluid");
    sphx_body fb = inner->src, wb = wall->tgt;
    const int D = fb->dim;
    sphx_ctx ctx = fb->ctx;
    const sphx_mesh_desc &body_mesh = inner->cl->mesh;
    const sphx_mesh_desc mesh = sub_mesh(body_mesh);
    const int max_cells = D == 2 ? CellLanes<2>::max_cells : CellLanes<3>::max_cells;
    for (int a = 0; a < D; ++a)
        if (mesh.all_cells[a] > max_cells)
            return fail(SPHX_ERR_INVALID_ARG, "mixed precision packs %d bits per cell axis; axis %d has %d cells",
                        D == 2 ? CellLanes<2>::bits : CellLanes<3>::bits, a, mesh.all_cells[a]);
    if (std::abs(wall->cl->mesh.grid_spacing - body_mesh.grid_spacing) > 0 ||
        std::abs(2.0 * p->h - body_mesh.grid_spacing) > 1e-12 * body_mesh.grid_spacing)
        return fail(SPHX_ERR_INVALID_ARG, "mixed precision needs one mesh with grid spacing equal to the cut-off");
    // host checks of uniform mass / volume and a static wall (after the queued work)
    SPHX_CUDA(cudaStreamSynchronize(ctx->stream));
    auto host_copy = [&](sphx_body b, const char *name, std::vector<double> &v) -> int {
        Field *f = b->find(name);
        if (!f || f->dtype != SPHX_F64)
            return fail(SPHX_ERR_NOT_FOUND, "variable %s missing", name);
        v.resize(b->n * f->ncomp);
        if (!v.empty())
            SPHX_CUDA(cudaMemcpy(v.data(), f->dev, v.size() * sizeof(double), cudaMemcpyDeviceToHost));
        return SPHX_OK;
    };
    std::vector<double> mass, vol, wvol, wmass, wvel, wacc, fprior;
    SPHX_TRY(host_copy(fb, "Mass", mass));
    SPHX_TRY(host_copy(fb, "VolumetricMeasure", vol));
    SPHX_TRY(host_copy(wb, "VolumetricMeasure", wvol));
    SPHX_TRY(host_copy(wb, "Mass", wmass));
    auto uniform = [](const std::vector<double> &v) {
        for (double x : v)
            if (x != v[0])
                return false;
        return true;
    };
    if (mass.empty() || !uniform(mass) || !uniform(vol) || (!wvol.empty() && (!uniform(wvol) || !uniform(wmass))))
        return fail(SPHX_ERR_INVALID_ARG, "mixed precision needs uniform particle mass and volume");
    if (wb->find("Velocity") && host_copy(wb, "Velocity", wvel) == SPHX_OK)
        for (double x : wvel)
            if (x != 0.0)
                return fail(SPHX_ERR_INVALID_ARG, "mixed precision needs a static wall");
    if (wb->find("Acceleration") && host_copy(wb, "Acceleration", wacc) == SPHX_OK)
        for (double x : wacc)
            if (x != 0.0)
                return fail(SPHX_ERR_INVALID_ARG, "mixed precision needs a static wall");
    if (fb->find("ForcePrior") && host_copy(fb, "ForcePrior", fprior) == SPHX_OK)
        for (size_t i = 0; i < fb->n; ++i)
            for (int d = 0; d < D; ++d)
                if (std::abs(fprior[size_t(d) * fb->n + i] - mass[i] * gravity[d]) > 1e-11 * std::abs(mass[i]))
                    return fail(SPHX_ERR_INVALID_ARG, "mixed precision needs gravity as the only prior force");

    sphx_mp mp = new sphx_mp_s();
    mp->ctx = ctx;
    ctx->retain();
    mp->dim = D;
    mp->n = fb->n;
    mp->nw = wb->n;
    size_t nc = 1;
    for (int a = 0; a < D; ++a)
        nc *= size_t(mesh.all_cells[a]);
    mp->ncells = nc;
    MPConst &k = mp->k;
    k.m = mesh_dev(mesh);
    k.inv_gs = 1.0 / mesh.grid_spacing;
    double wm = wmass.empty() ? 0.0 : wmass[0];
    for (int d = 0; d < 3; ++d)
        k.gd[d] = d < D ? gravity[d] : 0.0;
    k.p = make_params(D, mesh.grid_spacing, p->h, p->rho0, p->c0, vol[0], mass[0], p->sigma0, wall->tgt_inv_rho0 * wm,
                      wvol.empty() ? 0.0 : wvol[0], p->limiter_slope, k.gd);
    k.acoustic_cfl = p->acoustic_cfl;
    k.advection_cfl = p->advection_cfl;
    k.U_ref = p->U_ref;

    int st = SPHX_OK;
    auto bail = [&](int code) {
        sphx_mp_destroy(mp);
        return code;
    };
    if ((st = alloc_state(mp, mp->a)) != SPHX_OK || (st = alloc_state(mp, mp->b)) != SPHX_OK)
        return bail(st);
    size_t n = mp->n, nw = mp->nw, big = std::max(n, nw);
    mp->f_offset = mp->alloc<uint32_t>(nc + 1);
    mp->w_offset = mp->alloc<uint32_t>(nc + 1);
    mp->count = mp->alloc<uint32_t>(nc);
    mp->key = mp->alloc<uint32_t>(big);
    mp->rank = mp->alloc<uint32_t>(big);
    mp->perm = mp->alloc<uint32_t>(big);
    mp->ncell = mp->alloc<uint32_t>(n);
    mp->noff = mp->alloc<float>(3 * n);
    mp->w.geo = mp->alloc<float4>(nw);
    mp->w.n = mp->alloc<float4>(nw);
    mp->w.nw = nw;
    mp->in.count = mp->alloc<uint32_t>(n);
    mp->wl.count = mp->alloc<uint32_t>(n);
    mp->slots = mp->alloc<unsigned long long>(8);
    if (!mp->f_offset || !mp->w_offset || !mp->count || !mp->key || !mp->rank || !mp->perm || !mp->ncell ||
        !mp->noff || !mp->w.geo || !mp->w.n || !mp->in.count || !mp->wl.count || !mp->slots)
        return bail(fail(SPHX_ERR_OUT_OF_MEMORY, "mixed-precision allocation failed"));
    if (cudaMallocHost(&mp->h_slots, 8 * sizeof(unsigned long long)) != cudaSuccess)
        return bail(fail(SPHX_ERR_OUT_OF_MEMORY, "pinned allocation failed"));
    if ((st = alloc_lists(mp, mp->in, D == 2 ? 24 : 96)) != SPHX_OK ||
        (st = alloc_lists(mp, mp->wl, D == 2 ? 16 : 64)) != SPHX_OK)
        return bail(st);

    cudaStream_t s = ctx->stream;
    MeshDev m = k.m;
    // wall: cell-sorted once (static)
    Field *wpos = wb->find("Position"), *wn = wb->find("NormalDirection");
    if (!wpos || !wn)
        return bail(fail(SPHX_ERR_NOT_FOUND, "wall Position / NormalDirection missing"));
    if (cudaMemsetAsync(mp->count, 0, nc * sizeof(uint32_t), s) != cudaSuccess)
        return bail(fail(SPHX_ERR_CUDA, "memset failed"));
    if (nw > 0)
    {
        if (D == 2)
            k_wall_hash<2><<<grid_for(nw, 256), 256, 0, s>>>(nw, (const double *)wpos->dev, m, mp->key, mp->rank,
                                                              mp->count);
        else
            k_wall_hash<3><<<grid_for(nw, 256), 256, 0, s>>>(nw, (const double *)wpos->dev, m, mp->key, mp->rank,
                                                              mp->count);
        ctx->launches++;
    }
    if ((st = sort_keys(mp, nw, mp->w_offset)) != SPHX_OK)
        return bail(st);
    if (nw > 0)
    {
        if (D == 2)
            k_wall_load<2><<<grid_for(nw, 256), 256, 0, s>>>(nw, mp->perm, (const double *)wpos->dev,
                                                              (const double *)wn->dev, m, mp->w.geo, mp->w.n);
        else
            k_wall_load<3><<<grid_for(nw, 256), 256, 0, s>>>(nw, mp->perm, (const double *)wpos->dev,
                                                              (const double *)wn->dev, m, mp->w.geo, mp->w.n);
        ctx->launches++;
    }
    if ((st = import_fluid(mp, fb, p->rho0, p->c0)) != SPHX_OK)
        return bail(st);
    if (cudaStreamSynchronize(s) != cudaSuccess || cudaGetLastError() != cudaSuccess)
        return bail(fail(SPHX_ERR_CUDA, "mixed-precision set-up failed"));
    *out = mp;
    return SPHX_OK;
}

// Periodic viscous flow without walls: the taylor_green.cpp step (DensitySummationInner,
// ViscousForceInner, TransportVelocityCorrectionInner, Integration1stHalfInnerRiemann,
// Integration2ndHalf with the given limiter slope -- 0 for NoRiemann --,
// AdvectionViscousTimeStep, dt = min(acoustic dt, Dt), PeriodicConditionUsingCellLinkedList
// along every axis) on the mixed-precision layout.  The box must be a cube; its sub-cells
// tile it exactly (N = floor(L / h) per axis, spacing L / N >= h).
extern "C" int sphx_mp_create_periodic(sphx_body fb, const sphx_fluid_params *p, const double *lower,
                                       const double *upper, double viscosity, double tvc_coefficient, sphx_mp *out)
{
    if (!fb || !p || !lower || !upper || !out || !(p->h > 0) || !(viscosity >= 0) || !(tvc_coefficient >= 0))
        return fail(SPHX_ERR_INVALID_ARG, "invalid periodic-flow arguments");
    const int D = fb->dim;
    sphx_ctx ctx = fb->ctx;
    const double L = upper[0] - lower[0];
    for (int a = 0; a < D; ++a)
        if (!(upper[a] - lower[a] > 0) || std::abs((upper[a] - lower[a]) - L) > 1e-12 * L)
            return fail(SPHX_ERR_INVALID_ARG, "the periodic box must be a cube");
    const int N = int(std::floor(L / p->h));
    const int max_cells = D == 2 ? CellLanes<2>::max_cells : CellLanes<3>::max_cells;
    if (N < 2 * kReach + 1 || N > max_cells)
        return fail(SPHX_ERR_INVALID_ARG, "periodic box of %d sub-cells per axis (needs %d..%d)", N, 2 * kReach + 1,
                    max_cells);
    if (fb->n > size_t(kIndexMask) + 1)
        return fail(SPHX_ERR_INVALID_ARG, "periodic lists index at most %u particles", kIndexMask + 1);
    SPHX_CUDA(cudaStreamSynchronize(ctx->stream));
    std::vector<double> mass, vol;
    for (auto nm : {"Mass", "VolumetricMeasure"})
    {
        Field *f = fb->find(nm);
        if (!f || f->dtype != SPHX_F64)
            return fail(SPHX_ERR_NOT_FOUND, "variable %s missing", nm);
        std::vector<double> &v = nm[0] == 'M' ? mass : vol;
        v.resize(fb->n);
        if (fb->n)
            SPHX_CUDA(cudaMemcpy(v.data(), f->dev, fb->n * sizeof(double), cudaMemcpyDeviceToHost));
    }
    for (size_t i = 0; i < fb->n; ++i)
        if (mass[i] != mass[0] || vol[i] != vol[0])
            return fail(SPHX_ERR_INVALID_ARG, "mixed precision needs uniform particle mass and volume");
    if (fb->n == 0)
        return fail(SPHX_ERR_INVALID_ARG, "empty fluid body");

    sphx_mesh_desc mesh{};
    mesh.dim = D;
    mesh.grid_spacing = L / N;
    for (int a = 0; a < D; ++a)
    {
        mesh.all_cells[a] = N;
        mesh.lower[a] = lower[a];
    }
    sphx_mp mp = new sphx_mp_s();
    mp->ctx = ctx;
    ctx->retain();
    mp->dim = D;
    mp->n = fb->n;
    mp->nw = 0;
    size_t nc = 1;
    for (int a = 0; a < D; ++a)
        nc *= size_t(N);
    mp->ncells = nc;
    MPConst &k = mp->k;
    k.m = mesh_dev(mesh);
    k.inv_gs = 1.0 / mesh.grid_spacing;
    k.periodic = 1;
    for (int d = 0; d < 3; ++d)
    {
        k.gd[d] = 0.0;
        k.lo[d] = d < D ? lower[d] : 0.0;
        k.up[d] = d < D ? upper[d] : 0.0;
    }
    k.p = make_params(D, mesh.grid_spacing, p->h, p->rho0, p->c0, vol[0], mass[0], p->sigma0, 0.0, 0.0,
                      p->limiter_slope, k.gd);
    for (int d = 0; d < 3; ++d)
        k.p.wrap[d] = d < D ? uint32_t(N) << (d * (D == 2 ? CellLanes<2>::bits : CellLanes<3>::bits)) : 0u;
    k.p.mu2 = float(2.0 * viscosity);
    k.p.eps_h = float(0.01 * p->h);
    k.p.tvc_scale = float(tvc_coefficient * p->h * p->h);
    k.p.tvc_lim = float(100.0 * p->h * p->h);
    k.acoustic_cfl = p->acoustic_cfl;
    k.advection_cfl = p->advection_cfl;
    // AdvectionViscousTimeStep: reference speed max(U_ref, mu / rho0 / h) (fluid_time_step.cpp:67-74)
    k.U_ref = std::max(p->U_ref, viscosity / p->rho0 / p->h);

    int st = SPHX_OK;
    auto bail = [&](int code) {
        sphx_mp_destroy(mp);
        return code;
    };
    if ((st = alloc_state(mp, mp->a)) != SPHX_OK || (st = alloc_state(mp, mp->b)) != SPHX_OK)
        return bail(st);
    size_t n = mp->n;
    mp->f_offset = mp->alloc<uint32_t>(nc + 1);
    mp->w_offset = mp->alloc<uint32_t>(1);
    mp->count = mp->alloc<uint32_t>(nc);
    mp->key = mp->alloc<uint32_t>(n);
    mp->rank = mp->alloc<uint32_t>(n);
    mp->perm = mp->alloc<uint32_t>(n);
    mp->ncell = mp->alloc<uint32_t>(n);
    mp->noff = mp->alloc<float>(3 * n);
    mp->in.count = mp->alloc<uint32_t>(n);
    mp->wl.count = mp->alloc<uint32_t>(n);
    mp->slots = mp->alloc<unsigned long long>(8);
    if (!mp->f_offset || !mp->w_offset || !mp->count || !mp->key || !mp->rank || !mp->perm || !mp->ncell ||
        !mp->noff || !mp->in.count || !mp->wl.count || !mp->slots)
        return bail(fail(SPHX_ERR_OUT_OF_MEMORY, "mixed-precision allocation failed"));
    if (cudaMallocHost(&mp->h_slots, 8 * sizeof(unsigned long long)) != cudaSuccess)
        return bail(fail(SPHX_ERR_OUT_OF_MEMORY, "pinned allocation failed"));
    if ((st = alloc_lists(mp, mp->in, D == 2 ? 24 : 96)) != SPHX_OK || (st = alloc_lists(mp, mp->wl, 1)) != SPHX_OK)
        return bail(st);
    if (cudaMemsetAsync(mp->wl.count, 0, n * sizeof(uint32_t), ctx->stream) != cudaSuccess ||
        cudaMemsetAsync(mp->w_offset, 0, sizeof(uint32_t), ctx->stream) != cudaSuccess)
        return bail(fail(SPHX_ERR_CUDA, "memset failed"));
    if ((st = import_fluid(mp, fb, p->rho0, p->c0)) != SPHX_OK)
        return bail(st);
    if (cudaStreamSynchronize(ctx->stream) != cudaSuccess || cudaGetLastError() != cudaSuccess)
        return bail(fail(SPHX_ERR_CUDA, "mixed-precision set-up failed"));
    *out = mp;
    return SPHX_OK;
}

namespace
{
// Staging rows (n x (3 D + 2) doubles, enough for either direction), the side stream and
// its events, created on first use.
int ensure_host_io(sphx_mp mp)
{
    if (!mp->stage)
    {
        mp->stage = mp->alloc<double>(mp->n * size_t(3 * mp->dim + 2));
        if (!mp->stage)
            return fail(SPHX_ERR_CUDA, "cannot allocate the host-transfer staging rows");
    }
    if (!mp->side)
        SPHX_CUDA(cudaStreamCreateWithFlags(&mp->side, cudaStreamNonBlocking));
    if (!mp->ev_pos)
        SPHX_CUDA(cudaEventCreateWithFlags(&mp->ev_pos, cudaEventDisableTiming));
    if (!mp->ev_rest)
        SPHX_CUDA(cudaEventCreateWithFlags(&mp->ev_rest, cudaEventDisableTiming));
    return SPHX_OK;
}

// sphx_mp_upload_host: the positions are copied first and hashed, sorted, placed and
// searched on the context's stream while the other rows copy on the side stream; the
// state is placed once they have arrived.  The same state as sphx_body_upload of each row
// followed by sphx_mp_upload.
template <int D>
int upload_host(sphx_mp mp, const double *pos, const double *vel, const double *force, const double *rho,
                const double *drho_dt)
{
    const size_t n = mp->n;
    sphx_ctx ctx = mp->ctx;
    cudaStream_t s = ctx->stream;
    SPHX_TRY(ensure_host_io(mp));
    SPHX_CUDA(cudaStreamSynchronize(s)); // the staging rows and the state are free
    double *spos = mp->stage, *svel = spos + n * D, *sforce = svel + n * D, *srho = sforce + n * D,
           *sdrho = srho + n;
    const size_t vec = n * D * sizeof(double), sca = n * sizeof(double);
    if (n > 0)
    {
        SPHX_CUDA(cudaMemcpyAsync(spos, pos, vec, cudaMemcpyHostToDevice, s));
        SPHX_CUDA(cudaEventRecord(mp->ev_pos, s));
        SPHX_CUDA(cudaStreamWaitEvent(mp->side, mp->ev_pos, 0));
        SPHX_CUDA(cudaMemcpyAsync(svel, vel, vec, cudaMemcpyHostToDevice, mp->side));
        SPHX_CUDA(cudaMemcpyAsync(sforce, force, vec, cudaMemcpyHostToDevice, mp->side));
        SPHX_CUDA(cudaMemcpyAsync(srho, rho, sca, cudaMemcpyHostToDevice, mp->side));
        SPHX_CUDA(cudaMemcpyAsync(sdrho, drho_dt, sca, cudaMemcpyHostToDevice, mp->side));
        SPHX_CUDA(cudaEventRecord(mp->ev_rest, mp->side));
    }
    SPHX_CUDA(cudaMemsetAsync(mp->count, 0, mp->ncells * sizeof(uint32_t), s));
    if (n > 0)
    {
        k_mp_from_fp64<D><<<grid_for(n, 256), 256, 0, s>>>(n, spos, 1, D, mp->k, mp->ncell, mp->noff, mp->key,
                                                           mp->rank, mp->count);
        SPHX_LAUNCHED(ctx);
    }
    SPHX_TRY(sort_keys(mp, n, mp->f_offset));
    if (n > 0)
    {
        k_mp_place_geometry<D><<<grid_for(n, 256), 256, 0, s>>>(n, mp->perm, mp->ncell, mp->noff, mp->b);
        SPHX_LAUNCHED(ctx);
    }
    std::swap(mp->a, mp->b);
    if (n > 0)
    {
        SPHX_TRY(launch_build<D>(mp)); // reads the geometry only
        SPHX_CUDA(cudaStreamWaitEvent(s, mp->ev_rest, 0));
        k_mp_place_state<D><<<grid_for(n, 256), 256, 0, s>>>(n, mp->perm, svel, sforce, srho, sdrho,
                                                             double(mp->k.p.rho0), mp->k.p.c0 * mp->k.p.c0, mp->a);
        SPHX_LAUNCHED(ctx);
    }
    // maxima for the first time steps, from the loaded state
    SPHX_CUDA(cudaMemsetAsync(mp->slots, 0, 2 * sizeof(unsigned long long), s));
    if (n > 0)
    {
        k_mp_initial_max<D><<<grid_for(n, 256), 256, 0, s>>>(n, mp->k, mp->a, mp->slots, mp->slots + 1);
        SPHX_LAUNCHED(ctx);
    }
    mp->moved = false;
    SPHX_CUDA(cudaStreamSynchronize(s));
    return SPHX_OK;
}

template <int D>
int download_host(sphx_mp mp, double *pos, double *vel, double *rho, double *p)
{
    const size_t n = mp->n;
    cudaStream_t s = mp->ctx->stream;
    SPHX_TRY(ensure_host_io(mp));
    double *spos = mp->stage, *svel = spos + n * D, *srho = svel + n * D, *sp = srho + n;
    if (n > 0)
    {
        k_mp_export_rows<D><<<grid_for(n, 256), 256, 0, s>>>(n, mp->k, mp->a, spos, svel, srho, sp);
        SPHX_LAUNCHED(mp->ctx);
        const size_t vec = n * D * sizeof(double), sca = n * sizeof(double);
        SPHX_CUDA(cudaMemcpyAsync(pos, spos, vec, cudaMemcpyDeviceToHost, s));
        SPHX_CUDA(cudaMemcpyAsync(vel, svel, vec, cudaMemcpyDeviceToHost, s));
        SPHX_CUDA(cudaMemcpyAsync(rho, srho, sca, cudaMemcpyDeviceToHost, s));
        SPHX_CUDA(cudaMemcpyAsync(p, sp, sca, cudaMemcpyDeviceToHost, s));
    }
    SPHX_CUDA(cudaStreamSynchronize(s));
    return SPHX_OK;
}
} // namespace

extern "C" int sphx_mp_upload_host(sphx_mp mp, const double *position, const double *velocity, const double *force,
                                   const double *density, const double *density_change_rate)
{
    if (!mp || (mp->n > 0 && (!position || !velocity || !force || !density || !density_change_rate)))
        return fail(SPHX_ERR_INVALID_ARG, "sphx_mp_upload_host needs the five host rows");
    if (mp->k.periodic)
        return fail(SPHX_ERR_INVALID_ARG, "a periodic solver loads its state through sphx_mp_upload");
    return mp->dim == 2 ? upload_host<2>(mp, position, velocity, force, density, density_change_rate)
                        : upload_host<3>(mp, position, velocity, force, density, density_change_rate);
}

extern "C" int sphx_mp_download_host(sphx_mp mp, double *position, double *velocity, double *density,
                                     double *pressure)
{
    if (!mp || (mp->n > 0 && (!position || !velocity || !density || !pressure)))
        return fail(SPHX_ERR_INVALID_ARG, "sphx_mp_download_host needs the four host rows");
    return mp->dim == 2 ? download_host<2>(mp, position, velocity, density, pressure)
                        : download_host<3>(mp, position, velocity, density, pressure);
}

extern "C" int sphx_mp_upload(sphx_mp mp, sphx_body fb)
{
    if (!mp || !fb || fb->n != mp->n || fb->dim != mp->dim)
        return fail(SPHX_ERR_INVALID_ARG, "body does not match the mixed-precision solver");
    double rho0 = double(mp->k.p.rho0), c0 = mp->k.p.c0;
    SPHX_TRY(import_fluid(mp, fb, rho0, c0));
    SPHX_CUDA(cudaStreamSynchronize(mp->ctx->stream));
    return SPHX_OK;
}

extern "C" int sphx_mp_set_profiling(sphx_mp mp, int on)
{
    if (!mp)
        return fail(SPHX_ERR_INVALID_ARG, "null solver");
    SPHX_CUDA(cudaStreamSynchronize(mp->ctx->stream));
    collect_events(mp);
    mp->profiling = on != 0;
    mp->ms_first = mp->ms_second = 0;
    mp->n_first = mp->n_second = 0;
    return SPHX_OK;
}

extern "C" int sphx_mp_kernel_times(sphx_mp mp, double *out)
{
    if (!mp || !out)
        return fail(SPHX_ERR_INVALID_ARG, "null argument");
    SPHX_CUDA(cudaStreamSynchronize(mp->ctx->stream));
    collect_events(mp);
    out[0] = mp->ms_first;
    out[1] = double(mp->n_first);
    out[2] = mp->ms_second;
    out[3] = double(mp->n_second);
    return SPHX_OK;
}

extern "C" int sphx_mp_list_sizes(sphx_mp mp, uint64_t *out)
{
    if (!mp || !out)
        return fail(SPHX_ERR_INVALID_ARG, "null argument");
    SPHX_TRY(settle_configuration(mp));
    size_t n = mp->n;
    std::vector<uint32_t> a(n), b(n);
    if (n)
    {
        SPHX_CUDA(cudaMemcpyAsync(a.data(), mp->in.count, n * 4, cudaMemcpyDeviceToHost, mp->ctx->stream));
        SPHX_CUDA(cudaMemcpyAsync(b.data(), mp->wl.count, n * 4, cudaMemcpyDeviceToHost, mp->ctx->stream));
    }
    SPHX_CUDA(cudaStreamSynchronize(mp->ctx->stream));
    uint64_t si = 0, sw = 0;
    for (size_t i = 0; i < n; ++i)
    {
        si += a[i];
        sw += b[i];
    }
    out[0] = mp->n;
    out[1] = mp->nw;
    out[2] = si;
    out[3] = sw;
    out[4] = mp->in.cap;
    out[5] = mp->wl.cap;
    return SPHX_OK;
}

extern "C" int sphx_mp_destroy(sphx_mp mp)
{
    if (!mp)
        return SPHX_OK;
    sphx_ctx ctx = mp->ctx;
    cudaStreamSynchronize(ctx->stream);
    collect_events(mp);
    if (mp->side)
    {
        cudaStreamSynchronize(mp->side);
        cudaStreamDestroy(mp->side);
    }
    if (mp->ev_pos)
        cudaEventDestroy(mp->ev_pos);
    if (mp->ev_rest)
        cudaEventDestroy(mp->ev_rest);
    for (void *p : mp->owned)
        cudaFree(p);
    if (mp->h_slots)
        cudaFreeHost(mp->h_slots);
    delete mp;
    release(ctx);
    return SPHX_OK;
}

namespace
{
// Snapshot of the variables a sub-step modifies (the configuration is untouched).
struct Snapshot
{
    std::vector<void *> bufs;
    int take(sphx_mp mp, bool restore)
    {
        size_t n = mp->n, D = size_t(mp->dim);
        void *src[6] = {mp->a.dyn, mp->a.off, mp->a.force, mp->a.drho, mp->a.drho_dt, mp->slots};
        size_t bytes[6] = {n * sizeof(float4), D * n * 4, D * n * 4, n * 4, n * 4, 2 * sizeof(unsigned long long)};
        if (!restore)
        {
            bufs.assign(6, nullptr);
            for (int q = 0; q < 6; ++q)
                SPHX_CUDA(cudaMallocAsync(&bufs[q], std::max<size_t>(bytes[q], 1), mp->ctx->stream));
        }
        for (int q = 0; q < 6; ++q)
        {
            void *dst = restore ? src[q] : bufs[q];
            const void *from = restore ? bufs[q] : src[q];
            SPHX_CUDA(cudaMemcpyAsync(dst, from, bytes[q], cudaMemcpyDeviceToDevice, mp->ctx->stream));
        }
        return SPHX_OK;
    }
    void release(sphx_mp mp)
    {
        for (void *b : bufs)
            if (b)
                cudaFreeAsync(b, mp->ctx->stream);
        bufs.clear();
    }
};
} // namespace

extern "C" int sphx_mp_autotune(sphx_mp mp, int reps, int *best_block, int *best_strategy, double *best_ms)
{
    if (!mp || reps < 1)
        return fail(SPHX_ERR_INVALID_ARG, "invalid autotune arguments");
    if (mp->n == 0)
        return SPHX_OK;
    SPHX_TRY(settle_configuration(mp));
    double ac;
    SPHX_TRY(read_slot(mp, 0, &ac));
    double dt = mp->k.acoustic_cfl * mp->k.p.h / (ac + kTinyReal);
    Snapshot snap;
    SPHX_TRY(snap.take(mp, false));
    const int blocks[3] = {64, 128, 256};
    int keep_block = mp->block, keep_strategy = mp->strategy;
    bool keep_prof = mp->profiling;
    double best = 1e300;
    int bb = keep_block, bs = keep_strategy;
    cudaEvent_t e0, e1;
    SPHX_CUDA(cudaEventCreate(&e0));
    SPHX_CUDA(cudaEventCreate(&e1));
    int st = SPHX_OK;
    mp->profiling = false;
    for (int strategy = 0; strategy < 2 && st == SPHX_OK; ++strategy)
        for (int bi = 0; bi < 3 && st == SPHX_OK; ++bi)
        {
            mp->block = blocks[bi];
            mp->strategy = strategy;
            if ((st = snap.take(mp, true)) != SPHX_OK)
                break;
            if ((st = (mp->dim == 2 ? substep<2>(mp, dt) : substep<3>(mp, dt))) != SPHX_OK) // warm-up
                break;
            cudaEventRecord(e0, mp->ctx->stream);
            for (int r = 0; r < reps && st == SPHX_OK; ++r)
                st = mp->dim == 2 ? substep<2>(mp, dt) : substep<3>(mp, dt);
            cudaEventRecord(e1, mp->ctx->stream);
            if (cudaEventSynchronize(e1) != cudaSuccess)
                st = fail(SPHX_ERR_CUDA, "autotune timing failed");
            float ms = 0;
            cudaEventElapsedTime(&ms, e0, e1);
            if (st == SPHX_OK && ms / reps < best)
            {
                best = ms / reps;
                bb = blocks[bi];
                bs = strategy;
            }
        }
    int st2 = snap.take(mp, true);
    snap.release(mp);
    cudaStreamSynchronize(mp->ctx->stream);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    mp->profiling = keep_prof;
    if (st != SPHX_OK || st2 != SPHX_OK)
    {
        mp->block = keep_block;
        mp->strategy = keep_strategy;
        return st != SPHX_OK ? st : st2;
    }
    mp->block = bb;
    mp->strategy = bs;
    if (best_block)
        *best_block = bb;
    if (best_strategy)
        *best_strategy = bs;
    if (best_ms)
        *best_ms = best;
    return SPHX_OK;
}

extern "C" int sphx_mp_set_tuning(sphx_mp mp, int block, int strategy)
{
    if (!mp || block < 64 || block > 256 || block % 32 != 0 || strategy < 0 || strategy > 1)
        return fail(SPHX_ERR_INVALID_ARG, "block must be 64..256 in steps of 32, strategy 0 or 1");
    mp->block = block;
    mp->strategy = strategy;
    return SPHX_OK;
}

extern "C" int sphx_mp_advection_step(sphx_mp mp, int loop_style, int *substeps, double *advection_dt,
                                      double *physical_time)
{
    if (!mp || (loop_style != 0 && loop_style != 1))
        return fail(SPHX_ERR_INVALID_ARG, "invalid advection-step arguments");
    SPHX_TRY(mp->dim == 2 ? advection_step<2>(mp, loop_style, substeps, advection_dt)
                          : advection_step<3>(mp, loop_style, substeps, advection_dt));
    if (physical_time)
        *physical_time = mp->physical_time;
    return SPHX_OK;
}

extern "C" int sphx_mp_download(sphx_mp mp, sphx_body fb)
{
    if (!mp || !fb || fb->n != mp->n || fb->dim != mp->dim)
        return fail(SPHX_ERR_INVALID_ARG, "body does not match the mixed-precision solver");
    int D = mp->dim;
    Field *pos, *vel, *rho, *p, *force, *drho;
    SPHX_TRY(fb->require("Position", SPHX_F64, D, &pos));
    SPHX_TRY(fb->require("Velocity", SPHX_F64, D, &vel));
    SPHX_TRY(fb->require("Density", SPHX_F64, 1, &rho));
    SPHX_TRY(fb->require("Pressure", SPHX_F64, 1, &p));
    SPHX_TRY(fb->require("Force", SPHX_F64, D, &force));
    SPHX_TRY(fb->require("DensityChangeRate", SPHX_F64, 1, &drho));
    Field *fp = nullptr;
    if (mp->k.periodic)
        SPHX_TRY(fb->require("ForcePrior", SPHX_F64, D, &fp));
    double *fprior = fp ? static_cast<double *>(fp->dev) : nullptr;
    size_t n = mp->n;
    if (n > 0)
    {
        if (D == 2)
            k_mp_download<2><<<grid_for(n, 256), 256, 0, mp->ctx->stream>>>(
                n, mp->k, mp->a, (double *)pos->dev, (double *)vel->dev, (double *)rho->dev, (double *)p->dev,
                (double *)force->dev, (double *)drho->dev, fprior);
        else
            k_mp_download<3><<<grid_for(n, 256), 256, 0, mp->ctx->stream>>>(
                n, mp->k, mp->a, (double *)pos->dev, (double *)vel->dev, (double *)rho->dev, (double *)p->dev,
                (double *)force->dev, (double *)drho->dev, fprior);
        SPHX_LAUNCHED(mp->ctx);
    }
    SPHX_CUDA(cudaStreamSynchronize(mp->ctx->stream));
    return SPHX_OK;
}

extern "C" int sphx_mp_conservation(sphx_mp mp, double *out)
{
    if (!mp || !out)
        return fail(SPHX_ERR_INVALID_ARG, "null argument");
    sphx_ctx ctx = mp->ctx;
    unsigned np = unsigned(std::max(1, std::min(ctx->num_sms * 4, int(grid_for(std::max<size_t>(mp->n, 1), 256)))));
    SPHX_TRY(ctx->ensure_scratch(size_t(np) * 5 * sizeof(double)));
    double *part = static_cast<double *>(ctx->d_scratch);
    if (mp->dim == 2)
        k_mp_conservation<2><<<np, 256, 0, ctx->stream>>>(mp->n, mp->k, mp->a, part);
    else
        k_mp_conservation<3><<<np, 256, 0, ctx->stream>>>(mp->n, mp->k, mp->a, part);
    SPHX_LAUNCHED(ctx);
    std::vector<double> h(size_t(np) * 5);
    SPHX_CUDA(cudaMemcpyAsync(h.data(), part, h.size() * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    SPHX_CUDA(cudaStreamSynchronize(ctx->stream));
    for (int q = 0; q < 5; ++q)
    {
        double s = 0;
        for (unsigned b = 0; b < np; ++b)
            s += h[b * 5 + q];
        out[q] = s;
    }
    return SPHX_OK;
}

extern "C" int sphx_mp_upper_front(sphx_mp mp, int axis, const double *lo, const double *up, double *front)
{
    if (!mp || !lo || !up || !front || axis < 0 || axis >= mp->dim)
        return fail(SPHX_ERR_INVALID_ARG, "invalid upper-front arguments");
    sphx_ctx ctx = mp->ctx;
    SPHX_CUDA(cudaMemsetAsync(mp->slots + 2, 0, sizeof(unsigned long long), ctx->stream));
    unsigned g = unsigned(std::max(1, std::min(ctx->num_sms * 4, int(grid_for(std::max<size_t>(mp->n, 1), 256)))));
    double l2 = mp->dim == 3 ? lo[2] : 0.0, u2 = mp->dim == 3 ? up[2] : 0.0;
    if (mp->dim == 2)
        k_mp_upper_front<2><<<g, 256, 0, ctx->stream>>>(mp->n, mp->k, mp->a, axis, lo[0], lo[1], l2, up[0], up[1], u2,
                                                        mp->slots + 2);
    else
        k_mp_upper_front<3><<<g, 256, 0, ctx->stream>>>(mp->n, mp->k, mp->a, axis, lo[0], lo[1], l2, up[0], up[1], u2,
                                                        mp->slots + 2);
    SPHX_LAUNCHED(ctx);
    return read_slot(mp, 2, front);
}
