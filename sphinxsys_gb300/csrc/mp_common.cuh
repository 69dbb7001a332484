// Per-particle physics of the mixed-precision solvers, shared by the single-case solver
// (mixed.cu) and the batched solver (batch.cu) so both run the same arithmetic.
//
// The sweeps follow Integration1stHalfWithWallRiemann / Integration2ndHalfWithWallRiemann
// (fluid_integration.hpp:49-113,166-231) with the AcousticRiemannSolver and the
// TruncatedLinear limiter (riemann_solver.h), the wall terms of fluid_integration.hpp
// (static wall: zero wall velocity and acceleration), and the configuration build with
// the sums of DensitySummationComplexFreeSurface (density_summation.cpp:74-82,124-144).
//
// Precision: FP32 pair arithmetic; neighbour sums are compensated (plain FP32 partials over
// groups of kGroup neighbours, Kahan-added); positions are FP32 offsets from the lower
// corner of an integer sub-cell; position half-steps and the time-step maxima are FP64.
#pragma once

#include "sphx_device.cuh"
#include "sphx_internal.cuh"

namespace sphx
{
namespace mpc
{
constexpr float kTinyF = 2.71051e-20f; // TinyReal of the reference, base_data_type.h:207
constexpr int kGroup = 8;             // neighbours per plain partial sum
// neighbour records in flight per thread in the list sweeps: the 1st half's records are
// small (geo0 + pressure), the 2nd half's carry the velocity and use more registers
// (measured: 8 / 4 is 8% faster in the 1st half than 4 / 4 and 7% faster in the 2nd half
// than 8 / 8, 3D dam break dp = 0.006)
#ifndef SPHX_UNROLL_FIRST
#define SPHX_UNROLL_FIRST 8
#endif
#ifndef SPHX_UNROLL_SECOND
#define SPHX_UNROLL_SECOND 4
#endif
constexpr int kUnrollFirst = SPHX_UNROLL_FIRST, kUnrollSecond = SPHX_UNROLL_SECOND;
// the 2nd half's list entries loaded one batch ahead (see list_sweep)
#ifndef SPHX_PREFETCH_SECOND
#define SPHX_PREFETCH_SECOND 0
#endif
constexpr bool kPrefetchSecond = SPHX_PREFETCH_SECOND != 0;
constexpr int kCellBias = 4;          // |c_i - c_j| per axis handled by the packed difference
constexpr int kReach = 2;             // neighbour search reach in sub-cells (cut-off = 2 sub-cells)

// The solvers order and search particles on sub-cells of half the cell-linked-list spacing
// (spacing h for the cut-off 2h): the 5^D sub-cells around a particle hold about 42%
// fewer candidates than the 3^D cells of spacing 2h in 3D (31% in 2D).
inline sphx_mesh_desc sub_mesh(const sphx_mesh_desc &m)
{
    sphx_mesh_desc s = m;
    s.grid_spacing = 0.5 * m.grid_spacing;
    for (int a = 0; a < m.dim; ++a)
        s.all_cells[a] = 2 * m.all_cells[a];
    return s;
}

// Cell coordinates packed into 30 bits: 15 per axis in 2D, 10 per axis in 3D.
template <int D>
struct CellLanes
{
    static constexpr int bits = D == 2 ? 15 : 10;
    static constexpr uint32_t mask = (1u << bits) - 1u;
    static constexpr int max_cells = 1 << bits;
    static constexpr uint32_t bias = D == 2 ? (uint32_t(kCellBias) | (uint32_t(kCellBias) << 15))
                                            : (uint32_t(kCellBias) | (uint32_t(kCellBias) << 10) |
                                               (uint32_t(kCellBias) << 20));
};

// Sub-cell of a position for the mixed solvers: floor((x - lower) * (1 / gs)) clamped as
// cell_index clamps.  The product replaces cell_index's FP64 division (three divisions per
// particle were most of the re-hash on the slow FP64 pipe); a position within rounding of
// a cell face may land in the neighbouring cell, whose offset then lies within rounding of
// 0 or gs, which the search reach covers.
template <int D>
__device__ __forceinline__ void sub_cell_index(const MeshDev &m, double inv_gs, const double *x, int *c)
{
#pragma unroll
    for (int a = 0; a < D; ++a)
    {
        double f = floor((x[a] - m.lower[a]) * inv_gs);
        c[a] = f < 0.0 ? 0 : (f > double(m.grid_points[a] - 2) ? m.grid_points[a] - 2 : int(f));
    }
}

// New (cell, offset) of a particle that moved by its FP64 offset from the corner of cell c0
// (the offset may lie outside that cell): k = floor(offset / gs) cells along each axis,
// then the offset re-based to the new cell in FP64.  A periodic
// box wraps the cell over its all_cells cells (the position moves by one period, the offset
// stays); otherwise the cell is clamped to the mesh as sub_cell_index does.  In exact
// arithmetic this equals the re-hash of the absolute position (corner + offset) with half
// its FP64 operations, which run at 1/64 of the FP32 rate on GB300.
template <int D>
__device__ __forceinline__ void rehash_relative(const MeshDev &m, double inv_gs, bool periodic, const int *c0,
                                                const double *offset, int *c, double *noff)
{
#pragma unroll
    for (int a = 0; a < D; ++a)
    {
        const double o = offset[a];
        const int k = int(floor(o * inv_gs));
        const int ncell = m.all_cells[a];
        int ca = c0[a] + k, shift = k;
        if (periodic)
            ca = ca < 0 ? ca + ncell : (ca >= ncell ? ca - ncell : ca);
        else
        {
            ca = ca < 0 ? 0 : (ca > ncell - 1 ? ncell - 1 : ca);
            shift = ca - c0[a];
        }
        c[a] = ca;
        noff[a] = o - double(shift) * m.gs;
    }
}

template <int D>
__host__ __device__ __forceinline__ uint32_t pack_cell(const int *c)
{
    uint32_t p = 0;
    for (int d = 0; d < D; ++d)
        p |= uint32_t(c[d]) << (d * CellLanes<D>::bits);
    return p;
}
template <int D>
__host__ __device__ __forceinline__ void unpack_cell(uint32_t p, int *c)
{
    c[0] = c[1] = c[2] = 0;
    for (int d = 0; d < D; ++d)
        c[d] = int((p >> (d * CellLanes<D>::bits)) & CellLanes<D>::mask);
}

// Tile-grouped traversal of the sweeps: the sub-cells are grouped in boxes of t[0] x t[1]
// (x t[2]) sub-cells and the particles of one box are handed to consecutive threads, so a
// block's neighbour records span a compact window that stays in L1 instead of the long
// column a run of consecutive particles spans in the linear cell order.  The particle
// order, the neighbour lists and the arithmetic are unchanged: only which thread handles
// which particle.  nt[d] = boxes along axis d; t[0] == 0 turns the grouping off.
struct TileShape
{
    int t[3], nt[3];
};

template <int D>
__device__ __forceinline__ uint32_t tile_key(const TileShape &ts, const int *c)
{
    uint32_t k = 0;
#pragma unroll
    for (int d = 0; d < D; ++d)
        k = k * uint32_t(ts.nt[d]) + uint32_t(c[d] / ts.t[d]);
    return k;
}

struct MPParams
{
    float gs_f, rc_sqr, inv_h, fW;
    float rc_reach; // search reach: cut-off x (1 + 1e-4)
    float cW, cWw; // Wendland dW prefactor x 5/8 x particle volume (fluid, wall)
    float rho0, p0_over_rho0, Vol, mass, inv_mass;
    float rho0_over_sigma0, wall_factor; // wall_factor = rho0^2 m_w / (sigma0 m rho0_w)
    float inv_z, zgeo, s_lim;            // acoustic Riemann solver; s_lim = limiter slope / c0
    float g[3];
    double sigma0, c0, h;
    // periodic flow (sphx_mp_create_periodic): wrap[d] = cells along axis d shifted into
    // lane d (one period); 2 mu; 0.01 h; transport-velocity scaling and limiter factor
    uint32_t wrap[3];
    float mu2, eps_h, tvc_scale, tvc_lim;
};

// The reference's lattice number density (computeLatticeNumberDensity, adaptation.cpp:25-58:
// W summed over the lattice points i dp closer than the cut-off) evaluated with this
// solver's FP32 kernel, i.e. the arithmetic of wc2_W on the rounded constants fW and 1 / h
// and the squared distance as the sweeps form it, accumulated in FP64.  The density
// summation divides FP32 kernel sums by it, so the rounding of fW and 1 / h (up to 3 x 2^-24
// relative in the sum, 4e-5 of pressure at c0^2 = 240) cancels as it does in the
// reference's FP32 build, where sigma0 and the sums share one precision.
inline double lattice_sigma_fp32(int dim, float fW, float inv_h, double cutoff, double dp)
{
    const int depth = int(cutoff / dp) + 1;
    double sigma = 0.0;
    const int kd = dim == 3 ? depth : 0;
    for (int k = -kd; k <= kd; ++k)
        for (int j = -depth; j <= depth; ++j)
            for (int i = -depth; i <= depth; ++i)
            {
                const double x = i * dp, y = j * dp, z = k * dp;
                if (!(std::sqrt(x * x + y * y + z * z) < cutoff))
                    continue;
                const float xf = float(x), yf = float(y), zf = float(z);
                const float r2 = std::fma(zf, zf, std::fma(yf, yf, xf * xf));
                const float q = std::sqrt(r2) * inv_h;
                const float t = 1.0f - 0.5f * q;
                const float t2 = t * t;
                const float w = t2 * t2;
                const float poly = w * (1.0f + 2.0f * q);
                sigma += double(fW * poly);
            }
    return sigma;
}

// Constants of one fluid body against one static wall (same rounding for every solver).
// sigma0 is replaced by lattice_sigma_fp32 of the same lattice (spacing vol^(1/dim)).
inline MPParams make_params(int dim, double grid_spacing, double h, double rho0, double c0, double vol, double mass,
                            double sigma0, double wall_mass_over_rho0, double wall_vol, double limiter_slope,
                            const double *gravity)
{
    WendlandC2 wk = wendland(dim, h);
    MPParams k{};
    k.gs_f = float(grid_spacing);
    k.rc_sqr = float(wk.rc_sqr);
    k.rc_reach = float(std::sqrt(wk.rc_sqr) * (1.0 + 1e-4));
    k.inv_h = float(wk.inv_h);
    k.fW = float(wk.factor_W);
    k.cW = float(wk.factor_dW * 0.625 * vol);
    k.cWw = float(wk.factor_dW * 0.625 * wall_vol);
    k.rho0 = float(rho0);
    k.p0_over_rho0 = float(rho0 * c0 * c0 / rho0);
    k.Vol = float(vol);
    k.mass = float(mass);
    k.inv_mass = float(1.0 / mass);
    const double dp = dim == 3 ? std::cbrt(vol) : std::sqrt(vol);
    (void)sigma0; // the FP64 lattice sum of the drop-in; see lattice_sigma_fp32
    sigma0 = lattice_sigma_fp32(dim, k.fW, k.inv_h, wk.rc, dp);
    k.sigma0 = sigma0;
    k.rho0_over_sigma0 = float(rho0 / sigma0);
    k.wall_factor = float(wall_mass_over_rho0 * rho0 * rho0 / (sigma0 * mass));
    double Z = rho0 * c0;
    double inv_z = (Z + Z) / (Z * Z + Z * Z);
    k.inv_z = float(inv_z);
    k.zgeo = float(2.0 * Z * Z / (Z + Z));
    k.s_lim = float(limiter_slope * (0.5 * (rho0 + rho0) * inv_z));
    for (int d = 0; d < 3; ++d)
        k.g[d] = d < dim ? float(gravity[d]) : 0.f;
    k.c0 = c0;
    k.h = h;
    return k;
}

struct MPState
{
    float4 *geo0, *dyn; // {offset at the last configuration update, packed cell}; {velocity, pressure}
    // current offset from the cell corner as an FP32 pair: off = the FP64 offset rounded to
    // FP32 (what the pair arithmetic reads), off_lo = the FP32 rounding of its residual, so
    // the position integration carries the FP64 offset from step to step
    float *off, *off_lo, *force, *drho, *drho_dt, *drho_sum;
    float *pres; // the pressure of dyn.w as a dense array (the 1st half's gathers read 4 B)
    uint32_t *id;
    float *fprior, *shift; // periodic flow only: prior (viscous) force, transport-velocity shift
};

// FP64 offset of particle i along axis d, and its storage as the (off, off_lo) pair.
__device__ __forceinline__ double offset_of(const MPState &f, size_t n, size_t i, int d)
{
    return double(f.off[d * n + i]) + double(f.off_lo[d * n + i]);
}
__device__ __forceinline__ void store_offset(const MPState &f, size_t n, size_t i, int d, double x)
{
    const float hi = float(x);
    f.off[d * n + i] = hi;
    f.off_lo[d * n + i] = float(x - double(hi));
}
// Staging of new offsets between a re-hash and the gather into cell order: the FP32 pair
// of the FP64 offset, component d of particle i at noff[d * n + i] and noff[(3 + d) * n + i].
__device__ __forceinline__ void stage_offset(float *noff, size_t n, size_t i, int d, double x)
{
    const float hi = float(x);
    noff[d * n + i] = hi;
    noff[(3 + d) * n + i] = float(x - double(hi));
}

// Re-hash of particle i (cell c0 at the last configuration): its new sub-cell c and the
// staged offset pair.  A particle whose FP32 offset lies inside its sub-cell on every axis,
// away from the faces by a margin far above the residual, keeps its cell and its offset
// pair as they are, with no FP64 arithmetic (rehash_relative would give the same cell and
// the same offset); the others are re-based in FP64 by rehash_relative.
template <int D>
__device__ __forceinline__ void rehash_particle(const MeshDev &m, double inv_gs, float gs_f, bool periodic,
                                                const MPState &f, size_t n, size_t i, const int *c0, int *c,
                                                float *noff)
{
    bool inside = true;
#pragma unroll
    for (int d = 0; d < D; ++d)
    {
        const float o = f.off[d * n + i];
        inside = inside && o > 0.0f && o < gs_f * (1.0f - 1.0f / 65536.0f);
    }
    if (inside)
    {
#pragma unroll
        for (int d = 0; d < D; ++d)
        {
            c[d] = c0[d];
            noff[d * n + i] = f.off[d * n + i];
            noff[(3 + d) * n + i] = f.off_lo[d * n + i];
        }
        return;
    }
    double o[3] = {0.0, 0.0, 0.0}, no[3];
#pragma unroll
    for (int d = 0; d < D; ++d)
        o[d] = offset_of(f, n, i, d);
    rehash_relative<D>(m, inv_gs, periodic, c0, o, c, no);
#pragma unroll
    for (int d = 0; d < D; ++d)
        stage_offset(noff, n, i, d, no[d]);
}

// Position half-step x += dt / 2 v in FP64 on the stored pair.
__device__ __forceinline__ void half_step(const MPState &f, size_t n, size_t i, int d, double dt, float v)
{
    store_offset(f, n, i, d, offset_of(f, n, i, d) + 0.5 * dt * double(v));
}

struct MPWallData
{
    float4 *geo, *n;
};

struct MPNeighbors
{
    uint32_t *count, *J; // slot-major: slot s of particle i at J[s * n + i]
    unsigned cap;
    uint32_t limit = 0xffffffffu; // records the entries index (tested by the checked build)
    uint32_t mask = 0xffffffffu;  // index bits of an entry (periodic entries carry image codes)
};

// Entry e of list l indexes one of its records (always true unless built with SPHX_CHECK).
__device__ __forceinline__ bool entry_ok(uint32_t e, const MPNeighbors &l)
{
    return SPHX_CHECKED((e & l.mask) < l.limit, kCheckListEntry, e);
}

struct Kahan
{
    float s = 0.f, c = 0.f;
    __device__ __forceinline__ void add(float x)
    {
        float y = x - c;
        float t = s + y;
        c = (t - s) - y;
        s = t;
    }
    __device__ __forceinline__ float value() const { return s - c; }
};

// Packed FP32 (f32x2, sm_100 and later): one instruction applies the same IEEE operation,
// rounded to nearest, to two lanes, so a packed lane gives the bits of the scalar
// operation.  SPHX_PACKED_F32X2=0 builds the scalar form of the same operations.
#ifndef SPHX_PACKED_F32X2
#define SPHX_PACKED_F32X2 1
#endif
#ifndef SPHX_PACKED_SECOND
#define SPHX_PACKED_SECOND 1
#endif
#ifndef SPHX_PACKED_PERIODIC_SECOND
#define SPHX_PACKED_PERIODIC_SECOND 1
#endif
__device__ __forceinline__ float2 f2_add(float2 a, float2 b)
{
#if SPHX_PACKED_F32X2
    float2 d;
    asm("{.reg .b64 ra, rb, rd;\n\tmov.b64 ra, {%2, %3};\n\tmov.b64 rb, {%4, %5};\n\t"
        "add.rn.f32x2 rd, ra, rb;\n\tmov.b64 {%0, %1}, rd;}"
        : "=f"(d.x), "=f"(d.y)
        : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
    return d;
#else
    return make_float2(__fadd_rn(a.x, b.x), __fadd_rn(a.y, b.y));
#endif
}
__device__ __forceinline__ float2 f2_sub(float2 a, float2 b)
{
#if SPHX_PACKED_F32X2
    float2 d;
    asm("{.reg .b64 ra, rb, rd;\n\tmov.b64 ra, {%2, %3};\n\tmov.b64 rb, {%4, %5};\n\t"
        "sub.rn.f32x2 rd, ra, rb;\n\tmov.b64 {%0, %1}, rd;}"
        : "=f"(d.x), "=f"(d.y)
        : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
    return d;
#else
    return make_float2(__fsub_rn(a.x, b.x), __fsub_rn(a.y, b.y));
#endif
}
__device__ __forceinline__ float2 f2_fma(float2 a, float2 b, float2 c)
{
#if SPHX_PACKED_F32X2
    float2 d;
    asm("{.reg .b64 ra, rb, rc, rd;\n\tmov.b64 ra, {%2, %3};\n\tmov.b64 rb, {%4, %5};\n\t"
        "mov.b64 rc, {%6, %7};\n\tfma.rn.f32x2 rd, ra, rb, rc;\n\tmov.b64 {%0, %1}, rd;}"
        : "=f"(d.x), "=f"(d.y)
        : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y), "f"(c.x), "f"(c.y));
    return d;
#else
    return make_float2(fmaf(a.x, b.x, c.x), fmaf(a.y, b.y, c.y));
#endif
}

// Compensated neighbour sum: plain FP32 partials over groups, Kahan across groups.
struct Acc
{
    float part = 0.f;
    Kahan k;
    __device__ __forceinline__ void add(float x) { part += x; }
    __device__ __forceinline__ void flush()
    {
        k.add(part);
        part = 0.f;
    }
    __device__ __forceinline__ float value() const { return k.value(); }
};

// Two Acc of the x and y components with packed arithmetic: the partial takes
// fma(a, b, part) per component, the flush the Kahan steps per component, the same
// operations in the same order as two Acc fed with part += a * b (contracted to an fma).
struct Acc2
{
    float2 part = make_float2(0.f, 0.f), s = make_float2(0.f, 0.f), c = make_float2(0.f, 0.f);
    __device__ __forceinline__ void fma(float2 a, float2 b) { part = f2_fma(a, b, part); }
    __device__ __forceinline__ void flush()
    {
        const float2 y = f2_sub(part, c);
        const float2 t = f2_add(s, y);
        c = f2_sub(f2_sub(t, s), y);
        s = t;
        part = make_float2(0.f, 0.f);
    }
    __device__ __forceinline__ float x() const { return s.x - c.x; }
    __device__ __forceinline__ float y() const { return s.y - c.y; }
};

// Warp max of the order-preserving bits of v, one atomicMax per warp.
__device__ __forceinline__ void warp_max_to(unsigned long long *slot, double v)
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

// x_i - x_j from the packed cells and cell offsets.  pib = packed cell of i plus the lane
// bias: the 32-bit difference pib - p_j holds c_i - c_j + kCellBias in every lane (no
// borrow while |c_i - c_j| <= kCellBias), and each lane becomes an exact float through the
// 2^23 exponent pattern.
template <int D>
__device__ __forceinline__ void geo_dx(float gs, uint32_t pib, const float *oi, float4 gj, float *dx)
{
    const uint32_t dl = pib - __float_as_uint(gj.w);
    const float oj[3] = {gj.x, gj.y, gj.z};
#pragma unroll
    for (int d = 0; d < D; ++d)
    {
        uint32_t lane = (dl >> (d * CellLanes<D>::bits)) & CellLanes<D>::mask;
        float dc = __uint_as_float(0x4B000000u | lane) - (8388608.0f + float(kCellBias));
        dx[d] = fmaf(dc, gs, oi[d] - oj[d]);
    }
}

// geo_dx for the candidates of one run of for_each_candidate_run: the run's column fixes
// the cell differences of all axes but the last, so only the last lane is decoded per
// candidate.  Every difference is the same exact integer geo_dx forms, so dx is the same
// bit for bit.
template <int D>
struct RunDx
{
    float gs, kl; // kl = 2^23 + c_i of the last axis (exact)
    int c0, c1;
    const float *oi;
    __device__ __forceinline__ RunDx(float gs_, const int *ci, const float *oi_)
        : gs(gs_), kl(8388608.0f + float(ci[D - 1])), c0(ci[0]), c1(ci[1]), oi(oi_)
    {
    }
    __device__ __forceinline__ float column(int x) const { return float(c0 - x); }
    __device__ __forceinline__ float column_y(int y) const { return D == 3 ? float(c1 - y) : 0.0f; }
    __device__ __forceinline__ void dx(float dcx, float dcy, float4 gj, float *d) const
    {
        const uint32_t lane = (__float_as_uint(gj.w) >> ((D - 1) * CellLanes<D>::bits)) & CellLanes<D>::mask;
        const float dcl = kl - __uint_as_float(0x4B000000u | lane);
        d[0] = fmaf(dcx, gs, oi[0] - gj.x);
        if (D == 3)
        {
            d[1] = fmaf(dcy, gs, oi[1] - gj.y);
            d[2] = fmaf(dcl, gs, oi[2] - gj.z);
        }
        else
            d[1] = fmaf(dcl, gs, oi[1] - gj.y);
    }
};

// geo_dx with the x and y components packed (the same operations per component); oi01
// holds o_i along x and y.
template <int D>
__device__ __forceinline__ void geo_dx2(float gs, uint32_t pib, float2 oi01, float oi2, float4 gj, float *dx)
{
    const uint32_t dl = pib - __float_as_uint(gj.w);
    const float K = 8388608.0f + float(kCellBias);
    const float2 m01 = make_float2(__uint_as_float(0x4B000000u | (dl & CellLanes<D>::mask)),
                                   __uint_as_float(0x4B000000u | ((dl >> CellLanes<D>::bits) & CellLanes<D>::mask)));
    const float2 dc = f2_sub(m01, make_float2(K, K));
    const float2 d01 = f2_fma(dc, make_float2(gs, gs), f2_sub(oi01, make_float2(gj.x, gj.y)));
    dx[0] = d01.x;
    dx[1] = d01.y;
    if (D == 3)
    {
        const uint32_t lane = (dl >> (2 * CellLanes<D>::bits)) & CellLanes<D>::mask;
        const float dcz = __uint_as_float(0x4B000000u | lane) - K;
        dx[2] = fmaf(dcz, gs, oi2 - gj.z);
    }
}

template <int D>
__device__ __forceinline__ float sq(const float *dx)
{
    float s = dx[0] * dx[0] + dx[1] * dx[1];
    if (D == 3)
        s += dx[2] * dx[2];
    return s;
}

template <int D>
__device__ __forceinline__ float dot(const float *a, const float *b)
{
    float s = a[0] * b[0] + a[1] * b[1];
    if (D == 3)
        s += a[2] * b[2];
    return s;
}

// 1 / r (0 for coincident particles, whose kernel gradient is zero).
__device__ __forceinline__ float inv_dist(float r2) { return r2 > 0.f ? rsqrtf(r2) : 0.f; }

// Wendland C2 W(r) = fW t^4 (1 + 2q), t = 1 - q/2.
__device__ __forceinline__ float wc2_W(float fW, float inv_h, float r)
{
    float q = r * inv_h;
    float t = 1.0f - 0.5f * q;
    float t2 = t * t;
    return fW * (t2 * t2 * (1.0f + 2.0f * q));
}
// dW(r) V = c (q - 2)^3 q with c = fdW 5/8 V.
__device__ __forceinline__ float wc2_dWV(float c, float inv_h, float r)
{
    float q = r * inv_h;
    float t = q - 2.0f;
    return c * (t * t * t) * q;
}

// DissipativePJump of the AcousticRiemannSolver with the TruncatedLinear limiter.
__device__ __forceinline__ float p_jump(const MPParams &k, float u)
{
    return k.zgeo * u * fminf(k.s_lim * fmaxf(u, 0.0f), 1.0f);
}

// The window is pruned to the sub-cells that can hold a neighbour: for a particle at
// offset o in its sub-cell, the slab of sub-cell c + a along an axis lies a gs - o above
// it (a > 0) or o + (|a| - 1) gs below it (a < 0).  Columns whose gap in the leading axes
// reaches r are skipped, and the run along the last axis is cut to the sub-cells closer
// than sqrt(r^2 - gap^2).  r is the cut-off enlarged by 1e-4 relative, far above the
// rounding of the offsets, so every candidate the membership test accepts is visited;
// the order of the visited candidates is the unpruned order.
struct Reach
{
    const float *o;      // offsets of the particle in its sub-cell
    float gs, r, inv_gs; // sub-cell spacing, reach radius, 1 / spacing
    __device__ __forceinline__ Reach(const float *o_, float gs_, float r_) : o(o_), gs(gs_), r(r_), inv_gs(1.0f / gs_)
    {
    }
};

__device__ __forceinline__ float slab_gap(float o, float gs, int a)
{
    return a > 0 ? float(a) * gs - o : (a < 0 ? o + float(-a - 1) * gs : 0.0f);
}

// Sub-cells c + a, -lo <= a <= hi, closer than r along one axis (inv_gs = 1 / gs; the
// reach margin covers the rounding of the product).
__device__ __forceinline__ void axis_reach(float o, float inv_gs, float r, int &lo, int &hi)
{
    hi = max(0, min(kReach, int(ceilf((r + o) * inv_gs)) - 1));
    lo = max(0, min(kReach, int(ceilf((r - o) * inv_gs))));
}

// Sub-cell c inside the mesh, and its indices packed 16 bits per axis (for the check record).
template <int D>
__device__ __forceinline__ bool cell_in_mesh(const MeshDev &m, const int *c)
{
    bool in = true;
#pragma unroll
    for (int a = 0; a < D; ++a)
        in = in && c[a] >= 0 && c[a] < m.all_cells[a];
    return in;
}
template <int D>
__device__ __forceinline__ uint64_t packed_cell(const int *c)
{
    uint64_t p = 0;
#pragma unroll
    for (int a = 0; a < D; ++a)
        p |= uint64_t(uint16_t(c[a])) << (16 * a);
    return p;
}

// Candidate runs of the pruned (2 kReach + 1)^D window around sub-cell c: run(x, y, b, e)
// for every column (x, y) of the window (x alone in 2D) with the candidate particles
// [b, e) of its cells along the last axis; the cells of one instance start at cell_base
// (columns along the last axis are contiguous in the linear cell order).
template <int D, bool PRUNE, class R>
__device__ __forceinline__ void for_each_candidate_run(const MeshDev &m, uint32_t cell_base, const uint32_t *offset,
                                                       const int *c, const Reach &q, R &&run)
{
    // checked builds: the sub-cell lies in the mesh and every range is ordered
    if (!SPHX_CHECKED(cell_in_mesh<D>(m, c), kCheckCellIndex, packed_cell<D>(c)))
        return;
    auto span = [&](int x, int y, uint32_t b, uint32_t e) {
        if (SPHX_CHECKED(b <= e, kCheckCellRange, (uint64_t(b) << 32) | e))
            run(x, y, b, e);
    };
    if (!PRUNE)
    {
        const int lo0 = max(c[0] - kReach, 0), hi0 = min(c[0] + kReach, m.all_cells[0] - 1);
        const int lo1 = max(c[1] - kReach, 0), hi1 = min(c[1] + kReach, m.all_cells[1] - 1);
        if (D == 2)
        {
            for (int x = lo0; x <= hi0; ++x)
            {
                uint32_t a = cell_base + uint32_t(x) * uint32_t(m.all_cells[1]);
                span(x, 0, offset[a + uint32_t(lo1)], offset[a + uint32_t(hi1) + 1]);
            }
        }
        else
        {
            const int lo2 = max(c[2] - kReach, 0), hi2 = min(c[2] + kReach, m.all_cells[2] - 1);
            for (int x = lo0; x <= hi0; ++x)
                for (int y = lo1; y <= hi1; ++y)
                {
                    uint32_t a = cell_base +
                                 (uint32_t(x) * uint32_t(m.all_cells[1]) + uint32_t(y)) * uint32_t(m.all_cells[2]);
                    span(x, y, offset[a + uint32_t(lo2)], offset[a + uint32_t(hi2) + 1]);
                }
        }
        return;
    }
    const float r2 = q.r * q.r;
    int l0, h0;
    axis_reach(q.o[0], q.inv_gs, q.r, l0, h0);
    const int lo0 = max(c[0] - l0, 0), hi0 = min(c[0] + h0, m.all_cells[0] - 1);
    if (D == 2)
    {
        for (int x = lo0; x <= hi0; ++x)
        {
            const float gx = slab_gap(q.o[0], q.gs, x - c[0]);
            int l1, h1;
            axis_reach(q.o[1], q.inv_gs, sqrtf(fmaxf(r2 - gx * gx, 0.0f)), l1, h1);
            const int lo1 = max(c[1] - l1, 0), hi1 = min(c[1] + h1, m.all_cells[1] - 1);
            uint32_t a = cell_base + uint32_t(x) * uint32_t(m.all_cells[1]);
            span(x, 0, offset[a + uint32_t(lo1)], offset[a + uint32_t(hi1) + 1]);
        }
    }
    else
    {
        int l1, h1;
        axis_reach(q.o[1], q.inv_gs, q.r, l1, h1);
        const int lo1 = max(c[1] - l1, 0), hi1 = min(c[1] + h1, m.all_cells[1] - 1);
        for (int x = lo0; x <= hi0; ++x)
        {
            const float gx = slab_gap(q.o[0], q.gs, x - c[0]);
            for (int y = lo1; y <= hi1; ++y)
            {
                const float gy = slab_gap(q.o[1], q.gs, y - c[1]);
                const float g2 = gx * gx + gy * gy;
                if (!(g2 < r2))
                    continue;
                int l2, h2;
                axis_reach(q.o[2], q.inv_gs, sqrtf(r2 - g2), l2, h2);
                const int lo2 = max(c[2] - l2, 0), hi2 = min(c[2] + h2, m.all_cells[2] - 1);
                uint32_t a = cell_base +
                             (uint32_t(x) * uint32_t(m.all_cells[1]) + uint32_t(y)) * uint32_t(m.all_cells[2]);
                span(x, y, offset[a + uint32_t(lo2)], offset[a + uint32_t(hi2) + 1]);
            }
        }
    }
}

// Candidates of the pruned window one by one: f(j) in run order.
template <int D, bool PRUNE, class F>
__device__ __forceinline__ void for_each_candidate(const MeshDev &m, uint32_t cell_base, const uint32_t *offset,
                                                   const int *c, const Reach &q, F &&f)
{
    for_each_candidate_run<D, PRUNE>(m, cell_base, offset, c, q, [&](int, int, uint32_t b, uint32_t e) {
        for (uint32_t j = b; j < e; ++j)
            f(j);
    });
}

// Neighbour visits of one particle: stored lists (LISTS) or a sweep of the sub-cells with
// the same membership test as the build, in the same order, so both give the same sums.
struct Visit
{
    MeshDev m;
    uint32_t cell_base;
    const uint32_t *f_offset, *w_offset;
};

// This lane's place in its group of LANES consecutive lanes (0 when LANES is 1).
template <int LANES>
__device__ __forceinline__ unsigned lane_in_group()
{
    return LANES == 1 ? 0u : (threadIdx.x & unsigned(LANES - 1));
}

// Sum of v over the LANES lanes of this lane's group (consecutive lanes, LANES a power of
// two dividing 32); every lane of the group gets the sum.
template <int LANES>
__device__ __forceinline__ float group_sum(float v)
{
    if (LANES > 1)
    {
        const unsigned lane = threadIdx.x & 31u;
        const unsigned mask = ((1u << LANES) - 1u) << (lane & ~unsigned(LANES - 1));
#pragma unroll
        for (int o = LANES / 2; o > 0; o >>= 1)
            v += __shfl_xor_sync(mask, v, o);
    }
    return v;
}

// Calls pair(x) for every stored neighbour of i, with U neighbour records loaded
// before the arithmetic, and flush() after every kGroup neighbours; load(j) fetches what
// pair() consumes.  PREFETCH also loads the next U list entries before the current
// records are used (one list read in flight behind the record gathers); it pays where the
// records are small (1st half), not where the extra registers cost occupancy (2nd half).
// With LANES > 1 the lanes of a group share the particle: lane `sub` visits the list slots
// sub, sub + LANES, sub + 2 LANES, ... (its own compensated sums, combined afterwards).
template <bool PREFETCH, int U, int LANES = 1, class Load, class Pair, class Flush>
__device__ __forceinline__ void list_sweep(size_t i, size_t n, const MPNeighbors &l, Load &&load, Pair &&pair,
                                           Flush &&flush, unsigned sub = 0)
{
    static_assert(kGroup % U == 0, "groups hold whole unrolled batches");
    const unsigned call = min(l.count[i], l.cap);
    const unsigned c = LANES == 1 ? call : (call > sub ? (call - sub + LANES - 1) / LANES : 0u);
    const uint32_t *J = l.J + i + size_t(LANES == 1 ? 0u : sub) * n;
    const size_t stride = size_t(LANES) * n;
    unsigned s = 0;
    uint32_t jn[U];
    if (PREFETCH && c >= U)
    {
#pragma unroll
        for (int u = 0; u < U; ++u)
            jn[u] = __ldg(&J[size_t(u) * stride]);
    }
    for (; s + kGroup <= c; s += kGroup)
    {
#pragma unroll
        for (int h = 0; h < kGroup; h += U)
        {
            uint32_t jj[U];
            if (PREFETCH)
            {
#pragma unroll
                for (int u = 0; u < U; ++u)
                    jj[u] = jn[u];
                const unsigned nx = s + h + U;
                if (nx + U <= c)
                {
#pragma unroll
                    for (int u = 0; u < U; ++u)
                        jn[u] = __ldg(&J[size_t(nx + u) * stride]);
                }
            }
            else
            {
#pragma unroll
                for (int u = 0; u < U; ++u)
                    jj[u] = __ldg(&J[size_t(s + h + u) * stride]);
            }
            decltype(load(0u)) rec[U];
            bool ok[U];
#pragma unroll
            for (int u = 0; u < U; ++u)
                ok[u] = entry_ok(jj[u], l);
#pragma unroll
            for (int u = 0; u < U; ++u)
                rec[u] = ok[u] ? load(jj[u]) : decltype(load(0u)){};
#pragma unroll
            for (int u = 0; u < U; ++u)
                if (ok[u])
                    pair(rec[u]);
        }
        flush();
    }
    for (; s < c; ++s)
    {
        const uint32_t j = __ldg(&J[size_t(s) * stride]);
        if (entry_ok(j, l))
            pair(load(j));
    }
    flush();
}

// ---------------------------------------------------------------- asynchronous gathers
// cp.async copies of neighbour records from global into shared memory: the copy is in
// flight without holding registers, so a thread keeps DEPTH neighbours' records (and the
// list entries DEPTH further on) in flight while it computes, instead of the U records an
// unrolled register gather holds.
__device__ __forceinline__ void cp_async16(void *smem, const void *gmem)
{
    const unsigned a = unsigned(__cvta_generic_to_shared(smem));
    asm volatile("cp.async.ca.shared.global [%0], [%1], 16;\n" ::"r"(a), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async4(void *smem, const void *gmem)
{
    const unsigned a = unsigned(__cvta_generic_to_shared(smem));
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(a), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait()
{
    asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

// Per-thread ring of DEPTH slots in shared memory, slot-major (slot s of thread t at
// [s * blockDim + t], so a warp's lanes touch consecutive words: no bank conflicts).
template <int DEPTH>
struct AsyncRing
{
    float4 *a, *b;  // two 16-byte parts of a record (b may be unused)
    float *c;       // a 4-byte part (may be unused)
    uint32_t *idx;  // list entries DEPTH neighbours ahead
    unsigned tid, bd;
    __device__ __forceinline__ unsigned at(unsigned slot) const { return slot * bd + tid; }
};

// list_sweep with the records fetched through the ring: issue(j, slot) starts the copies of
// neighbour j into a slot, read(slot) returns the record, pair/flush as list_sweep.  The
// neighbours, their order and the kGroup flushes are those of list_sweep, so the sums are
// the same bit for bit.  Each iteration commits one copy group (possibly empty), so waiting
// for all but the DEPTH - 1 newest groups completes exactly the oldest neighbour's copies.
template <int DEPTH, class Issue, class Read, class Pair, class Flush>
__device__ __forceinline__ void list_sweep_async(size_t i, size_t n, const MPNeighbors &l,
                                                 const AsyncRing<DEPTH> &ring, Issue &&issue, Read &&read,
                                                 Pair &&pair, Flush &&flush)
{
    const unsigned c = min(l.count[i], l.cap);
    const uint32_t *J = l.J + i;
    // a bad entry (checked builds) is not copied: its pair reads the slot's stale record
    auto issue_entry = [&](uint32_t j, unsigned slot) {
        if (entry_ok(j, l))
            issue(j, slot);
    };
#pragma unroll
    for (int u = 0; u < DEPTH; ++u)
    {
        if (unsigned(u) < c)
            issue_entry(__ldg(&J[size_t(u) * n]), unsigned(u));
        if (unsigned(u + DEPTH) < c)
            cp_async4(&ring.idx[ring.at(u)], &J[size_t(u + DEPTH) * n]);
        cp_async_commit();
    }
    unsigned g = 0, slot = 0;
    for (unsigned s = 0; s < c; ++s)
    {
        cp_async_wait<DEPTH - 1>();
        const auto r = read(slot);
        pair(r); // consumes the slot before it is refilled
        const unsigned nx = s + DEPTH;
        if (nx < c)
        {
            issue_entry(ring.idx[ring.at(slot)], slot);
            if (nx + DEPTH < c)
                cp_async4(&ring.idx[ring.at(slot)], &J[size_t(nx + DEPTH) * n]);
        }
        cp_async_commit();
        if (++g == kGroup)
        {
            flush();
            g = 0;
        }
        slot = slot + 1 == DEPTH ? 0 : slot + 1;
    }
    flush();
    cp_async_wait<0>();
}

// Same visits by cell sweep: accepts the candidates the build accepted.
template <int D, bool PRUNE, class Load, class Pair, class Flush>
__device__ __forceinline__ void cell_sweep(const Visit &v, const uint32_t *offset, const int *ci, float gs, uint32_t pib,
                                           const float *oi, float rc_sqr, float rc_reach, size_t self,
                                           const float4 *geo, Load &&load, Pair &&pair, Flush &&flush)
{
    int g = 0;
    for_each_candidate<D, PRUNE>(v.m, v.cell_base, offset, ci, Reach(oi, gs, rc_reach), [&](uint32_t j) {
        if (size_t(j) == self)
            return;
        float dx[3];
        geo_dx<D>(gs, pib, oi, geo[j], dx);
        if (!(sq<D>(dx) < rc_sqr))
            return;
        pair(load(j));
        if (++g == kGroup)
        {
            flush();
            g = 0;
        }
    });
    flush();
}

struct FirstRec
{
    float4 g;
    float p;
};
struct SecondRec
{
    float4 g, v;
};

// 1st half of one particle: pressure force and density-rate dissipation against fluid and
// wall neighbours, velocity update and the first position half-step.  Returns the
// acoustic-time-step candidate c0 + |v|.
// DEPTH > 0: the stored lists with the neighbour records gathered through an AsyncRing of
// that depth (ring: slots for geo0 in a, the pressure in c).
// LANES > 1: the stored lists, LANES consecutive lanes on particle i (list slots strided
// over the lanes, sums combined by shuffles); the first lane of the group writes the state
// and returns the candidate, the others return -1e300.
template <int D, bool LISTS, int DEPTH = 0, int LANES = 1>
__device__ __forceinline__ double first_particle(size_t i, size_t n, const MPParams &k, const Visit &v, double dt,
                                                 const MPState &f, const MPWallData &w, const MPNeighbors &in,
                                                 const MPNeighbors &wl, const AsyncRing<DEPTH> *ring = nullptr)
{
    const float4 gi = f.geo0[i];
    const uint32_t pib = __float_as_uint(gi.w) + CellLanes<D>::bias;
    int ci[3] = {0, 0, 0};
    if (!LISTS)
        unpack_cell<D>(__float_as_uint(gi.w), ci);
    const float oi[3] = {gi.x, gi.y, gi.z};
    const float4 di = f.dyn[i];
    const float p_i = di.w;
    const float rho_i = k.rho0 + f.drho[i];
    // the x and y components in packed arithmetic (the same operations as the scalar z)
    // (measured slower here: the z force paired with the dissipation in a second packed
    // accumulator, 60 B of spills; p_i + p_j and p_i - p_j as one packed add, 12 B)
    const float2 oi01 = make_float2(gi.x, gi.y);
    Acc2 force01;
    Acc force2, rdis;
    auto pair = [&](const FirstRec &r) {
        float dx[3];
        geo_dx2<D>(k.gs_f, pib, oi01, oi[2], r.g, dx);
        float r2 = sq<D>(dx);
        float inv = inv_dist(r2);
        float dWV = wc2_dWV(k.cW, k.inv_h, r2 * inv);
        float sc = (p_i + r.p) * (dWV * inv);
        force01.fma(make_float2(-sc, -sc), make_float2(dx[0], dx[1]));
        if (D == 3)
            force2.add(-sc * dx[2]);
        rdis.add((p_i - r.p) * dWV);
    };
    auto flush = [&]() {
        force01.flush();
        if (D == 3)
            force2.flush();
        rdis.flush();
    };
    auto load = [&](uint32_t j) { return FirstRec{__ldg(&f.geo0[j]), __ldg(&f.pres[j])}; };
    if constexpr (DEPTH > 0)
    {
        const AsyncRing<DEPTH> &rg = *ring;
        auto issue = [&](uint32_t j, unsigned slot) {
            cp_async16(&rg.a[rg.at(slot)], &f.geo0[j]);
            cp_async4(&rg.c[rg.at(slot)], &f.pres[j]);
        };
        auto read = [&](unsigned slot) { return FirstRec{rg.a[rg.at(slot)], rg.c[rg.at(slot)]}; };
        list_sweep_async<DEPTH>(i, n, in, rg, issue, read, pair, flush);
    }
    else if (LISTS)
        list_sweep<true, kUnrollFirst, LANES>(i, n, in, load, pair, flush, lane_in_group<LANES>());
    else
        cell_sweep<D, true>(v, v.f_offset, ci, k.gs_f, pib, oi, k.rc_sqr, k.rc_reach, i, f.geo0, load, pair, flush);

    Acc2 wforce01; // x and y packed, as the fluid pairs
    Acc wforce2, wrdis;
    auto wpair = [&](const float4 &gj) {
        float dx[3];
        geo_dx2<D>(k.gs_f, pib, oi01, oi[2], gj, dx);
        float r2 = sq<D>(dx);
        float inv = inv_dist(r2);
        float dWV = wc2_dWV(k.cWw, k.inv_h, r2 * inv);
        // wall pressure p_i + rho_i r max(0, (F_prior / m - a_wall) . (-e)), static wall
        float p_w = p_i + rho_i * fmaxf(0.0f, -dot<D>(k.g, dx));
        float sc = (p_i + p_w) * (dWV * inv);
        wforce01.fma(make_float2(-sc, -sc), make_float2(dx[0], dx[1]));
        if (D == 3)
            wforce2.add(-sc * dx[2]);
        wrdis.add((p_i - p_w) * dWV);
    };
    auto wflush = [&]() {
        wforce01.flush();
        if (D == 3)
            wforce2.flush();
        wrdis.flush();
    };
    auto wload = [&](uint32_t j) { return __ldg(&w.geo[j]); };
    if (LISTS || DEPTH > 0)
        list_sweep<true, kUnrollFirst, LANES>(i, n, wl, wload, wpair, wflush, lane_in_group<LANES>());
    else
        cell_sweep<D, false>(v, v.w_offset, ci, k.gs_f, pib, oi, k.rc_sqr, k.rc_reach, ~size_t(0), w.geo, wload,
                             wpair, wflush);

    const float fv[3] = {force01.x(), force01.y(), force2.value()};
    const float wv[3] = {wforce01.x(), wforce01.y(), wforce2.value()};
    const float rv = rdis.value();
    float fsum[3], wfsum[3];
#pragma unroll
    for (int d = 0; d < D; ++d)
    {
        fsum[d] = group_sum<LANES>(fv[d]);
        wfsum[d] = group_sum<LANES>(wv[d]);
    }
    const float rsum = group_sum<LANES>(rv), wrsum = group_sum<LANES>(wrdis.value());
    if (lane_in_group<LANES>() != 0)
        return -1.0e300;
    f.drho_dt[i] = (rsum * k.inv_z) * rho_i + (wrsum * k.inv_z) * rho_i;
    float v2 = 0.f;
    float vn[3] = {di.x, di.y, di.z};
    const float dt_f = float(dt);
#pragma unroll
    for (int d = 0; d < D; ++d)
    {
        float F = f.force[d * n + i] + fsum[d] * k.Vol + wfsum[d] * k.Vol;
        f.force[d * n + i] = F;
        float vo = vn[d];
        // position half-step in FP64 (initialisation of the 1st half, old velocity)
        half_step(f, n, i, d, dt, vo);
        vn[d] = vo + (k.g[d] + F * k.inv_mass) * dt_f;
        v2 += vn[d] * vn[d];
    }
    // the pressure stays the one the neighbours of this sweep read
    f.dyn[i] = make_float4(vn[0], vn[1], D == 3 ? vn[2] : 0.f, p_i);
    return k.c0 + double(sqrtf(v2));
}

// 2nd half of one particle: the second position half-step, density rate and pressure
// dissipation against fluid and wall neighbours, density update.  Returns the
// advection-time-step candidate max(|v|^2, 4 h |F + F_prior| / m).
// DEPTH > 0: the stored lists with the neighbour records gathered through an AsyncRing of
// that depth (ring: slots for geo0 in a, dyn in b).  LANES as first_particle.
template <int D, bool LISTS, int DEPTH = 0, int LANES = 1>
__device__ __forceinline__ double second_particle(size_t i, size_t n, const MPParams &k, const Visit &v, double dt,
                                                  const MPState &f, const MPWallData &w, const MPNeighbors &in,
                                                  const MPNeighbors &wl, const AsyncRing<DEPTH> *ring = nullptr)
{
    const float4 gi = f.geo0[i];
    const uint32_t pib = __float_as_uint(gi.w) + CellLanes<D>::bias;
    int ci[3] = {0, 0, 0};
    if (!LISTS)
        unpack_cell<D>(__float_as_uint(gi.w), ci);
    const float oi[3] = {gi.x, gi.y, gi.z};
    const float4 di = f.dyn[i];
    const float vi[3] = {di.x, di.y, di.z};
    const float rho_i = k.rho0 + f.drho[i];
    // with SPHX_PACKED_SECOND the x and y components in packed arithmetic (the same
    // operations): measured 8 % faster when the kernel is held to 64 registers, slower
    // when it takes the 66 it would otherwise use
    const float2 oi01 = make_float2(gi.x, gi.y), vi01 = make_float2(di.x, di.y);
    Acc rate, pdis[3];
    Acc2 pdis01, zr;
    auto pair = [&](const SecondRec &r) {
        float dx[3];
        if (SPHX_PACKED_SECOND)
            geo_dx2<D>(k.gs_f, pib, oi01, oi[2], r.g, dx);
        else
            geo_dx<D>(k.gs_f, pib, oi, r.g, dx);
        float r2 = sq<D>(dx);
        float inv = inv_dist(r2);
        float dWV = wc2_dWV(k.cW, k.inv_h, r2 * inv);
        float dv[3];
        if (SPHX_PACKED_SECOND)
        {
            const float2 dv01 = f2_sub(vi01, make_float2(r.v.x, r.v.y));
            dv[0] = dv01.x;
            dv[1] = dv01.y;
        }
        else
        {
            dv[0] = vi[0] - r.v.x;
            dv[1] = vi[1] - r.v.y;
        }
        dv[2] = vi[2] - r.v.z;
        float u = dot<D>(dv, dx) * inv;
        float sc = p_jump(k, u) * (dWV * inv);
        if (SPHX_PACKED_SECOND)
        {
            pdis01.fma(make_float2(sc, sc), make_float2(dx[0], dx[1]));
            if (D == 3) // the z dissipation and the density rate share a packed pair
                zr.fma(make_float2(sc, u), make_float2(dx[2], dWV));
            else
                rate.add(u * dWV);
        }
        else
        {
            rate.add(u * dWV);
#pragma unroll
            for (int d = 0; d < D; ++d)
                pdis[d].add(sc * dx[d]);
        }
    };
    auto flush = [&]() {
        if (SPHX_PACKED_SECOND)
        {
            pdis01.flush();
            if (D == 3)
                zr.flush();
            else
                rate.flush();
        }
        else
        {
            rate.flush();
#pragma unroll
            for (int d = 0; d < D; ++d)
                pdis[d].flush();
        }
    };
    auto load = [&](uint32_t j) { return SecondRec{__ldg(&f.geo0[j]), __ldg(&f.dyn[j])}; };
    if constexpr (DEPTH > 0)
    {
        const AsyncRing<DEPTH> &rg = *ring;
        auto issue = [&](uint32_t j, unsigned slot) {
            cp_async16(&rg.a[rg.at(slot)], &f.geo0[j]);
            cp_async16(&rg.b[rg.at(slot)], &f.dyn[j]);
        };
        auto read = [&](unsigned slot) { return SecondRec{rg.a[rg.at(slot)], rg.b[rg.at(slot)]}; };
        list_sweep_async<DEPTH>(i, n, in, rg, issue, read, pair, flush);
    }
    else if (LISTS)
        list_sweep<kPrefetchSecond, kUnrollSecond, LANES>(i, n, in, load, pair, flush, lane_in_group<LANES>());
    else
        cell_sweep<D, true>(v, v.f_offset, ci, k.gs_f, pib, oi, k.rc_sqr, k.rc_reach, i, f.geo0, load, pair, flush);

    Acc wrate, wdis2;
    Acc2 wdis01; // x and y packed, as the fluid pairs
    auto wpair = [&](const SecondRec &r) {
        float dx[3];
        geo_dx2<D>(k.gs_f, pib, oi01, oi[2], r.g, dx);
        float r2 = sq<D>(dx);
        float inv = inv_dist(r2);
        float dWV = wc2_dWV(k.cWw, k.inv_h, r2 * inv);
        const float nj[3] = {r.v.x, r.v.y, r.v.z};
        float en = dot<D>(dx, nj);
        float sgn = en < 0.f ? -1.f : (en > 0.f ? 1.f : 0.f);
        // (v_i - (2 v_wall - v_i)) . e with a static wall; face velocity jump along n
        wrate.add(2.0f * (dot<D>(vi, dx) * inv) * dWV);
        float sc = p_jump(k, 2.0f * sgn * dot<D>(vi, nj)) * dWV * sgn;
        wdis01.fma(make_float2(sc, sc), make_float2(nj[0], nj[1]));
        if (D == 3)
            wdis2.add(sc * nj[2]);
    };
    auto wflush = [&]() {
        wrate.flush();
        wdis01.flush();
        if (D == 3)
            wdis2.flush();
    };
    auto wload = [&](uint32_t j) { return SecondRec{__ldg(&w.geo[j]), __ldg(&w.n[j])}; };
    if (LISTS || DEPTH > 0)
        list_sweep<false, kUnrollSecond, LANES>(i, n, wl, wload, wpair, wflush, lane_in_group<LANES>());
    else
        cell_sweep<D, false>(v, v.w_offset, ci, k.gs_f, pib, oi, k.rc_sqr, k.rc_reach, ~size_t(0), w.geo, wload,
                             wpair, wflush);

    const bool zr_rate = SPHX_PACKED_SECOND && D == 3;
    const float pv[3] = {SPHX_PACKED_SECOND ? pdis01.x() : pdis[0].value(),
                         SPHX_PACKED_SECOND ? pdis01.y() : pdis[1].value(),
                         SPHX_PACKED_SECOND ? zr.x() : pdis[2].value()};
    const float rate_v = zr_rate ? zr.y() : rate.value();
    const float wv[3] = {wdis01.x(), wdis01.y(), wdis2.value()};
    float psum[3], wpsum[3];
#pragma unroll
    for (int d = 0; d < D; ++d)
    {
        psum[d] = group_sum<LANES>(pv[d]);
        wpsum[d] = group_sum<LANES>(wv[d]);
    }
    const float ratesum = group_sum<LANES>(rate_v), wratesum = group_sum<LANES>(wrate.value());
    if (lane_in_group<LANES>() != 0)
        return -1.0e300;
    float drho_dt = f.drho_dt[i] + ratesum * rho_i + wratesum * rho_i;
    f.drho_dt[i] = drho_dt;
    f.drho[i] = f.drho[i] + drho_dt * float(0.5 * dt);
    float v2 = 0.f, a2 = 0.f;
#pragma unroll
    for (int d = 0; d < D; ++d)
    {
        float F = psum[d] * k.Vol + wpsum[d] * k.Vol;
        f.force[d * n + i] = F;
        half_step(f, n, i, d, dt, vi[d]);
        v2 += vi[d] * vi[d];
        float ft = F + k.mass * k.g[d];
        a2 += ft * ft;
    }
    return double(fmaxf(v2, 4.0f * float(k.h) * sqrtf(a2) * k.inv_mass));
}

// Configuration of one particle: fluid and wall neighbour lists (candidate order of the
// surrounding sub-cells) and the density-summation sum drho_sum = rho_sum - rho0, in one
// pass over the candidates.  (The two-phase form of build_particle_periodic measured
// slower here: the kernel sum is too light to repay the second read of the neighbours.)
template <int D>
__device__ __forceinline__ void build_particle(size_t i, size_t n, const MPParams &k, const Visit &v,
                                               const MPState &f, const MPWallData &w, const MPNeighbors &in,
                                               const MPNeighbors &wl, unsigned int *max_counts)
{
    const float4 gi = f.geo0[i];
    const uint32_t pib = __float_as_uint(gi.w) + CellLanes<D>::bias;
    int ci[3] = {0, 0, 0};
    unpack_cell<D>(__float_as_uint(gi.w), ci);
    const float oi[3] = {gi.x, gi.y, gi.z};
    Kahan sigma;
    unsigned cnt = 0;
    const RunDx<D> rd(k.gs_f, ci, oi);
    for_each_candidate_run<D, true>(v.m, v.cell_base, v.f_offset, ci, Reach(oi, k.gs_f, k.rc_reach),
                                    [&](int x, int y, uint32_t b, uint32_t e) {
                                        const float dcx = rd.column(x), dcy = rd.column_y(y);
                                        for (uint32_t j = b; j < e; ++j)
                                        {
                                            if (j == uint32_t(i))
                                                continue;
                                            float dx[3];
                                            rd.dx(dcx, dcy, f.geo0[j], dx);
                                            float r2 = sq<D>(dx);
                                            if (!(r2 < k.rc_sqr))
                                                continue;
                                            if (cnt < in.cap)
                                                in.J[size_t(cnt) * n + i] = j;
                                            ++cnt;
                                            sigma.add(wc2_W(k.fW, k.inv_h, sqrtf(r2)));
                                        }
                                    });
    Kahan wsig;
    unsigned wc = 0;
    for_each_candidate_run<D, false>(v.m, v.cell_base, v.w_offset, ci, Reach(oi, k.gs_f, k.rc_reach),
                                     [&](int x, int y, uint32_t b, uint32_t e) {
                                         const float dcx = rd.column(x), dcy = rd.column_y(y);
                                         for (uint32_t j = b; j < e; ++j)
                                         {
                                             float dx[3];
                                             rd.dx(dcx, dcy, w.geo[j], dx);
                                             float r2 = sq<D>(dx);
                                             if (!(r2 < k.rc_sqr))
                                                 continue;
                                             if (wc < wl.cap)
                                                 wl.J[size_t(wc) * n + i] = j;
                                             ++wc;
                                             wsig.add(wc2_W(k.fW, k.inv_h, sqrtf(r2)));
                                         }
                                     });
    in.count[i] = cnt;
    wl.count[i] = wc;
    warp_atomic_max(&max_counts[0], cnt);
    warp_atomic_max(&max_counts[1], wc);
    // rho_sum - rho0 = rho0 (W0 + sum W - sigma0) / sigma0 + wall term
    double dsig = (double(sigma.s) - k.sigma0) - double(sigma.c) + double(k.fW);
    f.drho_sum[i] = float(dsig) * k.rho0_over_sigma0 + wsig.value() * k.wall_factor;
}

// ---------------------------------------------------------------- periodic flow
// A periodic box is tiled by the sub-cells exactly (cell count per axis N_d >= 2 kReach + 1,
// spacing >= h), so the (2 kReach + 1)^D window of a particle wraps around the box and
// visits every sub-cell at most once.  A neighbour found through a wrapped cell is the
// image x_j + s L (s = -1 past the upper face, +1 past the lower one, per axis); its list
// entry carries s in two bits per axis above the particle index, and the packed cell
// difference of the pair gets s N_d added in lane d.  The sum stays exact modulo 2^32
// because every final lane value lies in [0, 2 kCellBias].
constexpr int kCodeShift = 26;
constexpr uint32_t kIndexMask = (1u << kCodeShift) - 1u;

template <int D>
__device__ __forceinline__ uint32_t wrap_corr(const MPParams &k, uint32_t e)
{
    uint32_t c = 0;
#pragma unroll
    for (int d = 0; d < D; ++d)
    {
        int s = int(e << (4 - 2 * d)) >> 30; // signed two-bit field of axis d
        c += uint32_t(s) * k.wrap[d];
    }
    return c;
}

// Candidate runs of the wrapped window around sub-cell c, pruned as for_each_candidate
// does: run(ax, by, sl, code, b, e) for the candidates [b, e) of one segment of a column,
// with ax, by the column's offset from c before wrapping (c_i - c_j + s N = -ax along x,
// -by along y), sl the image shift along the last axis, and code the per-axis image shifts
// (two bits per axis, two's complement) of the cells the segment's candidates lie in.
template <int D, class R>
__device__ __forceinline__ void for_each_run_periodic(const MeshDev &m, const uint32_t *offset, const int *c,
                                                      const Reach &q, R &&run)
{
    const int NL = m.all_cells[D - 1];
    const float r2 = q.r * q.r;
    auto last_axis = [&](uint32_t base, uint32_t code, float rl, int ax, int by) {
        int l, h;
        axis_reach(q.o[D - 1], q.inv_gs, rl, l, h);
        const int lo = c[D - 1] - l, hi = c[D - 1] + h;
        auto seg = [&](int z0, int z1, int s) {
            const uint32_t cd = code | ((uint32_t(s) & 3u) << (2 * (D - 1)));
            run(ax, by, s, cd, offset[base + uint32_t(z0)], offset[base + uint32_t(z1) + 1]);
        };
        if (lo < 0)
        {
            seg(lo + NL, NL - 1, 1);
            seg(0, hi, 0);
        }
        else if (hi >= NL)
        {
            seg(lo, NL - 1, 0);
            seg(0, hi - NL, -1);
        }
        else
            seg(lo, hi, 0);
    };
    int l0, h0;
    axis_reach(q.o[0], q.inv_gs, q.r, l0, h0);
    for (int a = -l0; a <= h0; ++a)
    {
        const float gx = slab_gap(q.o[0], q.gs, a);
        int x = c[0] + a;
        const int sx = x < 0 ? 1 : (x >= m.all_cells[0] ? -1 : 0);
        x += sx * m.all_cells[0];
        const uint32_t cx = uint32_t(sx) & 3u;
        if (D == 2)
            last_axis(uint32_t(x) * uint32_t(m.all_cells[1]), cx, sqrtf(fmaxf(r2 - gx * gx, 0.0f)), a, 0);
        else
        {
            int l1, h1;
            axis_reach(q.o[1], q.inv_gs, q.r, l1, h1);
            for (int b = -l1; b <= h1; ++b)
            {
                const float gy = slab_gap(q.o[1], q.gs, b);
                const float g2 = gx * gx + gy * gy;
                if (!(g2 < r2))
                    continue;
                int y = c[1] + b;
                const int sy = y < 0 ? 1 : (y >= m.all_cells[1] ? -1 : 0);
                y += sy * m.all_cells[1];
                last_axis((uint32_t(x) * uint32_t(m.all_cells[1]) + uint32_t(y)) * uint32_t(m.all_cells[2]),
                          cx | ((uint32_t(sy) & 3u) << 2), sqrtf(r2 - g2), a, b);
            }
        }
    }
}

// Candidates of the wrapped window one by one: f(j, code) in run order.
template <int D, class F>
__device__ __forceinline__ void for_each_candidate_periodic(const MeshDev &m, const uint32_t *offset, const int *c,
                                                            const Reach &q, F &&f)
{
    for_each_run_periodic<D>(m, offset, c, q, [&](int, int, int, uint32_t code, uint32_t b, uint32_t e) {
        for (uint32_t j = b; j < e; ++j)
            f(j, code);
    });
}

// Same visits as the stored periodic lists, by a sweep of the wrapped window.
template <int D, class Load, class Pair, class Flush>
__device__ __forceinline__ void cell_sweep_periodic(const MeshDev &m, const uint32_t *offset, const int *ci,
                                                    const MPParams &k, uint32_t pib, const float *oi, size_t self,
                                                    const float4 *geo, Load &&load, Pair &&pair, Flush &&flush)
{
    int g = 0;
    for_each_candidate_periodic<D>(m, offset, ci, Reach(oi, k.gs_f, k.rc_reach), [&](uint32_t j, uint32_t code) {
        if (size_t(j) == self && code == 0)
            return;
        const uint32_t e = j | (code << kCodeShift);
        float dx[3];
        geo_dx<D>(k.gs_f, pib + wrap_corr<D>(k, e), oi, geo[j], dx);
        if (!(sq<D>(dx) < k.rc_sqr))
            return;
        pair(load(e));
        if (++g == kGroup)
        {
            flush();
            g = 0;
        }
    });
    flush();
}

struct FirstRecP
{
    float4 g;
    float p;
    uint32_t corr;
};
struct SecondRecP
{
    float4 g, v;
    uint32_t corr;
};

// 1st half of one particle of a periodic flow without walls (Integration1stHalfInnerRiemann):
// pressure force, density-rate dissipation, v += (F_prior + F) / m dt, first position
// half-step.  Returns c0 + |v|.
template <int D, bool LISTS>
__device__ __forceinline__ double first_particle_periodic(size_t i, size_t n, const MPParams &k, const MeshDev &m,
                                                          const uint32_t *f_offset, double dt, const MPState &f,
                                                          const MPNeighbors &in)
{
    const float4 gi = f.geo0[i];
    const uint32_t pib = __float_as_uint(gi.w) + CellLanes<D>::bias;
    int ci[3] = {0, 0, 0};
    if (!LISTS)
        unpack_cell<D>(__float_as_uint(gi.w), ci);
    const float oi[3] = {gi.x, gi.y, gi.z};
    const float4 di = f.dyn[i];
    const float p_i = di.w;
    const float rho_i = k.rho0 + f.drho[i];
    // x and y in packed arithmetic, as first_particle
    const float2 oi01 = make_float2(gi.x, gi.y);
    Acc2 force01;
    Acc force2, rdis;
    auto pair = [&](const FirstRecP &r) {
        float dx[3];
        geo_dx2<D>(k.gs_f, pib + r.corr, oi01, oi[2], r.g, dx);
        float r2 = sq<D>(dx);
        float inv = inv_dist(r2);
        float dWV = wc2_dWV(k.cW, k.inv_h, r2 * inv);
        float sc = (p_i + r.p) * (dWV * inv);
        force01.fma(make_float2(-sc, -sc), make_float2(dx[0], dx[1]));
        if (D == 3)
            force2.add(-sc * dx[2]);
        rdis.add((p_i - r.p) * dWV);
    };
    auto flush = [&]() {
        force01.flush();
        if (D == 3)
            force2.flush();
        rdis.flush();
    };
    auto load = [&](uint32_t e) {
        const uint32_t j = e & kIndexMask;
        return FirstRecP{__ldg(&f.geo0[j]), __ldg(&f.pres[j]), wrap_corr<D>(k, e)};
    };
    if (LISTS)
        list_sweep<true, kUnrollFirst>(i, n, in, load, pair, flush);
    else
        cell_sweep_periodic<D>(m, f_offset, ci, k, pib, oi, i, f.geo0, load, pair, flush);

    f.drho_dt[i] = (rdis.value() * k.inv_z) * rho_i;
    float v2 = 0.f;
    float vn[3] = {di.x, di.y, di.z};
    const float dt_f = float(dt);
    const float fv[3] = {force01.x(), force01.y(), force2.value()};
#pragma unroll
    for (int d = 0; d < D; ++d)
    {
        float F = f.force[d * n + i] + fv[d] * k.Vol;
        f.force[d * n + i] = F;
        float vo = vn[d];
        half_step(f, n, i, d, dt, vo);
        vn[d] = vo + (f.fprior[d * n + i] + F) * k.inv_mass * dt_f;
        v2 += vn[d] * vn[d];
    }
    f.dyn[i] = make_float4(vn[0], vn[1], D == 3 ? vn[2] : 0.f, p_i);
    return k.c0 + double(sqrtf(v2));
}

// 2nd half of one particle of a periodic flow: Integration2ndHalfInnerRiemann (RIEMANN),
// or Integration2ndHalfInnerNoRiemann, whose pressure dissipation is zero, so the force
// sum is left out.  Returns max(|v|^2, 4 h |F + F_prior| / m).
template <int D, bool LISTS, bool RIEMANN>
__device__ __forceinline__ double second_particle_periodic(size_t i, size_t n, const MPParams &k, const MeshDev &m,
                                                           const uint32_t *f_offset, double dt, const MPState &f,
                                                           const MPNeighbors &in)
{
    const float4 gi = f.geo0[i];
    const uint32_t pib = __float_as_uint(gi.w) + CellLanes<D>::bias;
    int ci[3] = {0, 0, 0};
    if (!LISTS)
        unpack_cell<D>(__float_as_uint(gi.w), ci);
    const float oi[3] = {gi.x, gi.y, gi.z};
    const float4 di = f.dyn[i];
    const float vi[3] = {di.x, di.y, di.z};
    const float rho_i = k.rho0 + f.drho[i];
    // SPHX_PACKED_PERIODIC_SECOND: x and y of the geometry and the velocity difference in
    // packed arithmetic; held to 48 registers 3 % faster than the scalar form (unbounded,
    // at 52 registers, 10 % slower)
    const float2 oi01 = make_float2(gi.x, gi.y), vi01 = make_float2(di.x, di.y);
    Acc rate, pdis[3];
    auto pair = [&](const SecondRecP &r) {
        float dx[3];
        float dv[3];
        if (SPHX_PACKED_PERIODIC_SECOND)
        {
            geo_dx2<D>(k.gs_f, pib + r.corr, oi01, oi[2], r.g, dx);
            const float2 dv01 = f2_sub(vi01, make_float2(r.v.x, r.v.y));
            dv[0] = dv01.x;
            dv[1] = dv01.y;
        }
        else
        {
            geo_dx<D>(k.gs_f, pib + r.corr, oi, r.g, dx);
            dv[0] = vi[0] - r.v.x;
            dv[1] = vi[1] - r.v.y;
        }
        dv[2] = vi[2] - r.v.z;
        float r2 = sq<D>(dx);
        float inv = inv_dist(r2);
        float dWV = wc2_dWV(k.cW, k.inv_h, r2 * inv);
        float u = dot<D>(dv, dx) * inv;
        rate.add(u * dWV);
        if (RIEMANN)
        {
            float sc = p_jump(k, u) * (dWV * inv);
#pragma unroll
            for (int d = 0; d < D; ++d)
                pdis[d].add(sc * dx[d]);
        }
    };
    auto flush = [&]() {
        rate.flush();
        if (RIEMANN)
#pragma unroll
            for (int d = 0; d < D; ++d)
                pdis[d].flush();
    };
    auto load = [&](uint32_t e) {
        const uint32_t j = e & kIndexMask;
        return SecondRecP{__ldg(&f.geo0[j]), __ldg(&f.dyn[j]), wrap_corr<D>(k, e)};
    };
    if (LISTS)
        list_sweep<false, kUnrollSecond>(i, n, in, load, pair, flush);
    else
        cell_sweep_periodic<D>(m, f_offset, ci, k, pib, oi, i, f.geo0, load, pair, flush);

    float drho_dt = f.drho_dt[i] + rate.value() * rho_i;
    f.drho_dt[i] = drho_dt;
    f.drho[i] = f.drho[i] + drho_dt * float(0.5 * dt);
    float v2 = 0.f, a2 = 0.f;
#pragma unroll
    for (int d = 0; d < D; ++d)
    {
        float F = pdis[d].value() * k.Vol;
        f.force[d * n + i] = F;
        half_step(f, n, i, d, dt, vi[d]);
        v2 += vi[d] * vi[d];
        float ft = F + f.fprior[d * n + i];
        a2 += ft * ft;
    }
    return double(fmaxf(v2, 4.0f * float(k.h) * sqrtf(a2) * k.inv_mass));
}

// Configuration of one particle of a periodic flow, with the interactions that use only
// the configuration and the velocity of the step start, in the reference's order:
// DensitySummationInner (sum only; rho = rho_sum is set at the step start),
// ViscousForceInner (fixed viscosity; ForcePrior = the viscous force, the only prior
// force of the flow), TransportVelocityCorrectionInner (the position shift, applied at the
// step start so that a repeated build after a list regrowth does not apply it twice).
template <int D>
__device__ __forceinline__ void build_particle_periodic(size_t i, size_t n, const MPParams &k, const MeshDev &m,
                                                        const uint32_t *f_offset, const MPState &f,
                                                        const MPNeighbors &in, unsigned int *max_counts)
{
    const float4 gi = f.geo0[i];
    const uint32_t pib = __float_as_uint(gi.w) + CellLanes<D>::bias;
    int ci[3] = {0, 0, 0};
    unpack_cell<D>(__float_as_uint(gi.w), ci);
    const float oi[3] = {gi.x, gi.y, gi.z};
    unsigned cnt = 0;
    // per segment the cell differences of the column axes are -ax, -by and the last axis's
    // is c_i + sl N - c_j: only the last lane is decoded per candidate (the exact integer
    // differences geo_dx forms from the shifted lanes, so the same dx bit for bit)
    const int NL = m.all_cells[D - 1];
    for_each_run_periodic<D>(m, f_offset, ci, Reach(oi, k.gs_f, k.rc_reach),
                             [&](int ax, int by, int sl, uint32_t code, uint32_t b, uint32_t e) {
                                 const float dcx = float(-ax), dcy = float(-by);
                                 const float kl = 8388608.0f + float(ci[D - 1] + sl * NL);
                                 const uint32_t hi = code << kCodeShift;
                                 for (uint32_t j = b; j < e; ++j)
                                 {
                                     if (j == uint32_t(i) && code == 0)
                                         continue;
                                     const float4 gj = f.geo0[j];
                                     const uint32_t lane = (__float_as_uint(gj.w) >> ((D - 1) * CellLanes<D>::bits)) &
                                                           CellLanes<D>::mask;
                                     const float dcl = kl - __uint_as_float(0x4B000000u | lane);
                                     float dx[3];
                                     dx[0] = fmaf(dcx, k.gs_f, oi[0] - gj.x);
                                     if (D == 3)
                                     {
                                         dx[1] = fmaf(dcy, k.gs_f, oi[1] - gj.y);
                                         dx[2] = fmaf(dcl, k.gs_f, oi[2] - gj.z);
                                     }
                                     else
                                         dx[1] = fmaf(dcl, k.gs_f, oi[1] - gj.y);
                                     if (!(sq<D>(dx) < k.rc_sqr))
                                         continue;
                                     if (cnt < in.cap)
                                         in.J[size_t(cnt) * n + i] = j | hi;
                                     ++cnt;
                                 }
                             });
    in.count[i] = cnt;
    warp_atomic_max(&max_counts[0], cnt);
    // Two phases: the candidate loop above only tests and stores (the lanes of a warp
    // accept different candidates, and a warp runs the accepting branch whenever any lane
    // takes it); each lane now runs the kernel sums over its own stored entries, in the
    // stored order (written by this thread in this kernel: plain loads).  An overflowed
    // list is rebuilt by the caller with a larger capacity, so the sums of that pass are
    // discarded.  (16 % faster per advection step at 256^3 than one pass.)
    const float4 di = f.dyn[i];
    const float vi[3] = {di.x, di.y, di.z};
    Kahan sigma;
    Acc visc[3], tvc[3];
    const unsigned c = min(cnt, in.cap);
    for (unsigned s = 0; s < c; ++s)
    {
        const uint32_t e = in.J[size_t(s) * n + i];
        const uint32_t j = e & kIndexMask;
        float dx[3];
        geo_dx<D>(k.gs_f, pib + wrap_corr<D>(k, e), oi, f.geo0[j], dx);
        float r2 = sq<D>(dx);
        float inv = inv_dist(r2);
        float r = r2 * inv;
        sigma.add(wc2_W(k.fW, k.inv_h, r));
        float dWV = wc2_dWV(k.cW, k.inv_h, r);
        const float4 vj = __ldg(&f.dyn[j]);
        const float dv[3] = {vi[0] - vj.x, vi[1] - vj.y, vi[2] - vj.z};
        // e_ij . (B_i + B_j) e_ij = 2 without kernel correction
        float cv = k.mu2 * dWV / (r + k.eps_h);
        float ct = dWV * inv;
#pragma unroll
        for (int d = 0; d < D; ++d)
        {
            visc[d].add(cv * dv[d]);
            tvc[d].add(ct * dx[d]);
        }
        if ((s + 1) % kGroup == 0)
        {
#pragma unroll
            for (int d = 0; d < D; ++d)
            {
                visc[d].flush();
                tvc[d].flush();
            }
        }
    }
    double dsig = (double(sigma.s) - k.sigma0) - double(sigma.c) + double(k.fW);
    f.drho_sum[i] = float(dsig) * k.rho0_over_sigma0;
    float inc[3] = {0.f, 0.f, 0.f}, inc2 = 0.f;
#pragma unroll
    for (int d = 0; d < D; ++d)
    {
        visc[d].flush();
        tvc[d].flush();
        f.fprior[d * n + i] = visc[d].value() * k.Vol;
        inc[d] = -2.0f * tvc[d].value();
        inc2 += inc[d] * inc[d];
    }
    const float lim = fminf(k.tvc_lim * inc2, 1.0f);
#pragma unroll
    for (int d = 0; d < D; ++d)
        f.shift[d * n + i] = k.tvc_scale * lim * inc[d];
}

// Acoustic and advection maxima of the initial state (FP64).
template <int D>
__device__ __forceinline__ void initial_max(size_t i, size_t n, const MPParams &k, const double *gd, const MPState &f,
                                            double *vm, double *am)
{
    float4 di = f.dyn[i];
    const float vv[3] = {di.x, di.y, di.z};
    double v2 = 0, a2 = 0;
#pragma unroll
    for (int d = 0; d < D; ++d)
    {
        v2 += double(vv[d]) * double(vv[d]);
        double ft = double(f.force[d * n + i]) + (f.fprior ? double(f.fprior[d * n + i]) : double(k.mass) * gd[d]);
        a2 += ft * ft;
    }
    *vm = k.c0 + sqrt(v2);
    *am = fmax(v2, 4.0 * k.h * sqrt(a2) * double(k.inv_mass));
}
} // namespace mpc
} // namespace sphx
