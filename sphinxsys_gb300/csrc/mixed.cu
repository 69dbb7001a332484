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
#include "mp_tiled.cuh"
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
// Particles [first, end) of n (a chunk of the rows, or all of them).
__global__ void k_mp_from_fp64(size_t n, size_t first, size_t end, const double *__restrict__ pos,
                               size_t comp_stride, size_t row_stride, MPConst k, uint32_t *__restrict__ ncell,
                               float *__restrict__ noff, uint32_t *__restrict__ key, uint32_t *__restrict__ rank,
                               uint32_t *__restrict__ count)
{
    size_t i = first + size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= end)
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
        stage_offset(noff, n, i, d, x[d] - cell_corner(m, d, c[d]));
    ncell[i] = pack_cell<D>(c);
    uint32_t lc = linear_cell<D>(m, c);
    key[i] = lc;
    rank[i] = atomicAdd(&count[lc], 1u);
}

// FP64 reconstruction of a position from its (cell, offset) pair.  A periodic flow wraps
// it into its box, as PeriodicBounding does at the end of the advection step
// (domain_bounding.h:103-113); between the position update and the next re-hash the
// offset may still point outside the box.
__device__ __forceinline__ double reconstruct(const MPConst &k, int d, int cell, double offset)
{
    double x = cell_corner(k.m, d, cell) + offset;
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
__global__ void k_mp_rehash(size_t n, MPFluid f, MPConst k, uint32_t *__restrict__ ncell, float *__restrict__ noff,
                            uint32_t *__restrict__ key, uint32_t *__restrict__ rank, uint32_t *__restrict__ count)
{
    size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    const MeshDev &m = k.m;
    int c0[3];
    unpack_cell<D>(__float_as_uint(f.geo0[i].w), c0);
    int c[3] = {0, 0, 0};
    rehash_particle<D>(m, k.inv_gs, k.p.gs_f, k.periodic != 0, f, n, i, c0, c, noff);
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
    if (c < nseg)
        sort_segment(idx, offset[c], offset[c + 1]);
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
        dst.off_lo[d * n + k] = noff[(3 + d) * n + i];
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
// Particle handled by thread t: t itself, or the t-th particle of the tile-grouped order.
template <bool ORDER>
__device__ __forceinline__ size_t particle_of(size_t t, const uint32_t *__restrict__ order)
{
    return ORDER ? size_t(__ldg(&order[t])) : t;
}

// Blocks of 256 per SM the configuration build is compiled to fit (6: 40 registers,
// advection step 9.61 -> 9.52 ms at dp = 0.006 against the unbounded 48; 0: no bound): a
// build-time tuning parameter.
#ifndef SPHX_BUILD_MINB
#define SPHX_BUILD_MINB 6
#endif
#if SPHX_BUILD_MINB > 0
#define SPHX_BUILD_BOUNDS __launch_bounds__(256, SPHX_BUILD_MINB)
#else
#define SPHX_BUILD_BOUNDS
#endif

template <int D, bool ORDER>
__global__ void SPHX_BUILD_BOUNDS k_mp_build(size_t n, MPConst k, MPFluid f, const uint32_t *__restrict__ f_offset, MPWall w,
               const uint32_t *__restrict__ w_offset, MPLists in, MPLists wl, unsigned int *max_counts,
               const uint32_t *__restrict__ order)
{
    size_t t = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (t < n)
        build_particle<D>(particle_of<ORDER>(t, order), n, k.p, Visit{k.m, 0u, f_offset, w_offset}, f, w, in, wl,
                          max_counts);
}

// Tile key of every particle (cell order) for the tile-grouped traversal order.
template <int D>
__global__ void k_mp_tile_key(size_t n, const float4 *__restrict__ geo0, TileShape ts, uint32_t *__restrict__ key,
                              uint32_t *__restrict__ rank, uint32_t *__restrict__ count)
{
    size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    int c[3];
    unpack_cell<D>(__float_as_uint(geo0[i].w), c);
    const uint32_t t = tile_key<D>(ts, c);
    key[i] = t;
    rank[i] = atomicAdd(&count[t], 1u);
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
        store_offset(f, n, i, d, offset_of(f, n, i, d) + double(f.shift[d * n + i]));
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
                           float4 *__restrict__ dyn, float *__restrict__ pres, float p0_over_rho0, float half_dt)
{
    size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    float r = drho[i] + drho_dt[i] * half_dt;
    drho[i] = r;
    const float p = p0_over_rho0 * r;
    reinterpret_cast<float *>(dyn)[4 * i + 3] = p;
    pres[i] = p;
}

// at most 64 registers: 4 blocks of 256 threads per SM
// ---------------------------------------------------------------- tiled strategy
// Non-empty tiles of the tile-grouped order, compacted (tile_pos = exclusive scan of flags).
__global__ void k_mp_tile_flags(size_t nt, const uint32_t *__restrict__ tile_offset, uint32_t *__restrict__ flags)
{
    size_t t = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (t < nt)
        flags[t] = tile_offset[t + 1] > tile_offset[t] ? 1u : 0u;
}

__global__ void k_mp_tile_compact(size_t nt, const uint32_t *__restrict__ flags, const uint32_t *__restrict__ pos,
                                  uint32_t *__restrict__ tiles, unsigned int *count)
{
    size_t t = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (t >= nt)
        return;
    if (flags[t])
        tiles[pos[t]] = uint32_t(t);
    if (t == nt - 1)
        *count = pos[t] + flags[t];
}

// Largest window population (fluid, wall) over the non-empty tiles: one warp per tile.
template <int D>
__global__ void k_mp_tile_population(const unsigned int *ntiles, MeshDev m, TileShape ts,
                                     const uint32_t *__restrict__ tiles, const uint32_t *__restrict__ f_offset,
                                     const uint32_t *__restrict__ w_offset, unsigned int *maxes)
{
    const unsigned warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31u;
    if (warp >= *ntiles)
        return;
    Window<D> w;
    tile_window<D>(m, ts, tiles[warp], w);
    unsigned nf = 0, nw = 0;
    for (int col = int(lane); col < w.ncol; col += 32)
    {
        uint32_t a, b;
        column_cells<D>(m, w, col, a, b);
        nf += f_offset[b + 1] - f_offset[a];
        nw += w_offset[b + 1] - w_offset[a];
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
    {
        nf += __shfl_down_sync(0xffffffffu, nf, o);
        nw += __shfl_down_sync(0xffffffffu, nw, o);
    }
    if (lane == 0)
    {
        atomicMax(&maxes[0], nf);
        atomicMax(&maxes[1], nw);
    }
}

// Shared-memory layout of a tiled kernel: run tables, then the record arrays (sizes from the
// largest window: cap_f fluid and cap_w wall records).
struct TiledSmem
{
    uint32_t fbeg[kTileMaxCols], fbase[kTileMaxCols + 1], wbeg[kTileMaxCols], wbase[kTileMaxCols + 1], total[2];
};

// Sets up the window of this block's tile and its run tables; false if the window exceeds
// the staged capacity (never for capacities from k_mp_tile_population; the block then
// records the overflow and skips its tile).
template <int D>
__device__ __forceinline__ bool tiled_setup(const MeshDev &m, const TileGrid &g, const uint32_t *f_offset,
                                            const uint32_t *w_offset, unsigned cap_f, unsigned cap_w, TiledSmem &t,
                                            Staged<D> &sw, unsigned int *overflow)
{
    tile_window<D>(m, g.ts, g.tiles[blockIdx.x], sw.w);
    const uint32_t nf = window_table<D>(m, sw.w, f_offset, t.fbeg, t.fbase, &t.total[0]);
    const uint32_t nw = window_table<D>(m, sw.w, w_offset, t.wbeg, t.wbase, &t.total[1]);
    sw.fbeg = t.fbeg;
    sw.fbase = t.fbase;
    sw.wbeg = t.wbeg;
    sw.wbase = t.wbase;
    if (nf > cap_f || nw > cap_w)
    {
        if (threadIdx.x == 0)
            atomicAdd(overflow, 1u);
        return false;
    }
    return true;
}

template <int D>
__global__ void __launch_bounds__(256) k_mp_build_tiled(size_t n, MPConst k, MPFluid f,
                                                        const uint32_t *__restrict__ f_offset, MPWall w,
                                                        const uint32_t *__restrict__ w_offset, TileGrid g, MPLists in,
                                                        MPLists wl, unsigned int *max_counts, unsigned cap_f,
                                                        unsigned cap_w, unsigned int *overflow)
{
    extern __shared__ float4 dyn_smem[];
    __shared__ TiledSmem t;
    Staged<D> sw;
    if (!tiled_setup<D>(k.m, g, f_offset, w_offset, cap_f, cap_w, t, sw, overflow))
        return;
    float4 *fa = dyn_smem, *wa = dyn_smem + cap_f;
    for_each_staged<D>(sw.w, t.fbeg, t.fbase, [&](uint32_t j, uint32_t s) { fa[s] = f.geo0[j]; });
    for_each_staged<D>(sw.w, t.wbeg, t.wbase, [&](uint32_t j, uint32_t s) { wa[s] = w.geo[j]; });
    sw.fa = fa;
    sw.wa = wa;
    __syncthreads();
    const uint32_t tile = g.tiles[blockIdx.x];
    const uint32_t te = g.tile_offset[tile + 1];
    for (uint32_t q = g.tile_offset[tile] + threadIdx.x; q < te; q += blockDim.x)
        build_particle_tiled<D>(q, g.order[q], n, k.p, k.m, sw, f_offset, w_offset, f, in, wl, max_counts);
}

template <int D>
__global__ void __launch_bounds__(256) k_mp_first_tiled(size_t n, MPConst k, MPFluid f,
                                                        const uint32_t *__restrict__ f_offset, MPWall w,
                                                        const uint32_t *__restrict__ w_offset, TileGrid g, MPLists in,
                                                        MPLists wl, double dt, unsigned long long *ac_slot,
                                                        unsigned cap_f, unsigned cap_w, unsigned int *overflow)
{
    extern __shared__ float4 dyn_smem[];
    __shared__ TiledSmem t;
    Staged<D> sw;
    double vmax = -1.0e300;
    if (tiled_setup<D>(k.m, g, f_offset, w_offset, cap_f, cap_w, t, sw, overflow))
    {
        float4 *fa = dyn_smem, *fb = fa + cap_f, *wa = fb + cap_f, *wb = wa + cap_w;
        const Window<D> &win = sw.w;
        for_each_staged<D>(win, t.fbeg, t.fbase, [&](uint32_t j, uint32_t s) {
            const float4 gj = f.geo0[j];
            fa[s] = make_float4(gj.x, gj.y, gj.z, __ldg(&f.pres[j]));
            fb[s] = window_cell<D>(win, __float_as_uint(gj.w));
        });
        for_each_staged<D>(win, t.wbeg, t.wbase, [&](uint32_t j, uint32_t s) {
            const float4 gj = w.geo[j];
            wa[s] = gj;
            wb[s] = window_cell<D>(win, __float_as_uint(gj.w));
        });
        sw.fa = fa;
        sw.fb = fb;
        sw.wa = wa;
        sw.wb = wb;
        __syncthreads();
        in.limit = t.total[0]; // the entries index the staged records
        wl.limit = t.total[1];
        const uint32_t tile = g.tiles[blockIdx.x];
        const uint32_t te = g.tile_offset[tile + 1];
        for (uint32_t q = g.tile_offset[tile] + threadIdx.x; q < te; q += blockDim.x)
            vmax = fmax(vmax, first_particle_tiled<D>(q, g.order[q], n, k.p, sw, dt, f, in, wl));
    }
    warp_max_to(ac_slot, vmax);
}

template <int D>
__global__ void __launch_bounds__(256) k_mp_second_tiled(size_t n, MPConst k, MPFluid f,
                                                         const uint32_t *__restrict__ f_offset, MPWall w,
                                                         const uint32_t *__restrict__ w_offset, TileGrid g,
                                                         MPLists in, MPLists wl, double dt,
                                                         unsigned long long *adv_slot, unsigned cap_f, unsigned cap_w,
                                                         unsigned int *overflow)
{
    extern __shared__ float4 dyn_smem[];
    __shared__ TiledSmem t;
    Staged<D> sw;
    double amax = -1.0e300;
    if (tiled_setup<D>(k.m, g, f_offset, w_offset, cap_f, cap_w, t, sw, overflow))
    {
        float4 *fa = dyn_smem, *fb = fa + cap_f, *wa = fb + cap_f, *wb = wa + cap_w;
        float *fc = reinterpret_cast<float *>(wb + cap_w), *wc = fc + cap_f;
        const Window<D> &win = sw.w;
        for_each_staged<D>(win, t.fbeg, t.fbase, [&](uint32_t j, uint32_t s) {
            const float4 gj = f.geo0[j], vj = f.dyn[j];
            float4 c = window_cell<D>(win, __float_as_uint(gj.w));
            c.w = vj.y;
            fa[s] = make_float4(gj.x, gj.y, gj.z, vj.x);
            fb[s] = c;
            fc[s] = vj.z;
        });
        for_each_staged<D>(win, t.wbeg, t.wbase, [&](uint32_t j, uint32_t s) {
            const float4 gj = w.geo[j], nj = w.n[j];
            float4 c = window_cell<D>(win, __float_as_uint(gj.w));
            c.w = nj.y;
            wa[s] = make_float4(gj.x, gj.y, gj.z, nj.x);
            wb[s] = c;
            wc[s] = nj.z;
        });
        sw.fa = fa;
        sw.fb = fb;
        sw.fc = fc;
        sw.wa = wa;
        sw.wb = wb;
        sw.wc = wc;
        __syncthreads();
        in.limit = t.total[0];
        wl.limit = t.total[1];
        const uint32_t tile = g.tiles[blockIdx.x];
        const uint32_t te = g.tile_offset[tile + 1];
        for (uint32_t q = g.tile_offset[tile] + threadIdx.x; q < te; q += blockDim.x)
            amax = fmax(amax, second_particle_tiled<D>(q, g.order[q], n, k.p, sw, dt, f, in, wl));
    }
    warp_max_to(adv_slot, amax);
}

// ---------------------------------------------------------------- asynchronous gathers (strategy 3)
// The stored lists of strategy 0 with the neighbour records copied by cp.async into a
// per-thread ring in dynamic shared memory (DEPTH slots): same lists, order and arithmetic,
// so the results are those of strategy 0 bit for bit.
constexpr int kAsyncDepthFirst = 8, kAsyncDepthSecond = 8;

// Ring layout in the dynamic shared memory, DEPTH x blockDim slots per part:
// two parts (2nd half): a (16 B), b (16 B), idx (4 B) = 36 B per slot;
// one part (1st half): a (16 B), c (4 B), idx (4 B) = 24 B per slot (async_ring_bytes).
template <int DEPTH>
__device__ __forceinline__ AsyncRing<DEPTH> async_ring(void *smem, bool two_parts)
{
    AsyncRing<DEPTH> r;
    r.tid = threadIdx.x;
    r.bd = blockDim.x;
    const size_t slots = size_t(DEPTH) * blockDim.x;
    r.a = static_cast<float4 *>(smem);
    if (two_parts)
    {
        r.b = r.a + slots;
        r.c = nullptr;
        r.idx = reinterpret_cast<uint32_t *>(r.b + slots);
    }
    else
    {
        r.b = nullptr;
        r.c = reinterpret_cast<float *>(r.a + slots);
        r.idx = reinterpret_cast<uint32_t *>(r.c + slots);
    }
    return r;
}

template <int D, int DEPTH>
__global__ void __launch_bounds__(256) k_mp_first_async(size_t n, MPConst k, MPFluid f, MPWall w, MPLists in,
                                                        MPLists wl, double dt, unsigned long long *ac_slot)
{
    extern __shared__ float4 ring_smem[];
    const AsyncRing<DEPTH> ring = async_ring<DEPTH>(ring_smem, false);
    size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    double vmax = -1.0e300;
    if (i < n)
        vmax = first_particle<D, true, DEPTH>(i, n, k.p, Visit{k.m, 0u, nullptr, nullptr}, dt, f, w, in, wl, &ring);
    warp_max_to(ac_slot, vmax);
}

template <int D, int DEPTH>
__global__ void __launch_bounds__(256) k_mp_second_async(size_t n, MPConst k, MPFluid f, MPWall w, MPLists in,
                                                         MPLists wl, double dt, unsigned long long *adv_slot)
{
    extern __shared__ float4 ring_smem[];
    const AsyncRing<DEPTH> ring = async_ring<DEPTH>(ring_smem, true);
    size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    double amax = -1.0e300;
    if (i < n)
        amax = second_particle<D, true, DEPTH>(i, n, k.p, Visit{k.m, 0u, nullptr, nullptr}, dt, f, w, in, wl, &ring);
    warp_max_to(adv_slot, amax);
}

// Ring bytes per block (the layout of async_ring): 1st half 16 (geo0) + 4 (pressure) + 4
// (list entry), 2nd half 16 (geo0) + 16 (dyn) + 4 (list entry) per slot.
inline size_t async_ring_bytes(bool second, unsigned blk)
{
    return second ? size_t(kAsyncDepthSecond) * blk * (16 + 16 + 4) : size_t(kAsyncDepthFirst) * blk * (16 + 4 + 4);
}

// ---------------------------------------------------------------- persistent warps (strategy 4)
// The stored lists of strategy 0 with a grid of the resident capacity: each warp takes the
// next chunk of 32 consecutive particles from a counter until all are done, so no warp slot
// idles while a block waits for its slowest warp or while the last wave drains.  The same
// per-particle work: results equal strategy 0 bit for bit (the time-step maxima are exact
// maxima, independent of the order).
__device__ __forceinline__ size_t next_chunk(unsigned int *counter)
{
    unsigned c = 0;
    if ((threadIdx.x & 31u) == 0)
        c = atomicAdd(counter, 1u);
    return size_t(__shfl_sync(0xffffffffu, c, 0)) * 32u;
}

// Blocks of 256 the persistent 1st half is compiled to fit per SM (4: 64 registers with some
// spills; 3: ~80 registers without): a build-time tuning parameter.
#ifndef SPHX_PERSISTENT_FIRST_MINB
#define SPHX_PERSISTENT_FIRST_MINB 4
#endif

template <int D>
__global__ void __launch_bounds__(256, SPHX_PERSISTENT_FIRST_MINB) k_mp_first_persistent(size_t n, MPConst k, MPFluid f, MPWall w, MPLists in,
                                                             MPLists wl, double dt, unsigned long long *ac_slot,
                                                             unsigned int *counter)
{
    double vmax = -1.0e300;
    for (size_t base = next_chunk(counter); base < n; base = next_chunk(counter))
    {
        const size_t i = base + (threadIdx.x & 31u);
        if (i < n)
            vmax = fmax(vmax, first_particle<D, true>(i, n, k.p, Visit{k.m, 0u, nullptr, nullptr}, dt, f, w, in, wl));
    }
    warp_max_to(ac_slot, vmax);
}

template <int D>
__global__ void __launch_bounds__(256) k_mp_second_persistent(size_t n, MPConst k, MPFluid f, MPWall w, MPLists in,
                                                              MPLists wl, double dt, unsigned long long *adv_slot,
                                                              unsigned int *counter)
{
    double amax = -1.0e300;
    for (size_t base = next_chunk(counter); base < n; base = next_chunk(counter))
    {
        const size_t i = base + (threadIdx.x & 31u);
        if (i < n)
            amax = fmax(amax, second_particle<D, true>(i, n, k.p, Visit{k.m, 0u, nullptr, nullptr}, dt, f, w, in, wl));
    }
    warp_max_to(adv_slot, amax);
}

// ---------------------------------------------------------------- lanes per particle (strategies 5, 6)
// The stored lists of strategy 0 with LANES (2 or 4) consecutive lanes on each particle,
// 32 / LANES particles per warp: the lanes split the list slots (lane s takes slots s,
// s + LANES, ...), so a warp walks lists LANES times shorter and the lanes of a warp wait
// on fewer ragged list lengths.  Each lane keeps its own compensated sums, combined by warp
// shuffles at the end: a different summation order from strategy 0, so the results agree
// to FP32 rounding, not bit for bit.
template <int D, int LANES>
__global__ void __launch_bounds__(256, 4) k_mp_first_lanes(size_t n, MPConst k, MPFluid f, MPWall w, MPLists in,
                                                           MPLists wl, double dt, unsigned long long *ac_slot)
{
    const size_t t = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    double vmax = -1.0e300;
    if (t / LANES < n) // whole groups: blocks hold a multiple of LANES threads
        vmax = first_particle<D, true, 0, LANES>(t / LANES, n, k.p, Visit{k.m, 0u, nullptr, nullptr}, dt, f, w, in,
                                                 wl);
    warp_max_to(ac_slot, vmax);
}

template <int D, int LANES>
__global__ void k_mp_second_lanes(size_t n, MPConst k, MPFluid f, MPWall w, MPLists in, MPLists wl, double dt,
                                  unsigned long long *adv_slot)
{
    const size_t t = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    double amax = -1.0e300;
    if (t / LANES < n)
        amax = second_particle<D, true, 0, LANES>(t / LANES, n, k.p, Visit{k.m, 0u, nullptr, nullptr}, dt, f, w,
                                                  in, wl);
    warp_max_to(adv_slot, amax);
}

// Lanes per particle of strategies 5 and 6 (0 for the others).
inline int strategy_lanes(int strategy) { return strategy == 5 ? 2 : (strategy == 6 ? 4 : 0); }

// Blocks of 256 threads per SM the stored-list / cell sweeps are compiled to fit (the
// register cap follows: 4 -> 64, 5 -> 48 registers; 0 leaves the 2nd half unbounded: with
// the packed x / y arithmetic it would take 66): build-time tuning parameters.
#ifndef SPHX_FIRST_MINB
#define SPHX_FIRST_MINB 4
#endif
#ifndef SPHX_SECOND_MINB
#define SPHX_SECOND_MINB 4
#endif
#if SPHX_SECOND_MINB > 0
#define SPHX_SECOND_BOUNDS __launch_bounds__(256, SPHX_SECOND_MINB)
#else
#define SPHX_SECOND_BOUNDS
#endif
// Register caps of the sweeps independent of the block size (0: from the bounds above).
#ifndef SPHX_FIRST_MAXNREG
#define SPHX_FIRST_MAXNREG 0
#endif
#ifndef SPHX_SECOND_MAXNREG
#define SPHX_SECOND_MAXNREG 0
#endif
#if SPHX_FIRST_MAXNREG > 0
#define SPHX_FIRST_ATTR __maxnreg__(SPHX_FIRST_MAXNREG)
#else
#define SPHX_FIRST_ATTR __launch_bounds__(256, SPHX_FIRST_MINB)
#endif
#if SPHX_SECOND_MAXNREG > 0
#define SPHX_SECOND_ATTR __maxnreg__(SPHX_SECOND_MAXNREG)
#else
#define SPHX_SECOND_ATTR SPHX_SECOND_BOUNDS
#endif

template <int D, bool LISTS, bool ORDER>
__global__ void SPHX_FIRST_ATTR k_mp_first(size_t n, MPConst k, MPFluid f, const uint32_t *__restrict__ f_offset, MPWall w,
               const uint32_t *__restrict__ w_offset, MPLists in, MPLists wl, double dt,
               unsigned long long *ac_slot, const uint32_t *__restrict__ order)
{
    size_t t = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    double vmax = -1.0e300;
    if (t < n)
        vmax = first_particle<D, LISTS>(particle_of<ORDER>(t, order), n, k.p, Visit{k.m, 0u, f_offset, w_offset}, dt,
                                        f, w, in, wl);
    warp_max_to(ac_slot, vmax);
}

template <int D, bool LISTS, bool ORDER>
__global__ void SPHX_SECOND_ATTR k_mp_second(size_t n, MPConst k, MPFluid f, const uint32_t *__restrict__ f_offset, MPWall w,
                const uint32_t *__restrict__ w_offset, MPLists in, MPLists wl, double dt,
                unsigned long long *adv_slot, const uint32_t *__restrict__ order)
{
    size_t t = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    double amax = -1.0e300;
    if (t < n)
        amax = second_particle<D, LISTS>(particle_of<ORDER>(t, order), n, k.p, Visit{k.m, 0u, f_offset, w_offset},
                                         dt, f, w, in, wl);
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

// Blocks of 256 per SM the periodic 2nd half is compiled to fit (5: 48 registers; 0: no
// bound).
#ifndef SPHX_PERIODIC_SECOND_MINB
#define SPHX_PERIODIC_SECOND_MINB 5
#endif
#if SPHX_PERIODIC_SECOND_MINB > 0
#define SPHX_PERIODIC_SECOND_BOUNDS __launch_bounds__(256, SPHX_PERIODIC_SECOND_MINB)
#else
#define SPHX_PERIODIC_SECOND_BOUNDS
#endif

template <int D, bool LISTS, bool RIEMANN>
__global__ void SPHX_PERIODIC_SECOND_BOUNDS k_mp_second_periodic(size_t n, MPConst k, MPFluid f, const uint32_t *__restrict__ f_offset,
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
        dst.off_lo[d * n + k] = noff[(3 + d) * n + i];
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
    return reconstruct(k, d, c[d], offset_of(f, n, i, d));
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
// in the body's particle order, the values k_mp_download writes.  ROWS selects them:
// kRowsAll, kRowsVelocity (velocity and pressure, final once the last 1st half has run)
// or kRowsPosition (position and density, final after the 2nd half).
constexpr int kRowsAll = 3, kRowsVelocity = 1, kRowsPosition = 2;
template <int D, int ROWS>
__global__ void k_mp_export_rows(size_t n, MPConst k, MPFluid f, double *__restrict__ pos, double *__restrict__ vel,
                                 double *__restrict__ rho, double *__restrict__ p)
{
    size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    uint32_t o = f.id[i];
    if (ROWS & kRowsPosition)
    {
        int c[3];
        unpack_cell<D>(__float_as_uint(f.geo0[i].w), c);
#pragma unroll
        for (int d = 0; d < D; ++d)
            pos[size_t(o) * D + d] = position(k, f, n, i, d, c);
        rho[o] = double(k.p.rho0) + double(f.drho[i]);
    }
    if (ROWS & kRowsVelocity)
    {
        float4 di = f.dyn[i];
        const float v[3] = {di.x, di.y, di.z};
#pragma unroll
        for (int d = 0; d < D; ++d)
            vel[size_t(o) * D + d] = v[d];
        p[o] = di.w;
    }
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

// State check (sphx_mp_check_state): counts particles with a non-finite value in any
// evolving field (offset, velocity, pressure, density, density rate, force) and particles
// whose reconstructed position lies outside the mesh [lower, lower + all_cells gs].  The
// counts go to counts[0], counts[1] (one atomic per particle found).
template <int D>
__global__ void k_mp_check(size_t n, MPConst k, MPFluid f, unsigned long long *counts)
{
    for (size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += size_t(gridDim.x) * blockDim.x)
    {
        int c[3];
        unpack_cell<D>(__float_as_uint(f.geo0[i].w), c);
        const float4 di = f.dyn[i];
        bool fin = isfinite(di.x) && isfinite(di.y) && isfinite(di.z) && isfinite(di.w) && isfinite(f.drho[i]) &&
                   isfinite(f.drho_dt[i]);
        bool in = true;
#pragma unroll
        for (int d = 0; d < D; ++d)
        {
            fin = fin && isfinite(f.off[d * n + i]) && isfinite(f.off_lo[d * n + i]) && isfinite(f.force[d * n + i]);
            const double x = position(k, f, n, i, d, c);
            const double hi = k.m.lower[d] + double(k.m.all_cells[d]) * k.m.gs;
            in = in && !(x < k.m.lower[d] || x > hi);
        }
        // a non-finite offset has no position; it counts once, as non-finite
        if (!fin)
            atomicAdd(&counts[0], 1ull);
        else if (!in)
            atomicAdd(&counts[1], 1ull);
    }
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

// Chunks of the position rows sphx_mp_upload_host copies and hashes in a pipeline.
constexpr int kUploadChunks = 4;

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
    // device scalars: 0 acoustic max, 1 advection max, 2 misc, 3 build counts, 4-5 state
    // check, 6-7 tile preparation (window maxima, tile count, build overflow), 8 sweep
    // overflow of the tiled strategy, 10-11 chunk counters of the persistent sweeps
    unsigned long long *slots = nullptr;
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
    // host rows every advection step delivers (sphx_mp_set_host_rows), and the event that
    // releases the velocity rows after the last sub-step's 1st half
    double *host_pos = nullptr, *host_vel = nullptr, *host_rho = nullptr, *host_p = nullptr;
    cudaEvent_t ev_half = nullptr;
    cudaEvent_t ev_chunk[kUploadChunks] = {}; // position chunks of sphx_mp_upload_host
    int block = 128, strategy = 0;
    // tile-grouped traversal (TileShape): tile[0] == 0 keeps the cell order; `order` holds
    // the particles grouped by tile, recomputed at every configuration update
    int tile[3] = {0, 0, 0};
    uint32_t *order = nullptr, *tile_offset = nullptr;
    bool order_active = false;
    // tiled strategy (strategy 2): compacted non-empty tiles, scan scratch, the staged
    // capacities of the current configuration and the strategy the lists were built for
    uint32_t *tiles = nullptr, *tile_flags = nullptr, *tile_pos = nullptr;
    unsigned ntiles_ne = 0, cap_f = 0, cap_w = 0;
    bool lists_tiled = false;
    int lists_strategy = -1;
    size_t smem_set[5] = {0, 0, 0, 0, 0}; // dynamic shared memory granted to the tiled and ring kernels
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
    s.off_lo = mp->alloc<float>(D * n);
    s.force = mp->alloc<float>(D * n);
    s.drho = mp->alloc<float>(n);
    s.drho_dt = mp->alloc<float>(n);
    s.drho_sum = mp->alloc<float>(n);
    s.pres = mp->alloc<float>(n);
    s.id = mp->alloc<uint32_t>(n);
    if (!s.geo0 || !s.dyn || !s.off || !s.off_lo || !s.force || !s.drho || !s.drho_dt || !s.drho_sum || !s.pres ||
        !s.id)
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
    l.limit = uint32_t(&l == &mp->wl ? mp->nw : mp->n); // records the entries index
    l.mask = mp->k.periodic ? kIndexMask : 0xffffffffu;
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

TileShape tile_shape(sphx_mp mp, size_t *ntiles)
{
    TileShape ts{};
    size_t nt = 1;
    for (int d = 0; d < 3; ++d)
    {
        ts.t[d] = d < mp->dim ? std::max(mp->tile[d], 1) : 1;
        ts.nt[d] = d < mp->dim ? (mp->k.m.all_cells[d] + ts.t[d] - 1) / ts.t[d] : 1;
        nt *= size_t(ts.nt[d]);
    }
    *ntiles = nt;
    return ts;
}

// The tile-grouped traversal order of the current cell order (a stable counting sort of the
// particles by tile key), when a tile shape is set; dam-break (non-periodic) solver only.
template <int D>
int tile_order(sphx_mp mp)
{
    mp->order_active = false;
    if (!mp->tile[0] || mp->k.periodic || mp->n == 0)
        return SPHX_OK;
    sphx_ctx ctx = mp->ctx;
    cudaStream_t s = ctx->stream;
    const size_t n = mp->n;
    size_t nt = 0;
    const TileShape ts = tile_shape(mp, &nt);
    SPHX_CUDA(cudaMemsetAsync(mp->count, 0, nt * sizeof(uint32_t), s));
    k_mp_tile_key<D><<<grid_for(n, 256), 256, 0, s>>>(n, mp->a.geo0, ts, mp->key, mp->rank, mp->count);
    SPHX_LAUNCHED(ctx);
    SPHX_TRY(exclusive_scan(ctx, mp->count, mp->tile_offset, nt));
    k_mp_set_total<<<1, 1, 0, s>>>(mp->tile_offset, nt, uint32_t(n));
    SPHX_LAUNCHED(ctx);
    k_mp_scatter<<<grid_for(n, 256), 256, 0, s>>>(n, mp->key, mp->rank, mp->tile_offset, mp->order);
    SPHX_LAUNCHED(ctx);
    k_mp_sort_segments<<<grid_for(nt, 256), 256, 0, s>>>(nt, mp->tile_offset, mp->order);
    SPHX_LAUNCHED(ctx);
    mp->order_active = true;
    return SPHX_OK;
}

constexpr size_t kTiledSmemLimit = 200 * 1024; // dynamic shared memory a tiled block may take

TileGrid tile_grid(sphx_mp mp)
{
    size_t nt = 0;
    TileGrid g{};
    g.ts = tile_shape(mp, &nt);
    g.tiles = mp->tiles;
    g.tile_offset = mp->tile_offset;
    g.order = mp->order;
    return g;
}

// Grants a tiled kernel `bytes` of dynamic shared memory (raised only when needed).
template <class K>
int grant_smem(sphx_mp mp, int which, K kernel, size_t bytes)
{
    if (bytes > mp->smem_set[which])
    {
        SPHX_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(bytes)));
        mp->smem_set[which] = bytes;
    }
    return SPHX_OK;
}

// Non-empty tiles of the tile-grouped order and the largest window populations, read back
// to size the staged windows (synchronises).  Sets mp->lists_tiled when the largest window
// fits the shared-memory limit.
template <int D>
int tile_prepare(sphx_mp mp)
{
    sphx_ctx ctx = mp->ctx;
    cudaStream_t s = ctx->stream;
    size_t nt = 0;
    const TileShape ts = tile_shape(mp, &nt);
    unsigned int *res = reinterpret_cast<unsigned int *>(mp->slots + 6); // maxes, count, overflow
    SPHX_CUDA(cudaMemsetAsync(res, 0, 4 * sizeof(unsigned int), s));
    k_mp_tile_flags<<<grid_for(nt, 256), 256, 0, s>>>(nt, mp->tile_offset, mp->tile_flags);
    SPHX_LAUNCHED(ctx);
    SPHX_TRY(exclusive_scan(ctx, mp->tile_flags, mp->tile_pos, nt));
    k_mp_tile_compact<<<grid_for(nt, 256), 256, 0, s>>>(nt, mp->tile_flags, mp->tile_pos, mp->tiles, res + 2);
    SPHX_LAUNCHED(ctx);
    const size_t warps = std::min(nt, mp->n);
    k_mp_tile_population<D><<<grid_for(warps * 32, 256), 256, 0, s>>>(res + 2, mp->k.m, ts, mp->tiles, mp->f_offset,
                                                                      mp->w_offset, res);
    SPHX_LAUNCHED(ctx);
    SPHX_CUDA(cudaMemcpyAsync(mp->h_slots + 6, res, 4 * sizeof(unsigned int), cudaMemcpyDeviceToHost, s));
    SPHX_CUDA(cudaStreamSynchronize(s));
    const unsigned int *h = reinterpret_cast<const unsigned int *>(mp->h_slots + 6);
    mp->cap_f = std::max(h[0], 1u);
    mp->cap_w = std::max(h[1], 1u);
    mp->ntiles_ne = h[2];
    mp->lists_tiled = 36 * size_t(mp->cap_f + mp->cap_w) + 64 <= kTiledSmemLimit && mp->ntiles_ne > 0;
    return SPHX_OK;
}

template <int D>
int launch_build(sphx_mp mp)
{
    sphx_ctx ctx = mp->ctx;
    cudaStream_t s = ctx->stream;
    unsigned int *mc = reinterpret_cast<unsigned int *>(mp->slots + 3);
    SPHX_TRY(tile_order<D>(mp));
    mp->lists_tiled = false;
    if (mp->strategy == 2 && mp->order_active)
        SPHX_TRY(tile_prepare<D>(mp));
    mp->lists_strategy = mp->strategy;
    const unsigned tblk = unsigned(mp->block);
    if (mp->lists_tiled)
        SPHX_TRY(grant_smem(mp, 0, k_mp_build_tiled<D>, 16 * size_t(mp->cap_f + mp->cap_w)));
    unsigned int *overflow = reinterpret_cast<unsigned int *>(mp->slots + 6) + 3;
    for (int attempt = 0; attempt < 2; ++attempt)
    {
        SPHX_CUDA(cudaMemsetAsync(mc, 0, 2 * sizeof(unsigned int), s));
        if (mp->k.periodic)
            k_mp_build_periodic<D><<<grid_for(mp->n, 256), 256, 0, s>>>(mp->n, mp->k, mp->a, mp->f_offset, mp->in, mc);
        else if (mp->lists_tiled)
            k_mp_build_tiled<D><<<mp->ntiles_ne, tblk, 16 * size_t(mp->cap_f + mp->cap_w), s>>>(
                mp->n, mp->k, mp->a, mp->f_offset, mp->w, mp->w_offset, tile_grid(mp), mp->in, mp->wl, mc,
                mp->cap_f, mp->cap_w, overflow);
        else if (mp->order_active)
            k_mp_build<D, true><<<grid_for(mp->n, 256), 256, 0, s>>>(mp->n, mp->k, mp->a, mp->f_offset, mp->w,
                                                                    mp->w_offset, mp->in, mp->wl, mc, mp->order);
        else
            k_mp_build<D, false><<<grid_for(mp->n, 256), 256, 0, s>>>(mp->n, mp->k, mp->a, mp->f_offset, mp->w,
                                                                     mp->w_offset, mp->in, mp->wl, mc, nullptr);
        SPHX_LAUNCHED(ctx);
        SPHX_CUDA(cudaMemcpyAsync(mp->h_slots + 3, mc, 2 * sizeof(unsigned int), cudaMemcpyDeviceToHost, s));
        SPHX_CUDA(cudaMemcpyAsync(mp->h_slots + 7, mp->slots + 7, sizeof(unsigned long long), cudaMemcpyDeviceToHost,
                                  s));
        SPHX_CUDA(cudaStreamSynchronize(s));
        if (mp->lists_tiled && reinterpret_cast<const unsigned int *>(mp->h_slots + 7)[1] != 0)
            return fail(SPHX_ERR_CAPACITY, "a tile window exceeded its staged capacity");
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
            k_mp_rehash<D><<<grid_for(n, 256), 256, 0, s>>>(n, mp->a, mp->k, mp->ncell, mp->noff,
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
    if (mp->lists_tiled)
        SPHX_CUDA(cudaMemcpyAsync(mp->h_slots + 8, mp->slots + 8, sizeof(unsigned long long), cudaMemcpyDeviceToHost,
                                  mp->ctx->stream));
    SPHX_CUDA(cudaStreamSynchronize(mp->ctx->stream));
    if (mp->lists_tiled && mp->h_slots[8] != 0)
        return fail(SPHX_ERR_CAPACITY, "a tile window exceeded its staged capacity in a sweep");
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

template <int D, bool LISTS, bool ORDER>
void launch_first(sphx_mp mp, unsigned blk, double dt)
{
    const size_t n = mp->n;
    k_mp_first<D, LISTS, ORDER><<<grid_for(n, blk), blk, 0, mp->ctx->stream>>>(
        n, mp->k, mp->a, mp->f_offset, mp->w, mp->w_offset, mp->in, mp->wl, dt, mp->slots, mp->order);
}

template <int D, bool LISTS, bool ORDER>
void launch_second(sphx_mp mp, unsigned blk, double dt)
{
    const size_t n = mp->n;
    k_mp_second<D, LISTS, ORDER><<<grid_for(n, blk), blk, 0, mp->ctx->stream>>>(
        n, mp->k, mp->a, mp->f_offset, mp->w, mp->w_offset, mp->in, mp->wl, dt, mp->slots + 1, mp->order);
}

template <int D>
void launch_first_lanes(sphx_mp mp, unsigned blk, double dt)
{
    const size_t n = mp->n;
    cudaStream_t s = mp->ctx->stream;
    if (strategy_lanes(mp->strategy) == 2)
        k_mp_first_lanes<D, 2><<<grid_for(2 * n, blk), blk, 0, s>>>(n, mp->k, mp->a, mp->w, mp->in, mp->wl, dt,
                                                                    mp->slots);
    else
        k_mp_first_lanes<D, 4><<<grid_for(4 * n, blk), blk, 0, s>>>(n, mp->k, mp->a, mp->w, mp->in, mp->wl, dt,
                                                                    mp->slots);
}

template <int D>
void launch_second_lanes(sphx_mp mp, unsigned blk, double dt)
{
    const size_t n = mp->n;
    cudaStream_t s = mp->ctx->stream;
    if (strategy_lanes(mp->strategy) == 2)
        k_mp_second_lanes<D, 2><<<grid_for(2 * n, blk), blk, 0, s>>>(n, mp->k, mp->a, mp->w, mp->in, mp->wl, dt,
                                                                     mp->slots + 1);
    else
        k_mp_second_lanes<D, 4><<<grid_for(4 * n, blk), blk, 0, s>>>(n, mp->k, mp->a, mp->w, mp->in, mp->wl, dt,
                                                                     mp->slots + 1);
}

// Grid of the resident capacity for a persistent kernel (blocks per SM from the occupancy
// calculator, times the SMs), the chunk counters cleared before each launch.
template <class K>
int persistent_grid(sphx_mp mp, K kernel, unsigned blk, unsigned *grid)
{
    int per_sm = 0;
    SPHX_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, int(blk), 0));
    *grid = unsigned(std::max(1, per_sm) * std::max(1, mp->ctx->num_sms));
    return SPHX_OK;
}

template <int D>
int launch_first_persistent(sphx_mp mp, unsigned blk, double dt)
{
    unsigned grid = 0;
    SPHX_TRY(persistent_grid(mp, k_mp_first_persistent<D>, blk, &grid));
    unsigned int *counter = reinterpret_cast<unsigned int *>(mp->slots + 10);
    SPHX_CUDA(cudaMemsetAsync(counter, 0, sizeof(unsigned int), mp->ctx->stream));
    k_mp_first_persistent<D><<<grid, blk, 0, mp->ctx->stream>>>(mp->n, mp->k, mp->a, mp->w, mp->in, mp->wl, dt,
                                                                 mp->slots, counter);
    return SPHX_OK;
}

template <int D>
int launch_second_persistent(sphx_mp mp, unsigned blk, double dt)
{
    unsigned grid = 0;
    SPHX_TRY(persistent_grid(mp, k_mp_second_persistent<D>, blk, &grid));
    unsigned int *counter = reinterpret_cast<unsigned int *>(mp->slots + 11);
    SPHX_CUDA(cudaMemsetAsync(counter, 0, sizeof(unsigned int), mp->ctx->stream));
    k_mp_second_persistent<D><<<grid, blk, 0, mp->ctx->stream>>>(mp->n, mp->k, mp->a, mp->w, mp->in, mp->wl, dt,
                                                                  mp->slots + 1, counter);
    return SPHX_OK;
}

template <int D>
int launch_first_async(sphx_mp mp, unsigned blk, double dt)
{
    const size_t bytes = async_ring_bytes(false, blk);
    SPHX_TRY(grant_smem(mp, 3, k_mp_first_async<D, kAsyncDepthFirst>, bytes));
    k_mp_first_async<D, kAsyncDepthFirst><<<grid_for(mp->n, blk), blk, bytes, mp->ctx->stream>>>(
        mp->n, mp->k, mp->a, mp->w, mp->in, mp->wl, dt, mp->slots);
    return SPHX_OK;
}

template <int D>
int launch_second_async(sphx_mp mp, unsigned blk, double dt)
{
    const size_t bytes = async_ring_bytes(true, blk);
    SPHX_TRY(grant_smem(mp, 4, k_mp_second_async<D, kAsyncDepthSecond>, bytes));
    k_mp_second_async<D, kAsyncDepthSecond><<<grid_for(mp->n, blk), blk, bytes, mp->ctx->stream>>>(
        mp->n, mp->k, mp->a, mp->w, mp->in, mp->wl, dt, mp->slots + 1);
    return SPHX_OK;
}

template <int D>
int launch_first_tiled(sphx_mp mp, unsigned blk, double dt)
{
    const size_t bytes = 32 * size_t(mp->cap_f + mp->cap_w);
    SPHX_TRY(grant_smem(mp, 1, k_mp_first_tiled<D>, bytes));
    k_mp_first_tiled<D><<<mp->ntiles_ne, blk, bytes, mp->ctx->stream>>>(
        mp->n, mp->k, mp->a, mp->f_offset, mp->w, mp->w_offset, tile_grid(mp), mp->in, mp->wl, dt, mp->slots,
        mp->cap_f, mp->cap_w, reinterpret_cast<unsigned int *>(mp->slots + 8));
    return SPHX_OK;
}

template <int D>
int launch_second_tiled(sphx_mp mp, unsigned blk, double dt)
{
    const size_t bytes = 36 * size_t(mp->cap_f + mp->cap_w);
    SPHX_TRY(grant_smem(mp, 2, k_mp_second_tiled<D>, bytes));
    k_mp_second_tiled<D><<<mp->ntiles_ne, blk, bytes, mp->ctx->stream>>>(
        mp->n, mp->k, mp->a, mp->f_offset, mp->w, mp->w_offset, tile_grid(mp), mp->in, mp->wl, dt, mp->slots + 1,
        mp->cap_f, mp->cap_w, reinterpret_cast<unsigned int *>(mp->slots + 8));
    return SPHX_OK;
}

// Export of registered host rows from the last sub-step: velocity and pressure (final
// after its 1st half) on the side stream, concurrent with the 2nd half; position and
// density on the context's stream after the 2nd half.
template <int D>
int deliver_rows(sphx_mp mp, int rows)
{
    const size_t n = mp->n;
    cudaStream_t s = mp->ctx->stream;
    double *spos = mp->stage, *svel = spos + n * D, *srho = svel + n * D, *sp = srho + n;
    const size_t vec = n * D * sizeof(double), sca = n * sizeof(double);
    if (rows == kRowsVelocity)
    {
        SPHX_CUDA(cudaEventRecord(mp->ev_half, s));
        SPHX_CUDA(cudaStreamWaitEvent(mp->side, mp->ev_half, 0));
        k_mp_export_rows<D, kRowsVelocity><<<grid_for(n, 256), 256, 0, mp->side>>>(n, mp->k, mp->a, spos, svel,
                                                                                    srho, sp);
        SPHX_LAUNCHED(mp->ctx);
        SPHX_CUDA(cudaMemcpyAsync(mp->host_vel, svel, vec, cudaMemcpyDeviceToHost, mp->side));
        SPHX_CUDA(cudaMemcpyAsync(mp->host_p, sp, sca, cudaMemcpyDeviceToHost, mp->side));
    }
    else
    {
        k_mp_export_rows<D, kRowsPosition><<<grid_for(n, 256), 256, 0, s>>>(n, mp->k, mp->a, spos, svel, srho, sp);
        SPHX_LAUNCHED(mp->ctx);
        SPHX_CUDA(cudaMemcpyAsync(mp->host_pos, spos, vec, cudaMemcpyDeviceToHost, s));
        SPHX_CUDA(cudaMemcpyAsync(mp->host_rho, srho, sca, cudaMemcpyDeviceToHost, s));
    }
    return SPHX_OK;
}

// One acoustic sub-step; deliver: the last of an advection step with host rows registered.
template <int D>
int substep(sphx_mp mp, double dt, bool deliver = false)
{
    sphx_ctx ctx = mp->ctx;
    cudaStream_t s = ctx->stream;
    size_t n = mp->n;
    if (n == 0)
        return SPHX_OK;
    // the lists follow the strategy they were built for; the build reads the geometry of
    // the last configuration update only, so a rebuild here gives the same lists and sums
    if (!mp->k.periodic && (mp->strategy == 2) != (mp->lists_strategy == 2))
        SPHX_TRY(launch_build<D>(mp));
    unsigned blk = unsigned(mp->block);
    k_mp_init1<<<grid_for(n, 256), 256, 0, s>>>(n, mp->a.drho, mp->a.drho_dt, mp->a.dyn, mp->a.pres,
                                                mp->k.p.p0_over_rho0, float(0.5 * dt));
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
    else if (mp->lists_tiled)
        SPHX_TRY(launch_first_tiled<D>(mp, blk, dt));
    else if (mp->strategy == 3)
        SPHX_TRY(launch_first_async<D>(mp, blk, dt));
    else if (mp->strategy == 4)
        SPHX_TRY(launch_first_persistent<D>(mp, blk, dt));
    else if (strategy_lanes(mp->strategy))
        launch_first_lanes<D>(mp, blk, dt);
    else if (mp->strategy != 1)
        mp->order_active ? launch_first<D, true, true>(mp, blk, dt) : launch_first<D, true, false>(mp, blk, dt);
    else
        mp->order_active ? launch_first<D, false, true>(mp, blk, dt) : launch_first<D, false, false>(mp, blk, dt);
    SPHX_LAUNCHED(ctx);
    if (deliver)
        SPHX_TRY(deliver_rows<D>(mp, kRowsVelocity));
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
    else if (mp->lists_tiled)
        SPHX_TRY(launch_second_tiled<D>(mp, blk, dt));
    else if (mp->strategy == 3)
        SPHX_TRY(launch_second_async<D>(mp, blk, dt));
    else if (mp->strategy == 4)
        SPHX_TRY(launch_second_persistent<D>(mp, blk, dt));
    else if (strategy_lanes(mp->strategy))
        launch_second_lanes<D>(mp, blk, dt);
    else if (mp->strategy != 1)
        mp->order_active ? launch_second<D, true, true>(mp, blk, dt) : launch_second<D, true, false>(mp, blk, dt);
    else
        mp->order_active ? launch_second<D, false, true>(mp, blk, dt) : launch_second<D, false, false>(mp, blk, dt);
    SPHX_LAUNCHED(ctx);
    if (deliver)
        SPHX_TRY(deliver_rows<D>(mp, kRowsPosition));
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
    bool delivered = false;
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
        // the last sub-step (relaxation reaches Dt) delivers the registered host rows
        const bool deliver = mp->host_pos && relaxation + dt >= Dt;
        SPHX_TRY(substep<D>(mp, dt, deliver));
        delivered = delivered || deliver;
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
    if (delivered) // the rows are in host memory when the step returns
    {
        SPHX_CUDA(cudaStreamSynchronize(mp->side));
        SPHX_CUDA(cudaStreamSynchronize(mp->ctx->stream));
    }
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
            k_mp_from_fp64<2><<<grid_for(n, 256), 256, 0, s>>>(n, 0, n, (const double *)pos->dev, n, 1, mp->k, mp->ncell,
                                                               mp->noff, mp->key, mp->rank, mp->count);
        else
            k_mp_from_fp64<3><<<grid_for(n, 256), 256, 0, s>>>(n, 0, n, (const double *)pos->dev, n, 1, mp->k, mp->ncell,
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
    mp->noff = mp->alloc<float>(6 * n);
    mp->w.geo = mp->alloc<float4>(nw);
    mp->w.n = mp->alloc<float4>(nw);
    mp->w.nw = nw;
    mp->in.count = mp->alloc<uint32_t>(n);
    mp->wl.count = mp->alloc<uint32_t>(n);
    mp->slots = mp->alloc<unsigned long long>(12);
    mp->order = mp->alloc<uint32_t>(n);
    mp->tile_offset = mp->alloc<uint32_t>(nc + 1);
    mp->tiles = mp->alloc<uint32_t>(nc);
    mp->tile_flags = mp->alloc<uint32_t>(nc);
    mp->tile_pos = mp->alloc<uint32_t>(nc);
    if (!mp->f_offset || !mp->w_offset || !mp->count || !mp->key || !mp->rank || !mp->perm || !mp->ncell ||
        !mp->noff || !mp->w.geo || !mp->w.n || !mp->in.count || !mp->wl.count || !mp->slots || !mp->order ||
        !mp->tile_offset || !mp->tiles || !mp->tile_flags || !mp->tile_pos)
        return bail(fail(SPHX_ERR_OUT_OF_MEMORY, "mixed-precision allocation failed"));
    if (cudaMemsetAsync(mp->slots, 0, 12 * sizeof(unsigned long long), ctx->stream) != cudaSuccess)
        return bail(fail(SPHX_ERR_CUDA, "slot initialisation failed"));
    if (cudaMallocHost(&mp->h_slots, 12 * sizeof(unsigned long long)) != cudaSuccess)
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
    mp->noff = mp->alloc<float>(6 * n);
    mp->in.count = mp->alloc<uint32_t>(n);
    mp->wl.count = mp->alloc<uint32_t>(n);
    mp->slots = mp->alloc<unsigned long long>(12);
    if (!mp->f_offset || !mp->w_offset || !mp->count || !mp->key || !mp->rank || !mp->perm || !mp->ncell ||
        !mp->noff || !mp->in.count || !mp->wl.count || !mp->slots)
        return bail(fail(SPHX_ERR_OUT_OF_MEMORY, "mixed-precision allocation failed"));
    if (cudaMemsetAsync(mp->slots, 0, 12 * sizeof(unsigned long long), ctx->stream) != cudaSuccess)
        return bail(fail(SPHX_ERR_CUDA, "slot initialisation failed"));
    if (cudaMallocHost(&mp->h_slots, 12 * sizeof(unsigned long long)) != cudaSuccess)
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
    if (!mp->ev_half)
        SPHX_CUDA(cudaEventCreateWithFlags(&mp->ev_half, cudaEventDisableTiming));
    for (cudaEvent_t &e : mp->ev_chunk)
        if (!e)
            SPHX_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
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
    SPHX_CUDA(cudaMemsetAsync(mp->count, 0, mp->ncells * sizeof(uint32_t), s));
    SPHX_CUDA(cudaEventRecord(mp->ev_pos, s));
    if (n > 0)
    {
        // the position rows in chunks on the side stream, each hashed on the context's
        // stream as soon as it has arrived (the hash of one chunk overlaps the copy of the
        // next); then the other rows
        SPHX_CUDA(cudaStreamWaitEvent(mp->side, mp->ev_pos, 0));
        for (int c = 0; c < kUploadChunks; ++c)
        {
            const size_t b0 = n * size_t(c) / kUploadChunks, b1 = n * size_t(c + 1) / kUploadChunks;
            if (b1 == b0)
                continue;
            SPHX_CUDA(cudaMemcpyAsync(spos + b0 * D, pos + b0 * D, (b1 - b0) * D * sizeof(double),
                                      cudaMemcpyHostToDevice, mp->side));
            SPHX_CUDA(cudaEventRecord(mp->ev_chunk[c], mp->side));
            SPHX_CUDA(cudaStreamWaitEvent(s, mp->ev_chunk[c], 0));
            k_mp_from_fp64<D><<<grid_for(b1 - b0, 256), 256, 0, s>>>(n, b0, b1, spos, 1, D, mp->k, mp->ncell,
                                                                     mp->noff, mp->key, mp->rank, mp->count);
            SPHX_LAUNCHED(ctx);
        }
        SPHX_CUDA(cudaMemcpyAsync(svel, vel, vec, cudaMemcpyHostToDevice, mp->side));
        SPHX_CUDA(cudaMemcpyAsync(sforce, force, vec, cudaMemcpyHostToDevice, mp->side));
        SPHX_CUDA(cudaMemcpyAsync(srho, rho, sca, cudaMemcpyHostToDevice, mp->side));
        SPHX_CUDA(cudaMemcpyAsync(sdrho, drho_dt, sca, cudaMemcpyHostToDevice, mp->side));
        SPHX_CUDA(cudaEventRecord(mp->ev_rest, mp->side));
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
        k_mp_export_rows<D, kRowsAll><<<grid_for(n, 256), 256, 0, s>>>(n, mp->k, mp->a, spos, svel, srho, sp);
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

extern "C" int sphx_mp_set_host_rows(sphx_mp mp, double *position, double *velocity, double *density,
                                     double *pressure)
{
    if (!mp)
        return fail(SPHX_ERR_INVALID_ARG, "null solver");
    const bool none = !position && !velocity && !density && !pressure;
    if (!none && mp->n > 0 && (!position || !velocity || !density || !pressure))
        return fail(SPHX_ERR_INVALID_ARG, "sphx_mp_set_host_rows takes the four host rows, or none");
    if (!none)
        SPHX_TRY(ensure_host_io(mp));
    SPHX_CUDA(cudaStreamSynchronize(mp->ctx->stream));
    mp->host_pos = none ? nullptr : position;
    mp->host_vel = none ? nullptr : velocity;
    mp->host_rho = none ? nullptr : density;
    mp->host_p = none ? nullptr : pressure;
    return SPHX_OK;
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
    if (mp->ev_half)
        cudaEventDestroy(mp->ev_half);
    for (cudaEvent_t e : mp->ev_chunk)
        if (e)
            cudaEventDestroy(e);
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
        void *src[7] = {mp->a.dyn, mp->a.off, mp->a.off_lo, mp->a.force, mp->a.drho, mp->a.drho_dt, mp->slots};
        size_t bytes[7] = {n * sizeof(float4), D * n * 4, D * n * 4, D * n * 4, n * 4, n * 4,
                           2 * sizeof(unsigned long long)};
        if (!restore)
        {
            bufs.assign(7, nullptr);
            for (int q = 0; q < 7; ++q)
                SPHX_CUDA(cudaMallocAsync(&bufs[q], std::max<size_t>(bytes[q], 1), mp->ctx->stream));
        }
        for (int q = 0; q < 7; ++q)
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
    // candidate settings: strategies 0 and 1 in cell order, the tiled strategy 2 with
    // several tile shapes (sub-cells per axis), each with every block size
    struct Setting
    {
        int strategy, tile[3];
    };
    std::vector<Setting> settings = {{0, {0, 0, 0}}, {1, {0, 0, 0}}};
    if (!mp->k.periodic)
    {
        for (int st : {3, 4, 5, 6})
            settings.push_back(Setting{st, {0, 0, 0}});
        if (mp->dim == 3)
            for (const Setting &t : {Setting{2, {4, 4, 4}}, Setting{2, {4, 4, 8}}})
                settings.push_back(t);
        else
            for (const Setting &t : {Setting{2, {8, 8, 0}}, Setting{2, {4, 8, 0}}})
                settings.push_back(t);
    }
    int keep_block = mp->block, keep_strategy = mp->strategy;
    int keep_tile[3] = {mp->tile[0], mp->tile[1], mp->tile[2]};
    bool keep_prof = mp->profiling;
    double best = 1e300;
    int bb = keep_block, bs = keep_strategy;
    int bt[3] = {keep_tile[0], keep_tile[1], keep_tile[2]};
    cudaEvent_t e0, e1;
    SPHX_CUDA(cudaEventCreate(&e0));
    SPHX_CUDA(cudaEventCreate(&e1));
    int st = SPHX_OK;
    mp->profiling = false;
    for (size_t si = 0; si < settings.size() && st == SPHX_OK; ++si)
        for (int bi = 0; bi < 3 && st == SPHX_OK; ++bi)
        {
            const Setting &set = settings[si];
            const bool retile = set.tile[0] != mp->tile[0] || set.tile[1] != mp->tile[1] || set.tile[2] != mp->tile[2];
            mp->block = blocks[bi];
            mp->strategy = set.strategy;
            for (int d = 0; d < 3; ++d)
                mp->tile[d] = set.tile[d];
            if (retile) // the order, and for strategy 2 the lists, of the new shape
                st = mp->dim == 2 ? launch_build<2>(mp) : launch_build<3>(mp);
            if (st != SPHX_OK || (st = snap.take(mp, true)) != SPHX_OK)
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
                bs = set.strategy;
                for (int d = 0; d < 3; ++d)
                    bt[d] = set.tile[d];
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
        for (int d = 0; d < 3; ++d)
            mp->tile[d] = keep_tile[d];
        int st3 = mp->dim == 2 ? launch_build<2>(mp) : launch_build<3>(mp);
        return st != SPHX_OK ? st : (st2 != SPHX_OK ? st2 : st3);
    }
    mp->block = bb;
    mp->strategy = bs;
    for (int d = 0; d < 3; ++d)
        mp->tile[d] = bt[d];
    // lists and order of the chosen setting (the build reads the configuration geometry only)
    SPHX_TRY(mp->dim == 2 ? launch_build<2>(mp) : launch_build<3>(mp));
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
    if (!mp || block < 64 || block > 256 || block % 32 != 0 || strategy < 0 || strategy > 6)
        return fail(SPHX_ERR_INVALID_ARG, "block must be 64..256 in steps of 32, strategy 0 to 6");
    if (strategy >= 3 && mp->k.periodic)
        return fail(SPHX_ERR_INVALID_ARG, "strategies 3 and 4 serve the dam-break solver only");
    if (strategy == 2 && mp->k.periodic)
        return fail(SPHX_ERR_INVALID_ARG, "the tiled strategy serves the dam-break solver only");
    if (strategy == 2 && (mp->tile[0] > kTileMaxExtent || mp->tile[1] > kTileMaxExtent || mp->tile[2] > kTileMaxExtent))
        return fail(SPHX_ERR_INVALID_ARG, "the tiled strategy takes tiles of at most %d sub-cells per axis",
                    kTileMaxExtent);
    mp->block = block;
    mp->strategy = strategy;
    if (strategy == 2 && !mp->tile[0])
    {
        mp->tile[0] = mp->tile[1] = 4;
        mp->tile[2] = mp->dim == 3 ? 4 : 0;
    }
    return SPHX_OK; // the lists follow at the next sub-step (substep rebuilds them)
}

extern "C" int sphx_mp_get_tuning(sphx_mp mp, int *block, int *strategy, int *tile)
{
    if (!mp)
        return fail(SPHX_ERR_INVALID_ARG, "null solver");
    if (block)
        *block = mp->block;
    if (strategy)
        *strategy = mp->strategy;
    if (tile)
        for (int d = 0; d < 3; ++d)
            tile[d] = mp->tile[d];
    return SPHX_OK;
}

extern "C" int sphx_mp_set_tile(sphx_mp mp, int tx, int ty, int tz)
{
    if (!mp || tx < 0 || ty < 0 || tz < 0 || tx > 64 || ty > 64 || tz > 64 || (tx == 0) != (ty == 0) ||
        (mp->dim == 3 && (tx == 0) != (tz == 0)))
        return fail(SPHX_ERR_INVALID_ARG, "tile extents must be 1..64 sub-cells per axis, or all 0 (off)");
    if (tx && mp->k.periodic)
        return fail(SPHX_ERR_INVALID_ARG, "the tile-grouped traversal serves the dam-break solver only");
    if (mp->strategy == 2 && (!tx || tx > kTileMaxExtent || ty > kTileMaxExtent || tz > kTileMaxExtent))
        return fail(SPHX_ERR_INVALID_ARG, "the tiled strategy takes tiles of 1..%d sub-cells per axis",
                    kTileMaxExtent);
    SPHX_TRY(settle_configuration(mp));
    mp->tile[0] = tx;
    mp->tile[1] = ty;
    mp->tile[2] = mp->dim == 3 ? tz : 0;
    if (mp->n == 0)
        return SPHX_OK;
    // the order (and, for the tiled strategy, the staged-index lists) of the new shape
    return mp->dim == 2 ? launch_build<2>(mp) : launch_build<3>(mp);
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

extern "C" int sphx_mp_check_state(sphx_mp mp, uint64_t *non_finite, uint64_t *out_of_mesh)
{
    if (!mp)
        return fail(SPHX_ERR_INVALID_ARG, "null solver");
    sphx_ctx ctx = mp->ctx;
    SPHX_CUDA(cudaMemsetAsync(mp->slots + 4, 0, 2 * sizeof(unsigned long long), ctx->stream));
    if (mp->n > 0)
    {
        unsigned g = unsigned(std::max(1, std::min(ctx->num_sms * 4, int(grid_for(mp->n, 256)))));
        if (mp->dim == 2)
            k_mp_check<2><<<g, 256, 0, ctx->stream>>>(mp->n, mp->k, mp->a, mp->slots + 4);
        else
            k_mp_check<3><<<g, 256, 0, ctx->stream>>>(mp->n, mp->k, mp->a, mp->slots + 4);
        SPHX_LAUNCHED(ctx);
    }
    SPHX_CUDA(cudaMemcpyAsync(mp->h_slots + 4, mp->slots + 4, 2 * sizeof(unsigned long long), cudaMemcpyDeviceToHost,
                              ctx->stream));
    SPHX_CUDA(cudaStreamSynchronize(ctx->stream));
    const uint64_t nf = mp->h_slots[4], om = mp->h_slots[5];
    if (non_finite)
        *non_finite = nf;
    if (out_of_mesh)
        *out_of_mesh = om;
    if (nf || om)
        return fail(SPHX_ERR_NUMERIC, "mixed-precision state: %llu particles with non-finite values, %llu outside the mesh",
                    (unsigned long long)nf, (unsigned long long)om);
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
