// Tiled neighbour strategy of the mixed-precision dam-break solver (strategy 2): one thread
// block per box of sub-cells (a tile), the tile's neighbour window (the box grown by the
// search reach, clamped to the mesh) staged in shared memory, and per-particle neighbour
// lists that hold indices into that staged window instead of particle indices.
//
// It replaces the reference's device traversal: particle_for over an index range
// (particle_iterators_sycl.h:229-241) with each work item walking its cells
// (forInnerSearch / searchInRange, cell_linked_list.hpp:120-160).  The neighbours found,
// their order and the arithmetic on them are those of build_particle / first_particle /
// second_particle (mp_common.cuh), so the three strategies give the same results bit for
// bit; what changes is where the neighbour records come from (shared memory, staged once
// per block, instead of one L1/L2 gather per stored pair) and how a neighbour's cell offset
// is formed (exact small-integer floats relative to the window instead of the packed-lane
// decode).
//
// Window layout: the window is a set of columns along the last axis (x, y in 3D; x in 2D),
// each column one contiguous run of particles in the cell order.  Column c of the window
// starts at particle beg[c] and at staged index base[c]; a particle j of column c sits at
// staged index base[c] + (j - beg[c]).  Tiles hold at most kTileMaxExtent sub-cells per
// axis, so a window has at most kTileMaxCols columns.
#pragma once

#include "mp_common.cuh"

namespace sphx
{
namespace mpc
{
constexpr int kTileMaxExtent = 8;
constexpr int kTileMaxCols = (kTileMaxExtent + 2 * kReach) * (kTileMaxExtent + 2 * kReach);

// Non-empty tiles and the tile-grouped particle order: the particles of tile tiles[b] are
// order[tile_offset[tiles[b]] .. tile_offset[tiles[b] + 1]); lists are slot-major by order
// position (slot s of position t at J[s * n + t]).
struct TileGrid
{
    TileShape ts;
    const uint32_t *tiles, *tile_offset, *order;
};

template <int D>
struct Window
{
    int lo[3], hi[3];
    int ncol, ny; // columns over the leading axes; ny = window extent along axis 1 (3D)
};

template <int D>
__device__ __forceinline__ void tile_window(const MeshDev &m, const TileShape &ts, uint32_t tile, Window<D> &w)
{
    int tc[3] = {0, 0, 0};
    uint32_t r = tile;
#pragma unroll
    for (int d = D - 1; d >= 0; --d)
    {
        tc[d] = int(r % uint32_t(ts.nt[d]));
        r /= uint32_t(ts.nt[d]);
    }
    w.lo[2] = w.hi[2] = 0;
#pragma unroll
    for (int d = 0; d < D; ++d)
    {
        w.lo[d] = max(tc[d] * ts.t[d] - kReach, 0);
        w.hi[d] = min((tc[d] + 1) * ts.t[d] - 1 + kReach, m.all_cells[d] - 1);
    }
    if (D == 3)
    {
        w.ny = w.hi[1] - w.lo[1] + 1;
        w.ncol = (w.hi[0] - w.lo[0] + 1) * w.ny;
    }
    else
    {
        w.ny = 1;
        w.ncol = w.hi[0] - w.lo[0] + 1;
    }
}

// Linear cells of the first and last window cell of column col.
template <int D>
__device__ __forceinline__ void column_cells(const MeshDev &m, const Window<D> &w, int col, uint32_t &first,
                                             uint32_t &last)
{
    int c[3] = {0, 0, 0};
    if (D == 3)
    {
        c[0] = w.lo[0] + col / w.ny;
        c[1] = w.lo[1] + col % w.ny;
    }
    else
        c[0] = w.lo[0] + col;
    c[D - 1] = w.lo[D - 1];
    first = linear_cell<D>(m, c);
    c[D - 1] = w.hi[D - 1];
    last = linear_cell<D>(m, c);
}

// Column index of the window for leading cell coordinates (x) or (x, y).
template <int D>
__device__ __forceinline__ int column_of(const Window<D> &w, int x, int y)
{
    return D == 3 ? (x - w.lo[0]) * w.ny + (y - w.lo[1]) : x - w.lo[0];
}

// Run table of a window in shared memory: beg[c] (first particle of column c) and base[c]
// (its staged index), base[ncol] = the staged total, which it returns.  All threads of the
// block call it.
template <int D>
__device__ __forceinline__ uint32_t window_table(const MeshDev &m, const Window<D> &w, const uint32_t *offset,
                                                 uint32_t *beg, uint32_t *base, uint32_t *total)
{
    for (int col = threadIdx.x; col < w.ncol; col += blockDim.x)
    {
        uint32_t a, b;
        column_cells<D>(m, w, col, a, b);
        const uint32_t s = offset[a];
        beg[col] = s;
        base[col] = offset[b + 1] - s; // length, turned into the staged base below
    }
    __syncthreads();
    if (threadIdx.x < 32)
    {
        const int lane = threadIdx.x;
        const int per = (w.ncol + 31) / 32;
        uint32_t s = 0;
        for (int q = 0; q < per; ++q)
        {
            const int c = lane * per + q;
            if (c < w.ncol)
                s += base[c];
        }
        uint32_t incl = s;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1)
        {
            const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o)
                incl += y;
        }
        uint32_t run = incl - s;
        for (int q = 0; q < per; ++q)
        {
            const int c = lane * per + q;
            if (c < w.ncol)
            {
                const uint32_t l = base[c];
                base[c] = run;
                run += l;
            }
        }
        if (lane == 31)
        {
            *total = incl;
            base[w.ncol] = incl;
        }
    }
    __syncthreads();
    return *total;
}

// Calls f(j, s) for every particle j of the window with its staged index s, a warp per
// column.
template <int D, class F>
__device__ __forceinline__ void for_each_staged(const Window<D> &w, const uint32_t *beg, const uint32_t *base,
                                                F &&f)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    for (int col = warp; col < w.ncol; col += nwarps)
    {
        const uint32_t b0 = beg[col], s0 = base[col], len = base[col + 1] - s0;
        for (uint32_t k = lane; k < len; k += 32)
            f(b0 + k, s0 + k);
    }
}

// Cell coordinates relative to the window's lower corner as exact floats: the difference
// of two of them is the exact integer cell difference geo_dx forms from packed lanes.
template <int D>
__device__ __forceinline__ float4 window_cell(const Window<D> &w, uint32_t packed)
{
    int c[3];
    unpack_cell<D>(packed, c);
    return make_float4(float(c[0] - w.lo[0]), float(c[1] - w.lo[1]), D == 3 ? float(c[2] - w.lo[2]) : 0.0f, 0.0f);
}

// x_i - x_j from window-relative cells and cell offsets: fmaf(c_i - c_j, gs, o_i - o_j),
// the value geo_dx gives for the same pair.
template <int D>
__device__ __forceinline__ void tile_dx(float gs, const float *ci, const float *oi, float4 cj, float4 oj, float *dx)
{
    const float c[3] = {cj.x, cj.y, cj.z};
    const float o[3] = {oj.x, oj.y, oj.z};
#pragma unroll
    for (int d = 0; d < D; ++d)
        dx[d] = fmaf(ci[d] - c[d], gs, oi[d] - o[d]);
}
// Staged window of one block: fluid and wall run tables and record arrays in shared memory.
template <int D>
struct Staged
{
    Window<D> w;
    const uint32_t *fbeg, *fbase, *wbeg, *wbase;
    const float4 *fa, *fb, *wa, *wb; // record halves (see the sweeps)
    const float *fc, *wc;            // third part of the 2nd-half records
};

// Configuration of particle i at order position t (build_particle with the candidates read
// from the staged window): the same candidates in the same order, the same membership test
// and density sums; list entries are staged indices, slot-major by order position.
template <int D>
__device__ __forceinline__ void build_particle_tiled(size_t t, size_t i, size_t n, const MPParams &k, const MeshDev &m,
                                                     const Staged<D> &sw, const uint32_t *f_offset,
                                                     const uint32_t *w_offset, const MPState &f,
                                                     const MPNeighbors &in, const MPNeighbors &wl,
                                                     unsigned int *max_counts)
{
    const float4 gi = f.geo0[i];
    const uint32_t pib = __float_as_uint(gi.w) + CellLanes<D>::bias;
    int ci[3] = {0, 0, 0};
    unpack_cell<D>(__float_as_uint(gi.w), ci);
    const float oi[3] = {gi.x, gi.y, gi.z};
    Kahan sigma;
    unsigned cnt = 0;
    for_each_candidate_run<D, true>(m, 0u, f_offset, ci, Reach(oi, k.gs_f, k.rc_reach),
                                    [&](int x, int y, uint32_t b, uint32_t e) {
                                        const int col = column_of<D>(sw.w, x, y);
                                        const uint32_t s0 = sw.fbase[col] - sw.fbeg[col];
                                        for (uint32_t j = b; j < e; ++j)
                                        {
                                            if (j == uint32_t(i))
                                                continue;
                                            float dx[3];
                                            geo_dx<D>(k.gs_f, pib, oi, sw.fa[s0 + j], dx);
                                            float r2 = sq<D>(dx);
                                            if (!(r2 < k.rc_sqr))
                                                continue;
                                            if (cnt < in.cap)
                                                in.J[size_t(cnt) * n + t] = s0 + j;
                                            ++cnt;
                                            sigma.add(wc2_W(k.fW, k.inv_h, sqrtf(r2)));
                                        }
                                    });
    Kahan wsig;
    unsigned wcnt = 0;
    for_each_candidate_run<D, false>(m, 0u, w_offset, ci, Reach(oi, k.gs_f, k.rc_reach),
                                     [&](int x, int y, uint32_t b, uint32_t e) {
                                         const int col = column_of<D>(sw.w, x, y);
                                         const uint32_t s0 = sw.wbase[col] - sw.wbeg[col];
                                         for (uint32_t j = b; j < e; ++j)
                                         {
                                             float dx[3];
                                             geo_dx<D>(k.gs_f, pib, oi, sw.wa[s0 + j], dx);
                                             float r2 = sq<D>(dx);
                                             if (!(r2 < k.rc_sqr))
                                                 continue;
                                             if (wcnt < wl.cap)
                                                 wl.J[size_t(wcnt) * n + t] = s0 + j;
                                             ++wcnt;
                                             wsig.add(wc2_W(k.fW, k.inv_h, sqrtf(r2)));
                                         }
                                     });
    in.count[t] = cnt;
    wl.count[t] = wcnt;
    warp_atomic_max(&max_counts[0], cnt);
    warp_atomic_max(&max_counts[1], wcnt);
    double dsig = (double(sigma.s) - k.sigma0) - double(sigma.c) + double(k.fW);
    f.drho_sum[i] = float(dsig) * k.rho0_over_sigma0 + wsig.value() * k.wall_factor;
}

struct TiledRec1
{
    float4 o, c; // {offset, pressure}, {window cell}
};

// first_particle for particle i at order position t with staged records: fluid
// fa = {offset, p}, fb = {window cell}; wall wa = {offset}, wb = {window cell}.
template <int D>
__device__ __forceinline__ double first_particle_tiled(size_t t, size_t i, size_t n, const MPParams &k,
                                                       const Staged<D> &sw, double dt, const MPState &f,
                                                       const MPNeighbors &in, const MPNeighbors &wl)
{
    const float4 gi = f.geo0[i];
    const float4 cw = window_cell<D>(sw.w, __float_as_uint(gi.w));
    const float cif[3] = {cw.x, cw.y, cw.z};
    const float oi[3] = {gi.x, gi.y, gi.z};
    const float4 di = f.dyn[i];
    const float p_i = di.w;
    const float rho_i = k.rho0 + f.drho[i];
    Acc force[3], rdis;
    auto pair = [&](const TiledRec1 &r) {
        float dx[3];
        tile_dx<D>(k.gs_f, cif, oi, r.c, r.o, dx);
        float r2 = sq<D>(dx);
        float inv = inv_dist(r2);
        float dWV = wc2_dWV(k.cW, k.inv_h, r2 * inv);
        float sc = (p_i + r.o.w) * (dWV * inv);
#pragma unroll
        for (int d = 0; d < D; ++d)
            force[d].add(-sc * dx[d]);
        rdis.add((p_i - r.o.w) * dWV);
    };
    auto flush = [&]() {
#pragma unroll
        for (int d = 0; d < D; ++d)
            force[d].flush();
        rdis.flush();
    };
    auto load = [&](uint32_t s) { return TiledRec1{sw.fa[s], sw.fb[s]}; };
    list_sweep<false, kUnrollFirst>(t, n, in, load, pair, flush);

    Acc wforce[3], wrdis;
    auto wpair = [&](const TiledRec1 &r) {
        float dx[3];
        tile_dx<D>(k.gs_f, cif, oi, r.c, r.o, dx);
        float r2 = sq<D>(dx);
        float inv = inv_dist(r2);
        float dWV = wc2_dWV(k.cWw, k.inv_h, r2 * inv);
        float p_w = p_i + rho_i * fmaxf(0.0f, -dot<D>(k.g, dx));
        float sc = (p_i + p_w) * (dWV * inv);
#pragma unroll
        for (int d = 0; d < D; ++d)
            wforce[d].add(-sc * dx[d]);
        wrdis.add((p_i - p_w) * dWV);
    };
    auto wflush = [&]() {
#pragma unroll
        for (int d = 0; d < D; ++d)
            wforce[d].flush();
        wrdis.flush();
    };
    auto wload = [&](uint32_t s) { return TiledRec1{sw.wa[s], sw.wb[s]}; };
    list_sweep<false, kUnrollFirst>(t, n, wl, wload, wpair, wflush);

    f.drho_dt[i] = (rdis.value() * k.inv_z) * rho_i + (wrdis.value() * k.inv_z) * rho_i;
    float v2 = 0.f;
    float vn[3] = {di.x, di.y, di.z};
    const float dt_f = float(dt);
#pragma unroll
    for (int d = 0; d < D; ++d)
    {
        float F = f.force[d * n + i] + force[d].value() * k.Vol + wforce[d].value() * k.Vol;
        f.force[d * n + i] = F;
        float vo = vn[d];
        half_step(f, n, i, d, dt, vo);
        vn[d] = vo + (k.g[d] + F * k.inv_mass) * dt_f;
        v2 += vn[d] * vn[d];
    }
    f.dyn[i] = make_float4(vn[0], vn[1], D == 3 ? vn[2] : 0.f, p_i);
    return k.c0 + double(sqrtf(v2));
}

struct TiledRec2
{
    float4 o, c; // {offset, v_x | n_x}, {window cell, v_y | n_y}
    float z;     // v_z | n_z
};

// second_particle for particle i at order position t with staged records: fluid
// fa = {offset, v.x}, fb = {window cell, v.y}, fc = v.z; wall the same with the normal.
template <int D>
__device__ __forceinline__ double second_particle_tiled(size_t t, size_t i, size_t n, const MPParams &k,
                                                        const Staged<D> &sw, double dt, const MPState &f,
                                                        const MPNeighbors &in, const MPNeighbors &wl)
{
    const float4 gi = f.geo0[i];
    const float4 cw = window_cell<D>(sw.w, __float_as_uint(gi.w));
    const float cif[3] = {cw.x, cw.y, cw.z};
    const float oi[3] = {gi.x, gi.y, gi.z};
    const float4 di = f.dyn[i];
    const float vi[3] = {di.x, di.y, di.z};
    const float rho_i = k.rho0 + f.drho[i];
    Acc rate, pdis[3];
    auto pair = [&](const TiledRec2 &r) {
        float dx[3];
        tile_dx<D>(k.gs_f, cif, oi, r.c, r.o, dx);
        float r2 = sq<D>(dx);
        float inv = inv_dist(r2);
        float dWV = wc2_dWV(k.cW, k.inv_h, r2 * inv);
        const float dv[3] = {vi[0] - r.o.w, vi[1] - r.c.w, vi[2] - r.z};
        float u = dot<D>(dv, dx) * inv;
        rate.add(u * dWV);
        float sc = p_jump(k, u) * (dWV * inv);
#pragma unroll
        for (int d = 0; d < D; ++d)
            pdis[d].add(sc * dx[d]);
    };
    auto flush = [&]() {
        rate.flush();
#pragma unroll
        for (int d = 0; d < D; ++d)
            pdis[d].flush();
    };
    auto load = [&](uint32_t s) { return TiledRec2{sw.fa[s], sw.fb[s], sw.fc[s]}; };
    list_sweep<false, kUnrollSecond>(t, n, in, load, pair, flush);

    Acc wrate, wdis[3];
    auto wpair = [&](const TiledRec2 &r) {
        float dx[3];
        tile_dx<D>(k.gs_f, cif, oi, r.c, r.o, dx);
        float r2 = sq<D>(dx);
        float inv = inv_dist(r2);
        float dWV = wc2_dWV(k.cWw, k.inv_h, r2 * inv);
        const float nj[3] = {r.o.w, r.c.w, r.z};
        float en = dot<D>(dx, nj);
        float sgn = en < 0.f ? -1.f : (en > 0.f ? 1.f : 0.f);
        wrate.add(2.0f * (dot<D>(vi, dx) * inv) * dWV);
        float sc = p_jump(k, 2.0f * sgn * dot<D>(vi, nj)) * dWV * sgn;
#pragma unroll
        for (int d = 0; d < D; ++d)
            wdis[d].add(sc * nj[d]);
    };
    auto wflush = [&]() {
        wrate.flush();
#pragma unroll
        for (int d = 0; d < D; ++d)
            wdis[d].flush();
    };
    auto wload = [&](uint32_t s) { return TiledRec2{sw.wa[s], sw.wb[s], sw.wc[s]}; };
    list_sweep<false, kUnrollSecond>(t, n, wl, wload, wpair, wflush);

    float drho_dt = f.drho_dt[i] + rate.value() * rho_i + wrate.value() * rho_i;
    f.drho_dt[i] = drho_dt;
    f.drho[i] = f.drho[i] + drho_dt * float(0.5 * dt);
    float v2 = 0.f, a2 = 0.f;
#pragma unroll
    for (int d = 0; d < D; ++d)
    {
        float F = pdis[d].value() * k.Vol + wdis[d].value() * k.Vol;
        f.force[d * n + i] = F;
        half_step(f, n, i, d, dt, vi[d]);
        v2 += vi[d] * vi[d];
        float ft = F + k.mass * k.g[d];
        a2 += ft * ft;
    }
    return double(fmaxf(v2, 4.0f * float(k.h) * sqrtf(a2) * k.inv_mass));
}
} // namespace mpc
} // namespace sphx
