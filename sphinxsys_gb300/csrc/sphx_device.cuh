// Device-side mesh hashing shared by the kernels.
//
// Mesh::CellIndexFromPosition (src/shared/meshes/base_mesh.hxx:9-15): floor of the
// offset over the grid spacing, clamped to [0, all_grid_points - 2]; linear index
// row-major with the last axis fastest (base_mesh.hxx:68-78); Morton code with 10 bits
// per axis (base_mesh.hxx:80-99).
#pragma once

#include "sphx_internal.cuh"

namespace sphx
{
template <int D>
__device__ __forceinline__ void cell_index(const MeshDev &m, const double *x, int *c)
{
#pragma unroll
    for (int a = 0; a < D; ++a)
    {
        double f = floor((x[a] - m.lower[a]) / m.gs);
        int k = f < 0.0 ? 0 : (f > double(m.grid_points[a] - 2) ? m.grid_points[a] - 2 : int(f));
        c[a] = k;
    }
}

template <int D>
__device__ __forceinline__ uint32_t linear_cell(const MeshDev &m, const int *c)
{
    if (D == 2)
        return uint32_t(c[0]) * uint32_t(m.all_cells[1]) + uint32_t(c[1]);
    return uint32_t(c[0]) * uint32_t(m.all_cells[1]) * uint32_t(m.all_cells[2]) +
           uint32_t(c[1]) * uint32_t(m.all_cells[2]) + uint32_t(c[2]);
}

template <int D>
__device__ __forceinline__ void cell_from_linear(const MeshDev &m, uint32_t lc, int *c)
{
    if (D == 2)
    {
        c[1] = int(lc % uint32_t(m.all_cells[1]));
        c[0] = int(lc / uint32_t(m.all_cells[1]));
    }
    else
    {
        c[2] = int(lc % uint32_t(m.all_cells[2]));
        lc /= uint32_t(m.all_cells[2]);
        c[1] = int(lc % uint32_t(m.all_cells[1]));
        c[0] = int(lc / uint32_t(m.all_cells[1]));
    }
}

// Lower corner of cell index k along axis a.
__host__ __device__ __forceinline__ double cell_corner(const MeshDev &m, int a, int k)
{
    return m.lower[a] + double(k) * m.gs;
}

__host__ __device__ __forceinline__ uint32_t morton_code(uint32_t i)
{
    uint32_t x = i & 0x3ffu;
    x = (x | x << 16) & 0x30000ffu;
    x = (x | x << 8) & 0x300f00fu;
    x = (x | x << 4) & 0x30c30c3u;
    x = (x | x << 2) & 0x9249249u;
    return x;
}

template <int D>
__host__ __device__ __forceinline__ uint32_t morton_key(const int *c)
{
    if (D == 2)
        return morton_code(uint32_t(c[0])) | (morton_code(uint32_t(c[1])) << 1);
    return morton_code(uint32_t(c[0])) | (morton_code(uint32_t(c[1])) << 1) | (morton_code(uint32_t(c[2])) << 2);
}

// Order-preserving map of a double onto uint64 (for atomicMax of signed values).
__device__ __forceinline__ unsigned long long ordered_bits(double v)
{
    unsigned long long b = __double_as_longlong(v);
    return (b & 0x8000000000000000ull) ? ~b : (b | 0x8000000000000000ull);
}
__host__ __device__ __forceinline__ double from_ordered_bits(unsigned long long b)
{
    unsigned long long r = (b & 0x8000000000000000ull) ? (b & 0x7fffffffffffffffull) : ~b;
    double d;
    memcpy(&d, &r, sizeof(d));
    return d;
}

// atomicMax of v over the lanes that reach this call together: one atomic per group of
// converged lanes instead of one per lane on a single contended address.
__device__ __forceinline__ void warp_atomic_max(unsigned int *addr, unsigned int v)
{
    const unsigned mask = __activemask();
    const unsigned m = __reduce_max_sync(mask, v);
    if ((threadIdx.x & 31u) == unsigned(__ffs(mask) - 1))
        atomicMax(addr, m);
}

// Sorts the len distinct entries idx[b, b + len) held in R registers: all loads issued
// before any compare (one memory latency), R rounds of odd-even transposition, stores.
template <int R>
__device__ __forceinline__ void sort_in_registers(uint32_t *idx, uint32_t b, uint32_t len)
{
    uint32_t v[R];
#pragma unroll
    for (int q = 0; q < R; ++q)
        v[q] = uint32_t(q) < len ? idx[b + q] : 0xffffffffu;
#pragma unroll
    for (int r = 0; r < R; ++r)
    {
#pragma unroll
        for (int q = r & 1; q + 1 < R; q += 2)
        {
            const uint32_t lo = min(v[q], v[q + 1]), hi = max(v[q], v[q + 1]);
            v[q] = lo;
            v[q + 1] = hi;
        }
    }
#pragma unroll
    for (int q = 0; q < R; ++q)
        if (uint32_t(q) < len)
            idx[b + q] = v[q];
}

// Puts the entries of one cell segment idx[b, e) (distinct particle indices, in the order
// of the atomic ranks) in ascending order, so the cell order does not depend on the order
// in which the atomics ran.  Segments of up to 16 entries are sorted in registers; an
// insertion sort in memory, whose dependent loads cost a latency each, takes the rest.
__device__ __forceinline__ void sort_segment(uint32_t *idx, uint32_t b, uint32_t e)
{
    const uint32_t len = e - b;
    if (len < 2)
        return;
    if (len <= 4)
        sort_in_registers<4>(idx, b, len);
    else if (len <= 8)
        sort_in_registers<8>(idx, b, len);
    else if (len <= 16)
        sort_in_registers<16>(idx, b, len);
    else
        for (uint32_t k = b + 1; k < e; ++k)
        {
            const uint32_t v = idx[k];
            uint32_t q = k;
            while (q > b && idx[q - 1] > v)
            {
                idx[q] = idx[q - 1];
                --q;
            }
            idx[q] = v;
        }
}
} // namespace sphx
