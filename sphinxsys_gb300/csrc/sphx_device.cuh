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
} // namespace sphx
