// Cell linked list (counting sort of particles into cells), device exclusive scan and
// the Morton particle sort.
//
// Reference: UpdateCellLinkedList (src/shared/shared_ck/particle_dynamics/
// configuration_dynamics/update_cell_linked_list.hpp:40-106), BaseCellLinkedList::
// UpdateCellLists (src/shared/meshes/cell_linked_list.cpp:84-101), Mesh cell hashing
// (src/shared/meshes/base_mesh.hxx:9-26,68-99), ParticleSorting
// (src/shared/particle_dynamics/configuration_dynamics/particle_sorting.cpp:25-58).
#include <algorithm>
#include <mutex>

#include "sphx_device.cuh"
#include "sphx_internal.cuh"

using namespace sphx;

namespace
{
constexpr unsigned kBlock = 256;
constexpr unsigned kScanItems = 8;                  // items per thread in the scan
constexpr unsigned kScanTile = kBlock * kScanItems; // items per block

// Hash every particle into its cell and take its arrival rank in that cell.
template <int D>
__global__ void k_hash_count(size_t n, const double *__restrict__ pos, MeshDev m, uint32_t *__restrict__ cell_of,
                             uint32_t *__restrict__ rank, uint32_t *__restrict__ count)
{
    size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    double x[3] = {0, 0, 0};
#pragma unroll
    for (int a = 0; a < D; ++a)
        x[a] = pos[a * n + i];
    int c[3];
    cell_index<D>(m, x, c);
    uint32_t lc = linear_cell<D>(m, c);
    cell_of[i] = lc;
    rank[i] = atomicAdd(&count[lc], 1u);
}

// Block-local exclusive scan helper: each thread owns kScanItems consecutive items.
__device__ uint32_t block_exclusive_scan(uint32_t v, uint32_t *smem_warp, uint32_t &block_total)
{
    const unsigned lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    uint32_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1)
    {
        uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= unsigned(o))
            x += y;
    }
    if (lane == 31)
        smem_warp[warp] = x;
    __syncthreads();
    if (warp == 0)
    {
        uint32_t w = lane < (blockDim.x >> 5) ? smem_warp[lane] : 0u;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1)
        {
            uint32_t y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= unsigned(o))
                w += y;
        }
        smem_warp[lane] = w;
    }
    __syncthreads();
    uint32_t warp_prefix = warp > 0 ? smem_warp[warp - 1] : 0u;
    block_total = smem_warp[(blockDim.x >> 5) - 1];
    __syncthreads();
    return warp_prefix + x - v;
}

// Pass 1: per-tile sums.
__global__ void k_scan_tile_sums(const uint32_t *__restrict__ in, size_t n, uint32_t *__restrict__ tile_sums)
{
    __shared__ uint32_t sw[32];
    size_t base = size_t(blockIdx.x) * kScanTile + size_t(threadIdx.x) * kScanItems;
    uint32_t s = 0;
#pragma unroll
    for (unsigned k = 0; k < kScanItems; ++k)
        if (base + k < n)
            s += in[base + k];
    uint32_t total;
    block_exclusive_scan(s, sw, total);
    if (threadIdx.x == 0)
        tile_sums[blockIdx.x] = total;
}

// Pass 2: exclusive scan of the tile sums by one block (loops over chunks).
__global__ void k_scan_tile_prefix(uint32_t *__restrict__ tile_sums, size_t ntiles, uint32_t *__restrict__ total_out)
{
    __shared__ uint32_t sw[32];
    uint32_t carry = 0;
    for (size_t base = 0; base < ntiles; base += blockDim.x)
    {
        size_t i = base + threadIdx.x;
        uint32_t v = i < ntiles ? tile_sums[i] : 0u;
        uint32_t tot;
        uint32_t ex = block_exclusive_scan(v, sw, tot);
        if (i < ntiles)
            tile_sums[i] = carry + ex;
        carry += tot;
        __syncthreads();
    }
    if (threadIdx.x == 0 && total_out)
        *total_out = carry;
}

// Pass 3: scan inside each tile, offset by the tile prefix.
__global__ void k_scan_apply(const uint32_t *__restrict__ in, uint32_t *__restrict__ out, size_t n,
                             const uint32_t *__restrict__ tile_prefix)
{
    __shared__ uint32_t sw[32];
    size_t base = size_t(blockIdx.x) * kScanTile + size_t(threadIdx.x) * kScanItems;
    uint32_t v[kScanItems];
    uint32_t s = 0;
#pragma unroll
    for (unsigned k = 0; k < kScanItems; ++k)
    {
        v[k] = base + k < n ? in[base + k] : 0u;
        s += v[k];
    }
    uint32_t total;
    uint32_t run = tile_prefix[blockIdx.x] + block_exclusive_scan(s, sw, total);
#pragma unroll
    for (unsigned k = 0; k < kScanItems; ++k)
        if (base + k < n)
        {
            out[base + k] = run;
            run += v[k];
        }
}

__global__ void k_count_keys(size_t n, const uint32_t *__restrict__ key, uint32_t *__restrict__ rank,
                             uint32_t *__restrict__ count)
{
    size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i < n)
        rank[i] = atomicAdd(&count[key[i]], 1u);
}

// offset[nkeys] = total, closing the CellOffset array (cell_linked_list.cpp:171-174).
__global__ void k_set_total(uint32_t *offset, uint32_t nkeys, uint32_t total) { offset[nkeys] = total; }

__global__ void k_scatter(size_t n, const uint32_t *__restrict__ cell_of, const uint32_t *__restrict__ rank,
                          const uint32_t *__restrict__ offset, uint32_t *__restrict__ particle_index)
{
    size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    const uint32_t slot = offset[cell_of[i]] + rank[i];
    if (SPHX_CHECKED(slot < n, kCheckCellRange, slot))
        particle_index[slot] = uint32_t(i);
}

// Puts each cell's particles in ascending index order.
__global__ void k_sort_segments(size_t nseg, const uint32_t *__restrict__ offset, uint32_t *__restrict__ idx)
{
    size_t c = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (c < nseg)
        sort_segment(idx, offset[c], offset[c + 1]);
}

// Cell-ordered copies of the positions: exact FP64 and the FP32 offset from the lower
// corner of the particle's cell (for the neighbour-search pre-filter).
template <int D>
__global__ void k_gather_sorted(size_t n, const uint32_t *__restrict__ idx, const uint32_t *__restrict__ cell_of,
                                const double *__restrict__ pos, MeshDev m, double *__restrict__ spos,
                                float *__restrict__ soff)
{
    size_t k = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (k >= n)
        return;
    uint32_t i = idx[k];
    int c[3];
    cell_from_linear<D>(m, cell_of[i], c);
#pragma unroll
    for (int a = 0; a < D; ++a)
    {
        double x = pos[a * n + i];
        spos[a * n + k] = x;
        soff[a * n + k] = float(x - cell_corner(m, a, c[a]));
    }
}

// ---------------------------------------------------------------- periodic images
__global__ void k_entry_init(size_t n, int dim, const double *__restrict__ pos, size_t E, double *__restrict__ epos,
                             uint32_t *__restrict__ eidx)
{
    size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    for (int a = 0; a < dim; ++a)
        epos[a * E + i] = pos[a * n + i];
    eidx[i] = uint32_t(i);
}

// 1 for the entries that get an image on this side: lower < x < lower + rc (side 0) or
// upper - rc < x < upper (side 1), strict as in domain_bounding.cpp:20-50
__global__ void k_image_flags(size_t n_cur, size_t E, const double *__restrict__ epos, int axis, double lo, double hi,
                              uint32_t *__restrict__ flag)
{
    size_t e = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (e >= n_cur)
        return;
    double x = epos[axis * E + e];
    flag[e] = (x > lo && x < hi) ? 1u : 0u;
}

__global__ void k_image_emit(size_t n_cur, int dim, size_t E, double *__restrict__ epos, uint32_t *__restrict__ eidx,
                             const uint32_t *__restrict__ flag, const uint32_t *__restrict__ scan, size_t base,
                             int axis, double shift)
{
    size_t e = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (e >= n_cur || !flag[e])
        return;
    size_t k = base + scan[e];
    for (int a = 0; a < dim; ++a)
        epos[a * E + k] = epos[a * E + e] + (a == axis ? shift : 0.0);
    eidx[k] = eidx[e];
}

template <int D>
__global__ void k_entry_hash(size_t ne, size_t E, const double *__restrict__ epos, MeshDev m,
                             uint32_t *__restrict__ cell_of, uint32_t *__restrict__ rank, uint32_t *__restrict__ count)
{
    size_t e = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (e >= ne)
        return;
    double x[3] = {0, 0, 0};
#pragma unroll
    for (int a = 0; a < D; ++a)
        x[a] = epos[a * E + e];
    int c[3];
    cell_index<D>(m, x, c);
    uint32_t lc = linear_cell<D>(m, c);
    cell_of[e] = lc;
    rank[e] = atomicAdd(&count[lc], 1u);
}

template <int D>
__global__ void k_entry_gather(size_t ne, const uint32_t *__restrict__ perm, const uint32_t *__restrict__ cell_of,
                               size_t E, const double *__restrict__ epos, const uint32_t *__restrict__ eidx,
                               MeshDev m, uint32_t *__restrict__ pidx, double *__restrict__ spos,
                               float *__restrict__ soff)
{
    size_t k = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (k >= ne)
        return;
    uint32_t e = perm[k];
    int c[3];
    cell_from_linear<D>(m, cell_of[e], c);
    pidx[k] = eidx[e];
#pragma unroll
    for (int a = 0; a < D; ++a)
    {
        double x = epos[a * E + e];
        spos[a * ne + k] = x;
        soff[a * ne + k] = float(x - cell_corner(m, a, c[a]));
    }
}

template <int D>
__global__ void k_periodic_bounding(size_t n, double *__restrict__ pos, int axis, double lower, double upper)
{
    size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    double x = pos[axis * n + i];
    double L = upper - lower;
    if (x < lower)
        x += L;
    if (x > upper)
        x -= L;
    pos[axis * n + i] = x;
}

template <int D>
__global__ void k_morton_key(size_t n, const double *__restrict__ pos, MeshDev m, uint32_t *__restrict__ key)
{
    size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    double x[3] = {0, 0, 0};
#pragma unroll
    for (int a = 0; a < D; ++a)
        x[a] = pos[a * n + i];
    int c[3];
    cell_index<D>(m, x, c);
    key[i] = morton_key<D>(c);
}

template <typename T>
__global__ void k_permute(size_t n, int ncomp, const uint32_t *__restrict__ perm, const T *__restrict__ src,
                          T *__restrict__ dst)
{
    size_t k = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (k >= n)
        return;
    uint32_t i = perm[k];
    for (int c = 0; c < ncomp; ++c)
        dst[c * n + k] = src[c * n + i];
}

__global__ void k_sorted_id(size_t n, const uint32_t *__restrict__ original_id, uint32_t *__restrict__ sorted_id)
{
    size_t k = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (k < n)
        sorted_id[original_id[k]] = uint32_t(k);
}

__global__ void k_morton_rank_key(size_t n, const double *__restrict__ pos, MeshDev m, int dim,
                                  const uint32_t *__restrict__ morton_rank, uint32_t *__restrict__ key)
{
    size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    double x[3] = {0, 0, 0};
    for (int a = 0; a < dim; ++a)
        x[a] = pos[a * n + i];
    int c[3];
    uint32_t lc;
    if (dim == 2)
    {
        cell_index<2>(m, x, c);
        lc = linear_cell<2>(m, c);
    }
    else
    {
        cell_index<3>(m, x, c);
        lc = linear_cell<3>(m, c);
    }
    key[i] = morton_rank[lc];
}
} // namespace

namespace sphx
{
int exclusive_scan(sphx_ctx ctx, const uint32_t *d_in, uint32_t *d_out, size_t n)
{
    if (n == 0)
        return SPHX_OK;
    size_t ntiles = (n + kScanTile - 1) / kScanTile;
    SPHX_TRY(ctx->ensure_scratch((ntiles + 1) * sizeof(uint32_t)));
    uint32_t *tiles = static_cast<uint32_t *>(ctx->d_scratch);
    k_scan_tile_sums<<<unsigned(ntiles), kBlock, 0, ctx->stream>>>(d_in, n, tiles);
    SPHX_LAUNCHED(ctx);
    k_scan_tile_prefix<<<1, 1024, 0, ctx->stream>>>(tiles, ntiles, tiles + ntiles);
    SPHX_LAUNCHED(ctx);
    k_scan_apply<<<unsigned(ntiles), kBlock, 0, ctx->stream>>>(d_in, d_out, n, tiles);
    SPHX_LAUNCHED(ctx);
    return SPHX_OK;
}

size_t scan_scratch_entries(size_t n) { return (n + kScanTile - 1) / kScanTile + 1; }

// The same three passes on a stream with caller-owned tile scratch of
// scan_scratch_entries(n) entries; enqueues only (no allocation, no synchronisation), so a
// stream capture may record it.
int exclusive_scan_into(cudaStream_t s, const uint32_t *d_in, uint32_t *d_out, size_t n, uint32_t *tiles)
{
    if (n == 0)
        return SPHX_OK;
    size_t ntiles = (n + kScanTile - 1) / kScanTile;
    k_scan_tile_sums<<<unsigned(ntiles), kBlock, 0, s>>>(d_in, n, tiles);
    SPHX_CUDA(cudaGetLastError());
    k_scan_tile_prefix<<<1, 1024, 0, s>>>(tiles, ntiles, tiles + ntiles);
    SPHX_CUDA(cudaGetLastError());
    k_scan_apply<<<unsigned(ntiles), kBlock, 0, s>>>(d_in, d_out, n, tiles);
    SPHX_CUDA(cudaGetLastError());
    return SPHX_OK;
}

// Stable counting sort of n keys in [0, nkeys): d_offset[nkeys+1] gets the key offsets,
// d_perm[k] the index of the k-th particle in key order (ascending index within a key).
int counting_sort_by_key(sphx_ctx ctx, const uint32_t *d_key, size_t n, uint32_t nkeys, uint32_t *d_offset,
                         uint32_t *d_count, uint32_t *d_rank, uint32_t *d_perm)
{
    cudaStream_t s = ctx->stream;
    SPHX_CUDA(cudaMemsetAsync(d_count, 0, size_t(nkeys) * sizeof(uint32_t), s));
    SPHX_CUDA(cudaMemsetAsync(d_offset + nkeys, 0, sizeof(uint32_t), s));
    if (n == 0)
    {
        SPHX_CUDA(cudaMemsetAsync(d_offset, 0, size_t(nkeys) * sizeof(uint32_t), s));
        return SPHX_OK;
    }
    k_count_keys<<<grid_for(n, kBlock), kBlock, 0, s>>>(n, d_key, d_rank, d_count);
    SPHX_LAUNCHED(ctx);
    SPHX_TRY(exclusive_scan(ctx, d_count, d_offset, nkeys));
    k_set_total<<<1, 1, 0, s>>>(d_offset, nkeys, uint32_t(n));
    SPHX_LAUNCHED(ctx);
    k_scatter<<<grid_for(n, kBlock), kBlock, 0, s>>>(n, d_key, d_rank, d_offset, d_perm);
    SPHX_LAUNCHED(ctx);
    k_sort_segments<<<grid_for(nkeys, kBlock), kBlock, 0, s>>>(nkeys, d_offset, d_perm);
    SPHX_LAUNCHED(ctx);
    return SPHX_OK;
}
} // namespace sphx

// Entry buffers of at least ne entries; the first `keep` entries survive a regrowth (the
// SoA stride changes with the capacity).
int sphx_cell_list_s::reserve_entries(size_t ne, size_t keep)
{
    if (ne <= entry_cap && entry_pos)
        return SPHX_OK;
    size_t cap = std::max<size_t>(ne + ne / 2, 64);
    double *pos = nullptr;
    uint32_t *idx = nullptr, *flag = nullptr, *scan = nullptr, *perm = nullptr;
    SPHX_CUDA(cudaMalloc(&pos, 3 * cap * sizeof(double)));
    SPHX_CUDA(cudaMalloc(&idx, cap * sizeof(uint32_t)));
    SPHX_CUDA(cudaMalloc(&flag, cap * sizeof(uint32_t)));
    SPHX_CUDA(cudaMalloc(&scan, cap * sizeof(uint32_t)));
    SPHX_CUDA(cudaMalloc(&perm, cap * sizeof(uint32_t)));
    if (keep && entry_pos)
    {
        for (int a = 0; a < mesh.dim; ++a)
            SPHX_CUDA(cudaMemcpyAsync(pos + a * cap, entry_pos + a * entry_cap, keep * sizeof(double),
                                      cudaMemcpyDeviceToDevice, ctx->stream));
        SPHX_CUDA(cudaMemcpyAsync(idx, entry_idx, keep * sizeof(uint32_t), cudaMemcpyDeviceToDevice, ctx->stream));
        SPHX_CUDA(cudaStreamSynchronize(ctx->stream));
    }
    cudaFree(entry_pos);
    cudaFree(entry_idx);
    cudaFree(entry_flag);
    cudaFree(entry_scan);
    cudaFree(entry_perm);
    entry_pos = pos;
    entry_idx = idx;
    entry_flag = flag;
    entry_scan = scan;
    entry_perm = perm;
    entry_cap = cap;
    return SPHX_OK;
}

int sphx_cell_list_s::reserve(size_t np)
{
    if (np <= capacity && particle_index)
        return SPHX_OK;
    cudaFree(particle_index);
    cudaFree(cell_of);
    cudaFree(rank);
    cudaFree(sorted_pos);
    cudaFree(sorted_off);
    particle_index = cell_of = rank = nullptr;
    sorted_pos = nullptr;
    sorted_off = nullptr;
    size_t cap = std::max<size_t>(np, 1);
    SPHX_CUDA(cudaMalloc(&particle_index, std::max(cap, ncells) * sizeof(uint32_t)));
    SPHX_CUDA(cudaMalloc(&cell_of, cap * sizeof(uint32_t)));
    SPHX_CUDA(cudaMalloc(&rank, cap * sizeof(uint32_t)));
    SPHX_CUDA(cudaMalloc(&sorted_pos, 3 * cap * sizeof(double)));
    SPHX_CUDA(cudaMalloc(&sorted_off, 3 * cap * sizeof(float)));
    capacity = cap;
    return SPHX_OK;
}

extern "C" int sphx_cell_list_create(sphx_ctx ctx, const sphx_mesh_desc *mesh, size_t particle_capacity,
                                     sphx_cell_list *out)
{
    if (!ctx || !mesh || !out || (mesh->dim != 2 && mesh->dim != 3) || !(mesh->grid_spacing > 0))
        return fail(SPHX_ERR_INVALID_ARG, "invalid cell list arguments");
    size_t nc = 1;
    for (int a = 0; a < mesh->dim; ++a)
    {
        if (mesh->all_cells[a] < 1)
            return fail(SPHX_ERR_INVALID_ARG, "mesh axis %d has no cells", a);
        nc *= size_t(mesh->all_cells[a]);
    }
    if (nc >= 0xffffffffull)
        return fail(SPHX_ERR_INVALID_ARG, "mesh of %zu cells exceeds 32-bit cell indices", nc);
    sphx_cell_list cl = new sphx_cell_list_s();
    cl->ctx = ctx;
    ctx->retain();
    cl->mesh = *mesh;
    cl->ncells = nc;
    SPHX_CUDA(cudaMalloc(&cl->cell_offset, (nc + 1) * sizeof(uint32_t)));
    SPHX_CUDA(cudaMalloc(&cl->cell_count, nc * sizeof(uint32_t)));
    SPHX_CUDA(cudaMemsetAsync(cl->cell_offset, 0, (nc + 1) * sizeof(uint32_t), ctx->stream));
    int st = cl->reserve(particle_capacity);
    if (st != SPHX_OK)
    {
        sphx_cell_list_destroy(cl);
        return st;
    }
    *out = cl;
    return SPHX_OK;
}

extern "C" int sphx_cell_list_destroy(sphx_cell_list cl)
{
    if (!cl)
        return SPHX_OK;
    cudaStreamSynchronize(cl->ctx->stream);
    cudaFree(cl->cell_offset);
    cudaFree(cl->cell_count);
    cudaFree(cl->particle_index);
    cudaFree(cl->cell_of);
    cudaFree(cl->rank);
    cudaFree(cl->sorted_pos);
    cudaFree(cl->sorted_off);
    cudaFree(cl->entry_pos);
    cudaFree(cl->entry_idx);
    cudaFree(cl->entry_flag);
    cudaFree(cl->entry_scan);
    cudaFree(cl->entry_perm);
    sphx_ctx ctx = cl->ctx;
    delete cl;
    release(ctx);
    return SPHX_OK;
}

namespace
{
// Cell list of the particles and their periodic images: entries are generated axis by axis
// (lower-side images of all current entries, then upper-side ones, in entry order), then
// sorted into cells by a stable counting sort of the entry numbers.
int update_periodic(sphx_cell_list cl, sphx_body body, const double *pos)
{
    sphx_ctx ctx = cl->ctx;
    cudaStream_t s = ctx->stream;
    const int D = body->dim;
    size_t n = body->n;
    SPHX_TRY(cl->reserve_entries(2 * n + 64, 0));
    if (n > 0)
    {
        k_entry_init<<<grid_for(n, kBlock), kBlock, 0, s>>>(n, D, pos, cl->entry_cap, cl->entry_pos, cl->entry_idx);
        SPHX_LAUNCHED(ctx);
    }
    size_t n_cur = n;
    for (int a = 0; a < D; ++a)
    {
        if (!(cl->periodic_mask & (1 << a)))
            continue;
        double lo = cl->per_lower[a], up = cl->per_upper[a], rc = cl->per_cutoff, L = up - lo;
        size_t n_axis = n_cur; // the entries this axis images (both sides)
        for (int side = 0; side < 2; ++side)
        {
            if (n_axis == 0)
                break;
            double band_lo = side == 0 ? lo : up - rc, band_hi = side == 0 ? lo + rc : up;
            k_image_flags<<<grid_for(n_axis, kBlock), kBlock, 0, s>>>(n_axis, cl->entry_cap, cl->entry_pos, a,
                                                                       band_lo, band_hi, cl->entry_flag);
            SPHX_LAUNCHED(ctx);
            uint32_t total = 0;
            SPHX_TRY(exclusive_scan(ctx, cl->entry_flag, cl->entry_scan, n_axis));
            // total = last scan value + last flag
            uint32_t last[2] = {0, 0};
            SPHX_CUDA(cudaMemcpyAsync(&last[0], cl->entry_scan + n_axis - 1, 4, cudaMemcpyDeviceToHost, s));
            SPHX_CUDA(cudaMemcpyAsync(&last[1], cl->entry_flag + n_axis - 1, 4, cudaMemcpyDeviceToHost, s));
            SPHX_CUDA(cudaStreamSynchronize(s));
            total = last[0] + last[1];
            if (total == 0)
                continue;
            if (n_cur + total > cl->entry_cap)
            {
                // regrowth keeps the entries generated so far; flags and scan are recomputed
                SPHX_TRY(cl->reserve_entries(n_cur + total, n_cur));
                k_image_flags<<<grid_for(n_axis, kBlock), kBlock, 0, s>>>(n_axis, cl->entry_cap, cl->entry_pos, a,
                                                                           band_lo, band_hi, cl->entry_flag);
                SPHX_LAUNCHED(ctx);
                SPHX_TRY(exclusive_scan(ctx, cl->entry_flag, cl->entry_scan, n_axis));
            }
            k_image_emit<<<grid_for(n_axis, kBlock), kBlock, 0, s>>>(n_axis, D, cl->entry_cap, cl->entry_pos,
                                                                      cl->entry_idx, cl->entry_flag, cl->entry_scan,
                                                                      n_cur, a, side == 0 ? L : -L);
            SPHX_LAUNCHED(ctx);
            n_cur += total;
        }
    }
    size_t ne = n_cur;
    SPHX_TRY(cl->reserve(ne));
    cl->n = n;
    cl->n_entries = ne;
    MeshDev m = mesh_dev(cl->mesh);
    SPHX_CUDA(cudaMemsetAsync(cl->cell_count, 0, cl->ncells * sizeof(uint32_t), s));
    if (ne > 0)
    {
        if (D == 2)
            k_entry_hash<2><<<grid_for(ne, kBlock), kBlock, 0, s>>>(ne, cl->entry_cap, cl->entry_pos, m, cl->cell_of,
                                                                    cl->rank, cl->cell_count);
        else
            k_entry_hash<3><<<grid_for(ne, kBlock), kBlock, 0, s>>>(ne, cl->entry_cap, cl->entry_pos, m, cl->cell_of,
                                                                    cl->rank, cl->cell_count);
        SPHX_LAUNCHED(ctx);
    }
    SPHX_TRY(exclusive_scan(ctx, cl->cell_count, cl->cell_offset, cl->ncells));
    k_set_total<<<1, 1, 0, s>>>(cl->cell_offset, uint32_t(cl->ncells), uint32_t(ne));
    SPHX_LAUNCHED(ctx);
    if (ne == 0)
        return SPHX_OK;
    if (cl->entry_cap < ne)
        SPHX_TRY(cl->reserve_entries(ne, ne));
    k_scatter<<<grid_for(ne, kBlock), kBlock, 0, s>>>(ne, cl->cell_of, cl->rank, cl->cell_offset, cl->entry_perm);
    SPHX_LAUNCHED(ctx);
    k_sort_segments<<<grid_for(cl->ncells, kBlock), kBlock, 0, s>>>(cl->ncells, cl->cell_offset, cl->entry_perm);
    SPHX_LAUNCHED(ctx);
    if (D == 2)
        k_entry_gather<2><<<grid_for(ne, kBlock), kBlock, 0, s>>>(ne, cl->entry_perm, cl->cell_of, cl->entry_cap,
                                                                  cl->entry_pos, cl->entry_idx, m, cl->particle_index,
                                                                  cl->sorted_pos, cl->sorted_off);
    else
        k_entry_gather<3><<<grid_for(ne, kBlock), kBlock, 0, s>>>(ne, cl->entry_perm, cl->cell_of, cl->entry_cap,
                                                                  cl->entry_pos, cl->entry_idx, m, cl->particle_index,
                                                                  cl->sorted_pos, cl->sorted_off);
    SPHX_LAUNCHED(ctx);
    return SPHX_OK;
}
} // namespace

extern "C" int sphx_cell_list_set_periodic(sphx_cell_list cl, int axis, double lower, double upper, double cutoff)
{
    if (!cl || axis < 0 || axis >= cl->mesh.dim || !(upper > lower) || !(cutoff > 0) ||
        !(2.0 * cutoff < upper - lower))
        return fail(SPHX_ERR_INVALID_ARG, "invalid periodic axis (axis %d, [%g, %g], cut-off %g)", axis, lower, upper,
                    cutoff);
    cl->periodic_mask |= 1 << axis;
    cl->per_lower[axis] = lower;
    cl->per_upper[axis] = upper;
    cl->per_cutoff = cutoff;
    return SPHX_OK;
}

extern "C" int sphx_cell_list_num_entries(sphx_cell_list cl, size_t *n_entries)
{
    if (!cl || !n_entries)
        return fail(SPHX_ERR_INVALID_ARG, "null argument");
    *n_entries = cl->n_entries;
    return SPHX_OK;
}

extern "C" int sphx_periodic_bounding(sphx_body body, int axis, double lower, double upper)
{
    if (!body || axis < 0 || axis >= body->dim || !(upper > lower))
        return fail(SPHX_ERR_INVALID_ARG, "invalid periodic bounding");
    Field *pos;
    SPHX_TRY(body->need("Position", SPHX_F64, body->dim, &pos));
    if (body->n == 0)
        return SPHX_OK;
    double *p = static_cast<double *>(pos->dev);
    if (body->dim == 2)
        k_periodic_bounding<2><<<grid_for(body->n, kBlock), kBlock, 0, body->ctx->stream>>>(body->n, p, axis, lower,
                                                                                           upper);
    else
        k_periodic_bounding<3><<<grid_for(body->n, kBlock), kBlock, 0, body->ctx->stream>>>(body->n, p, axis, lower,
                                                                                           upper);
    SPHX_LAUNCHED(body->ctx);
    return SPHX_OK;
}

extern "C" int sphx_cell_list_update(sphx_cell_list cl, sphx_body body)
{
    if (!cl || !body)
        return fail(SPHX_ERR_INVALID_ARG, "null argument");
    if (body->dim != cl->mesh.dim)
        return fail(SPHX_ERR_INVALID_ARG, "body dimension %d differs from mesh dimension %d", body->dim, cl->mesh.dim);
    Field *pos;
    SPHX_TRY(body->need("Position", SPHX_F64, body->dim, &pos));
    sphx_ctx ctx = cl->ctx;
    size_t n = body->n;
    if (cl->periodic_mask)
        return update_periodic(cl, body, static_cast<const double *>(pos->dev));
    SPHX_TRY(cl->reserve(n));
    cl->n = n;
    cl->n_entries = n;
    cudaStream_t s = ctx->stream;
    MeshDev m = mesh_dev(cl->mesh);
    const double *p = static_cast<const double *>(pos->dev);
    SPHX_CUDA(cudaMemsetAsync(cl->cell_count, 0, cl->ncells * sizeof(uint32_t), s));
    if (n > 0)
    {
        if (body->dim == 2)
            k_hash_count<2><<<grid_for(n, kBlock), kBlock, 0, s>>>(n, p, m, cl->cell_of, cl->rank, cl->cell_count);
        else
            k_hash_count<3><<<grid_for(n, kBlock), kBlock, 0, s>>>(n, p, m, cl->cell_of, cl->rank, cl->cell_count);
        SPHX_LAUNCHED(ctx);
    }
    SPHX_TRY(exclusive_scan(ctx, cl->cell_count, cl->cell_offset, cl->ncells));
    k_set_total<<<1, 1, 0, s>>>(cl->cell_offset, uint32_t(cl->ncells), uint32_t(n));
    SPHX_LAUNCHED(ctx);
    if (n == 0)
        return SPHX_OK;
    k_scatter<<<grid_for(n, kBlock), kBlock, 0, s>>>(n, cl->cell_of, cl->rank, cl->cell_offset, cl->particle_index);
    SPHX_LAUNCHED(ctx);
    k_sort_segments<<<grid_for(cl->ncells, kBlock), kBlock, 0, s>>>(cl->ncells, cl->cell_offset, cl->particle_index);
    SPHX_LAUNCHED(ctx);
    if (body->dim == 2)
        k_gather_sorted<2><<<grid_for(n, kBlock), kBlock, 0, s>>>(n, cl->particle_index, cl->cell_of, p, m,
                                                                  cl->sorted_pos, cl->sorted_off);
    else
        k_gather_sorted<3><<<grid_for(n, kBlock), kBlock, 0, s>>>(n, cl->particle_index, cl->cell_of, p, m,
                                                                  cl->sorted_pos, cl->sorted_off);
    SPHX_LAUNCHED(ctx);
    return SPHX_OK;
}

extern "C" int sphx_cell_list_num_cells(sphx_cell_list cl, size_t *ncells)
{
    if (!cl || !ncells)
        return fail(SPHX_ERR_INVALID_ARG, "null argument");
    *ncells = cl->ncells;
    return SPHX_OK;
}

extern "C" int sphx_cell_list_download(sphx_cell_list cl, uint32_t *cell_offset, uint32_t *particle_index, size_t n)
{
    if (!cl)
        return fail(SPHX_ERR_INVALID_ARG, "null cell list");
    if (n != cl->n)
        return fail(SPHX_ERR_INVALID_ARG, "cell list holds %zu particles, not %zu", cl->n, n);
    cudaStream_t s = cl->ctx->stream;
    if (cell_offset)
        SPHX_CUDA(cudaMemcpyAsync(cell_offset, cl->cell_offset, (cl->ncells + 1) * sizeof(uint32_t),
                                  cudaMemcpyDeviceToHost, s));
    if (particle_index && n > 0)
        SPHX_CUDA(cudaMemcpyAsync(particle_index, cl->particle_index, n * sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
    SPHX_CUDA(cudaStreamSynchronize(s));
    return SPHX_OK;
}

extern "C" int sphx_exclusive_scan_u32(sphx_ctx ctx, const uint32_t *d_in, uint32_t *d_out, size_t n, uint32_t *total)
{
    if (!ctx || (n > 0 && (!d_in || !d_out)))
        return fail(SPHX_ERR_INVALID_ARG, "invalid scan arguments");
    if (n == 0)
    {
        if (total)
            *total = 0;
        return SPHX_OK;
    }
    // The last entry of the input participates in the total only.
    SPHX_TRY(exclusive_scan(ctx, d_in, d_out, n));
    if (total)
    {
        uint32_t last_in = 0, last_out = 0;
        SPHX_CUDA(cudaMemcpyAsync(&last_in, d_in + n - 1, sizeof(uint32_t), cudaMemcpyDeviceToHost, ctx->stream));
        SPHX_CUDA(cudaMemcpyAsync(&last_out, d_out + n - 1, sizeof(uint32_t), cudaMemcpyDeviceToHost, ctx->stream));
        SPHX_CUDA(cudaStreamSynchronize(ctx->stream));
        *total = last_out + last_in;
    }
    return SPHX_OK;
}

extern "C" int sphx_particle_sorting(sphx_body body, const sphx_mesh_desc *mesh)
{
    if (!body || !mesh || mesh->dim != body->dim)
        return fail(SPHX_ERR_INVALID_ARG, "invalid sorting arguments");
    sphx_ctx ctx = body->ctx;
    cudaStream_t s = ctx->stream;
    size_t n = body->n;
    Field *pos, *oid, *sid;
    SPHX_TRY(body->need("Position", SPHX_F64, body->dim, &pos));
    SPHX_TRY(body->require("OriginalID", SPHX_U32, 1, &oid));
    SPHX_TRY(body->require("SortedID", SPHX_U32, 1, &sid));
    if (n == 0)
        return SPHX_OK;
    size_t nc = 1;
    for (int a = 0; a < mesh->dim; ++a)
    {
        if (mesh->all_cells[a] > 1024)
            return fail(SPHX_ERR_INVALID_ARG, "Morton keys hold 10 bits per axis; mesh axis %d has %d cells", a,
                        mesh->all_cells[a]);
        nc *= size_t(mesh->all_cells[a]);
    }
    // Rank of each cell in Morton order (cells with distinct keys; keys are unique per cell).
    std::vector<uint32_t> key_of_cell(nc);
    std::vector<uint32_t> order(nc);
    for (size_t lc = 0; lc < nc; ++lc)
    {
        int c[3];
        size_t r = lc;
        if (mesh->dim == 2)
        {
            c[1] = int(r % mesh->all_cells[1]);
            c[0] = int(r / mesh->all_cells[1]);
            key_of_cell[lc] = morton_key<2>(c);
        }
        else
        {
            c[2] = int(r % mesh->all_cells[2]);
            r /= mesh->all_cells[2];
            c[1] = int(r % mesh->all_cells[1]);
            c[0] = int(r / mesh->all_cells[1]);
            key_of_cell[lc] = morton_key<3>(c);
        }
        order[lc] = uint32_t(lc);
    }
    std::sort(order.begin(), order.end(), [&](uint32_t a, uint32_t b) { return key_of_cell[a] < key_of_cell[b]; });
    std::vector<uint32_t> rank_of_cell(nc);
    for (size_t r = 0; r < nc; ++r)
        rank_of_cell[order[r]] = uint32_t(r);
    // device buffers: morton_rank[nc], key[n], offset[nc+1], count[nc], rank[n], perm[n], tmp
    size_t words = nc + n + (nc + 1) + nc + n + n;
    size_t max_field = 0;
    for (auto &kv : body->fields)
        max_field = std::max(max_field, size_t(kv.second.ncomp) * dtype_size(kv.second.dtype));
    size_t tmp_bytes = max_field * n;
    uint32_t *buf = nullptr;
    void *tmp = nullptr;
    SPHX_CUDA(cudaMallocAsync((void **)&buf, words * sizeof(uint32_t), s));
    SPHX_CUDA(cudaMallocAsync(&tmp, tmp_bytes, s));
    uint32_t *d_mrank = buf, *d_key = d_mrank + nc, *d_off = d_key + n, *d_cnt = d_off + nc + 1,
             *d_rank = d_cnt + nc, *d_perm = d_rank + n;
    SPHX_CUDA(cudaMemcpyAsync(d_mrank, rank_of_cell.data(), nc * sizeof(uint32_t), cudaMemcpyHostToDevice, s));
    k_morton_rank_key<<<grid_for(n, kBlock), kBlock, 0, s>>>(n, static_cast<const double *>(pos->dev),
                                                              mesh_dev(*mesh), body->dim, d_mrank, d_key);
    SPHX_LAUNCHED(ctx);
    SPHX_TRY(counting_sort_by_key(ctx, d_key, n, uint32_t(nc), d_off, d_cnt, d_rank, d_perm));
    for (auto &kv : body->fields)
    {
        if (kv.first == "SortedID")
            continue;
        Field &f = kv.second;
        size_t bytes = n * f.ncomp * dtype_size(f.dtype);
        if (f.dtype == SPHX_F64)
            k_permute<double><<<grid_for(n, kBlock), kBlock, 0, s>>>(n, f.ncomp, d_perm,
                                                                     static_cast<const double *>(f.dev),
                                                                     static_cast<double *>(tmp));
        else
            k_permute<uint32_t><<<grid_for(n, kBlock), kBlock, 0, s>>>(n, f.ncomp, d_perm,
                                                                       static_cast<const uint32_t *>(f.dev),
                                                                       static_cast<uint32_t *>(tmp));
        SPHX_LAUNCHED(ctx);
        SPHX_CUDA(cudaMemcpyAsync(f.dev, tmp, bytes, cudaMemcpyDeviceToDevice, s));
    }
    k_sorted_id<<<grid_for(n, kBlock), kBlock, 0, s>>>(n, static_cast<const uint32_t *>(oid->dev),
                                                        static_cast<uint32_t *>(sid->dev));
    SPHX_LAUNCHED(ctx);
    SPHX_CUDA(cudaFreeAsync(buf, s));
    SPHX_CUDA(cudaFreeAsync(tmp, s));
    SPHX_CUDA(cudaStreamSynchronize(s));
    return SPHX_OK;
}

// ---------------------------------------------------------------------------------------
// Exclusive scan that allocates nothing.
//
// Some callers cannot allocate device memory while they run: an application whose device
// memory belongs to another allocator (a framework's caching pool that has reserved the
// GPU and forbids allocations behind its back), or a time-stepping loop that must not pay
// the implicit device-wide synchronisation of cudaMalloc / cudaFree.  This entry point
// computes the same result as sphx_exclusive_scan_u32 with its per-tile partial sums in a
// fixed device array of this library instead of the context's growable scratch buffer.
//
// The array is a file-scope __device__ variable: every GPU that loads the library holds
// it (kNoAllocScanMaxTiles + 1 words, 128 KiB) until the process exits.  Host code cannot
// use the array's name as a device address, so the first call on each device looks the
// address up with cudaGetSymbolAddress (with that device current) and caches it; make that
// first call before any stream capture.  All calls share the one array and it keeps the
// last call's contents; every word a call reads is written earlier in the same call, so
// nothing has to be cleared first.  Calls whose work overlaps on the GPU (two streams,
// or two host threads at once) race on the array: serialise them on one stream.
constexpr size_t kNoAllocScanMaxTiles = 32768;
constexpr size_t kNoAllocScanMaxN = kNoAllocScanMaxTiles * kScanTile; // 67,108,864 entries

static __device__ __align__(256) uint32_t g_noalloc_scan_scratch[kNoAllocScanMaxTiles + 1];

namespace
{
constexpr int kNoAllocMaxDevices = 64;
std::mutex g_noalloc_mutex;
uint32_t *g_noalloc_scratch_ptr[kNoAllocMaxDevices] = {};

// Device address of the scratch array on the current device (looked up once per device).
int noalloc_scratch(uint32_t **out)
{
    int device = -1;
    SPHX_CUDA(cudaGetDevice(&device));
    if (device < 0 || device >= kNoAllocMaxDevices)
        return fail(SPHX_ERR_INVALID_ARG, "device %d beyond the %d devices the scratch table covers", device,
                    kNoAllocMaxDevices);
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    if (!g_noalloc_scratch_ptr[device])
    {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scan_scratch);
        if (e != cudaSuccess)
            return cuda_fail(e, "cudaGetSymbolAddress(g_noalloc_scan_scratch)", __FILE__, __LINE__);
        g_noalloc_scratch_ptr[device] = static_cast<uint32_t *>(p);
    }
    *out = g_noalloc_scratch_ptr[device];
    return SPHX_OK;
}
} // namespace

extern "C" int sphx_exclusive_scan_u32_noalloc(void *stream, const uint32_t *d_in, uint32_t *d_out, size_t n,
                                               uint32_t *total)
{
    if (n > 0 && (!d_in || !d_out))
        return fail(SPHX_ERR_INVALID_ARG, "null device buffer");
    if (n > kNoAllocScanMaxN)
        return fail(SPHX_ERR_INVALID_ARG,
                    "sphx_exclusive_scan_u32_noalloc scans at most %zu entries (fixed scratch); got %zu",
                    kNoAllocScanMaxN, n);
    if (n == 0)
    {
        if (total)
            *total = 0;
        return SPHX_OK;
    }
    uint32_t *tiles = nullptr;
    SPHX_TRY(noalloc_scratch(&tiles));
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    size_t ntiles = (n + kScanTile - 1) / kScanTile;
    k_scan_tile_sums<<<unsigned(ntiles), kBlock, 0, s>>>(d_in, n, tiles);
    SPHX_CUDA(cudaGetLastError());
    k_scan_tile_prefix<<<1, 1024, 0, s>>>(tiles, ntiles, tiles + ntiles);
    SPHX_CUDA(cudaGetLastError());
    k_scan_apply<<<unsigned(ntiles), kBlock, 0, s>>>(d_in, d_out, n, tiles);
    SPHX_CUDA(cudaGetLastError());
    if (total)
    {
        SPHX_CUDA(cudaMemcpyAsync(total, tiles + ntiles, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
        SPHX_CUDA(cudaStreamSynchronize(s));
    }
    return SPHX_OK;
}
