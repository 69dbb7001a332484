// Internal declarations shared by the translation units of libsphx_cuda.so.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <map>
#include <string>
#include <vector>

#include "../../include/sphx/sphx.h"
#include "sphx_check.cuh"

namespace sphx
{
// TinyReal of the reference (src/shared/common/base_data_type.h:207).
constexpr double kTinyReal = 2.71051e-20;

int fail(int code, const char *fmt, ...);
int cuda_fail(cudaError_t e, const char *what, const char *file, int line);

#define SPHX_CUDA(call)                                                                                            \
    do                                                                                                             \
    {                                                                                                              \
        cudaError_t _e = (call);                                                                                   \
        if (_e != cudaSuccess)                                                                                     \
            return ::sphx::cuda_fail(_e, #call, __FILE__, __LINE__);                                               \
    } while (0)

#define SPHX_LAUNCHED(ctx)                                                                                         \
    do                                                                                                             \
    {                                                                                                              \
        (ctx)->launches++;                                                                                         \
        cudaError_t _e = cudaGetLastError();                                                                       \
        if (_e != cudaSuccess)                                                                                     \
            return ::sphx::cuda_fail(_e, "kernel launch", __FILE__, __LINE__);                                     \
    } while (0)

#define SPHX_TRY(expr)                                                                                             \
    do                                                                                                             \
    {                                                                                                              \
        int _s = (expr);                                                                                           \
        if (_s != SPHX_OK)                                                                                         \
            return _s;                                                                                             \
    } while (0)

inline size_t dtype_size(sphx_dtype t) { return t == SPHX_F64 ? 8 : 4; }

struct Field
{
    sphx_dtype dtype = SPHX_F64;
    int ncomp = 1;
    void *dev = nullptr;
};

// Mesh as the kernels see it (Mesh, base_mesh.h / base_mesh.hxx).
struct MeshDev
{
    double lower[3];
    double gs;
    int all_cells[3];
    int grid_points[3];
};
MeshDev mesh_dev(const sphx_mesh_desc &m);

// Wendland C2 constants (kernel_wendland_c2.cpp:8-17, base_kernel.cpp:6-30).
struct WendlandC2
{
    double h, inv_h, rc, rc_sqr, factor_W, factor_dW;
    float prefilter_sqr; // FP32 rejection threshold, slightly above rc^2 / gs^2 scale
};
WendlandC2 wendland(int dim, double h);

// Kernel-launch helpers.
inline unsigned grid_for(size_t n, unsigned block) { return unsigned((n + block - 1) / block); }
} // namespace sphx

struct sphx_ctx_s
{
    int device = 0;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    uint64_t launches = 0;
    int num_sms = 0;
    // reduction slots (device) and their pinned host mirror
    unsigned long long *d_red = nullptr;
    unsigned long long *h_red = nullptr;
    // growable device scratch (scan partials, permutations)
    void *d_scratch = nullptr;
    size_t scratch_bytes = 0;
    int ensure_scratch(size_t bytes);
    // Bodies, cell lists and relations hold a reference: sphx_ctx_destroy only frees the
    // context once every object created on it has been destroyed, whatever the order.
    int refs = 1;
    void retain() { ++refs; }
};
namespace sphx
{
void release(sphx_ctx ctx);
}

struct sphx_body_s
{
    sphx_ctx ctx = nullptr;
    int dim = 3;
    size_t n = 0;
    std::map<std::string, sphx::Field> fields;
    sphx::Field *find(const char *name)
    {
        auto it = fields.find(name);
        return it == fields.end() ? nullptr : &it->second;
    }
    // Variable `name` with the given type/components, registering it when absent.
    int require(const char *name, sphx_dtype dtype, int ncomp, sphx::Field **out);
    // Variable that must already exist (with matching type).
    int need(const char *name, sphx_dtype dtype, int ncomp, sphx::Field **out);
};

struct sphx_cell_list_s
{
    sphx_ctx ctx = nullptr;
    sphx_mesh_desc mesh{};
    size_t ncells = 0;
    size_t capacity = 0; // particles
    size_t n = 0;        // particles in the last update
    uint32_t *cell_offset = nullptr;   // ncells + 1
    uint32_t *cell_count = nullptr;    // ncells
    uint32_t *particle_index = nullptr; // capacity
    uint32_t *cell_of = nullptr;       // capacity
    uint32_t *rank = nullptr;          // capacity
    double *sorted_pos = nullptr;      // dim x capacity, cell order (FP64)
    float *sorted_off = nullptr;       // dim x capacity, cell order, offset from the cell's lower corner
    int reserve(size_t n);
    // Periodic images (PeriodicConditionUsingCellLinkedList): with periodic axes the list
    // holds n_entries >= n entries, the particles and their images; particle_index,
    // sorted_pos and sorted_off then describe entries (stride n_entries).
    size_t n_entries = 0;
    int periodic_mask = 0;
    double per_lower[3] = {0, 0, 0}, per_upper[3] = {0, 0, 0}, per_cutoff = 0;
    size_t entry_cap = 0;
    double *entry_pos = nullptr; // dim x entry_cap (SoA), entries in generation order
    uint32_t *entry_idx = nullptr, *entry_flag = nullptr, *entry_scan = nullptr, *entry_perm = nullptr;
    int reserve_entries(size_t ne, size_t keep);
};

struct sphx_relation_s
{
    sphx_ctx ctx = nullptr;
    bool inner = true;
    sphx_body src = nullptr, tgt = nullptr;
    sphx_cell_list cl = nullptr;
    double h = 0;
    int depth = 1;
    double tgt_inv_rho0 = 1.0;
    bool store_W = false, store_r = false;
    int cap = 0;       // slots per source particle
    size_t n_src = 0;  // source particles the storage is sized for
    uint32_t *count = nullptr;
    uint32_t *j = nullptr;
    double *dW = nullptr, *W = nullptr, *r = nullptr, *e = nullptr;
    double *wsum = nullptr; // inner: W0 + sum W; contact: sum W inv_rho0 m_j
    int allocate(int cap, size_t n_src);
    void release();
};

namespace sphx
{
// Implemented in cell_list.cu; used by particle sorting.
int counting_sort_by_key(sphx_ctx ctx, const uint32_t *d_key, size_t n, uint32_t nkeys, uint32_t *d_offset,
                         uint32_t *d_count, uint32_t *d_rank, uint32_t *d_perm);
int exclusive_scan(sphx_ctx ctx, const uint32_t *d_in, uint32_t *d_out, size_t n);
// Scan with caller-owned scratch (scan_scratch_entries(n) uint32 entries); 3 launches, no
// allocation or synchronisation.
size_t scan_scratch_entries(size_t n);
int exclusive_scan_into(cudaStream_t s, const uint32_t *d_in, uint32_t *d_out, size_t n, uint32_t *tiles);
} // namespace sphx
