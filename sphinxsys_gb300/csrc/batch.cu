// Batched mixed-precision dam breaks (sphx_batch_*): many independent instances of one
// dimension advanced together.
//
// Each instance runs the Dambreak.cpp:166-220 loop with its own time steps: the advection
// dt, the density summation, its own number of acoustic sub-steps and the configuration
// update.  One launch per kernel and sub-step covers every instance: particles of all
// instances are concatenated in one cell-ordered array (each instance's cells occupy a
// disjoint range of one global cell index space, so one counting sort keeps every
// instance contiguous), a thread finds its instance by a binary search over the instance
// starts, and instances whose relaxation time has reached their advection dt skip the
// remaining sub-steps.  Per-instance time steps, relaxation times and sub-step counters live
// on the device; a one-block control kernel advances them after each sub-step.  The acoustic
// loop is either driven from the host (one flag read per sub-step) or captured once as a
// CUDA graph whose conditional WHILE node repeats the sub-step until no instance is active.
// A per-instance cap on sub-steps per advection step ends the loop with an error flag.
//
// The per-particle arithmetic is the single-case mixed solver's (mp_common.cuh), so an
// instance advances exactly as sphx_mp_* advances that case alone.
#include <algorithm>
#include <cmath>
#include <vector>

#include "mp_common.cuh"
#include "sphx_internal.cuh"

using namespace sphx;
using namespace sphx::mpc;

namespace
{
constexpr int kMaxSubsteps = 1 << 20; // default and largest cap of acoustic sub-steps per advection step

struct BInst
{
    MeshDev m;
    MPParams p;
    double gd[3];
    uint32_t cell_base, ncells;
    uint32_t p_start, p_count, w_start, w_count;
    double acoustic_cfl, advection_cfl, U_ref;
    double inv_gs; // 1 / sub-cell spacing
};

struct BRun
{
    double dt, Dt, relax, time;
    unsigned long long ac, adv;
    int active, substeps, iter, error;
};

__device__ __forceinline__ int find_instance(const uint32_t *starts, int count, uint32_t i)
{
    int lo = 0, hi = count - 1;
    while (lo < hi)
    {
        int mid = (lo + hi + 1) >> 1;
        if (starts[mid] <= i)
            lo = mid;
        else
            hi = mid - 1;
    }
    return lo;
}

// Per-instance max of one lane value: a warp reduction when the warp holds one instance,
// one atomic per active lane at instance boundaries.  Inactive instances are skipped.
__device__ __forceinline__ void instance_max(BRun *run, int b, bool lane_active, double v, bool adv)
{
    int b0 = __shfl_sync(0xffffffffu, b, 0);
    bool uniform = __all_sync(0xffffffffu, b == b0);
    if (uniform)
    {
        if (run[b0].active)
            warp_max_to(adv ? &run[b0].adv : &run[b0].ac, lane_active ? v : -1.0e300);
    }
    else if (lane_active)
        atomicMax(adv ? &run[b].adv : &run[b].ac, ordered_bits(v));
}

// ---------------------------------------------------------------- hashing and sorting
template <int D>
__device__ __forceinline__ void store_hash(const BInst &k, const int *c, uint32_t *ncell, size_t i, uint32_t *key,
                                           uint32_t *rank, uint32_t *cnt)
{
    ncell[i] = pack_cell<D>(c);
    uint32_t key_i = k.cell_base + linear_cell<D>(k.m, c);
    key[i] = key_i;
    rank[i] = atomicAdd(&cnt[key_i], 1u);
}

template <int D>
__device__ __forceinline__ void hash_position(const BInst &k, const double *x, uint32_t *ncell, float *noff, size_t n,
                                              size_t i, uint32_t *key, uint32_t *rank, uint32_t *cnt)
{
    int c[3] = {0, 0, 0};
    sub_cell_index<D>(k.m, k.inv_gs, x, c);
#pragma unroll
    for (int d = 0; d < D; ++d)
        stage_offset(noff, n, i, d, x[d] - cell_corner(k.m, d, c[d]));
    store_hash<D>(k, c, ncell, i, key, rank, cnt);
}

template <int D>
__global__ void k_b_from_fp64(size_t n, const double *__restrict__ pos, const uint32_t *__restrict__ starts,
                              int count, const BInst *__restrict__ inst, uint32_t *__restrict__ ncell,
                              float *__restrict__ noff, uint32_t *__restrict__ key, uint32_t *__restrict__ rank,
                              uint32_t *__restrict__ cnt)
{
    size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    const BInst &k = inst[find_instance(starts, count, uint32_t(i))];
    double x[3] = {0, 0, 0};
#pragma unroll
    for (int d = 0; d < D; ++d)
        x[d] = pos[d * n + i];
    hash_position<D>(k, x, ncell, noff, n, i, key, rank, cnt);
}

template <int D>
__global__ void k_b_rehash(size_t n, MPState f, const uint32_t *__restrict__ starts, int count,
                           const BInst *__restrict__ inst, uint32_t *__restrict__ ncell, float *__restrict__ noff,
                           uint32_t *__restrict__ key, uint32_t *__restrict__ rank, uint32_t *__restrict__ cnt)
{
    size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    const BInst &k = inst[find_instance(starts, count, uint32_t(i))];
    int c0[3];
    unpack_cell<D>(__float_as_uint(f.geo0[i].w), c0);
    int c[3] = {0, 0, 0};
    rehash_particle<D>(k.m, k.inv_gs, k.p.gs_f, false, f, n, i, c0, c, noff);
    store_hash<D>(k, c, ncell, i, key, rank, cnt);
}

__global__ void k_b_scatter(size_t n, const uint32_t *__restrict__ key, const uint32_t *__restrict__ rank,
                            const uint32_t *__restrict__ offset, uint32_t *__restrict__ perm)
{
    size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i < n)
        perm[offset[key[i]] + rank[i]] = uint32_t(i);
}

__global__ void k_b_sort_segments(size_t nseg, const uint32_t *__restrict__ offset, uint32_t *__restrict__ idx)
{
    size_t c = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (c < nseg)
        sort_segment(idx, offset[c], offset[c + 1]);
}

__global__ void k_b_set_total(uint32_t *offset, size_t ncells, uint32_t total) { offset[ncells] = total; }

template <int D>
__global__ void k_b_gather(size_t n, const uint32_t *__restrict__ perm, const uint32_t *__restrict__ ncell,
                           const float *__restrict__ noff, MPState src, MPState dst)
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
}

template <int D>
__global__ void k_b_wall_load(size_t nw, const uint32_t *__restrict__ perm, const double *__restrict__ pos,
                              const double *__restrict__ nrm, const uint32_t *__restrict__ wstarts, int count,
                              const BInst *__restrict__ inst, float4 *__restrict__ geo, float4 *__restrict__ n_out)
{
    size_t k = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (k >= nw)
        return;
    uint32_t i = perm[k];
    const BInst &b = inst[find_instance(wstarts, count, i)];
    double x[3] = {0, 0, 0};
#pragma unroll
    for (int d = 0; d < D; ++d)
        x[d] = pos[d * nw + i];
    int c[3] = {0, 0, 0};
    cell_index<D>(b.m, x, c);
    float o[3] = {0.f, 0.f, 0.f}, nn[3] = {0.f, 0.f, 0.f};
#pragma unroll
    for (int d = 0; d < D; ++d)
    {
        o[d] = float(x[d] - cell_corner(b.m, d, c[d]));
        nn[d] = float(nrm[d * nw + i]);
    }
    geo[k] = make_float4(o[0], o[1], o[2], __uint_as_float(pack_cell<D>(c)));
    n_out[k] = make_float4(nn[0], nn[1], nn[2], 0.f);
}

template <int D>
__global__ void k_b_wall_hash(size_t nw, const double *__restrict__ pos, const uint32_t *__restrict__ wstarts,
                              int count, const BInst *__restrict__ inst, uint32_t *__restrict__ key,
                              uint32_t *__restrict__ rank, uint32_t *__restrict__ cnt)
{
    size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= nw)
        return;
    const BInst &k = inst[find_instance(wstarts, count, uint32_t(i))];
    double x[3] = {0, 0, 0};
#pragma unroll
    for (int d = 0; d < D; ++d)
        x[d] = pos[d * nw + i];
    int c[3] = {0, 0, 0};
    cell_index<D>(k.m, x, c);
    uint32_t key_i = k.cell_base + linear_cell<D>(k.m, c);
    key[i] = key_i;
    rank[i] = atomicAdd(&cnt[key_i], 1u);
}

// ---------------------------------------------------------------- configuration + density sums
template <int D>
__global__ void k_b_build(size_t n, const uint32_t *__restrict__ starts, int count, const BInst *__restrict__ inst, MPState f,
              const uint32_t *__restrict__ f_offset, MPWallData w, const uint32_t *__restrict__ w_offset,
              MPNeighbors in, MPNeighbors wl, unsigned int *max_counts)
{
    size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    const BInst &k = inst[find_instance(starts, count, uint32_t(i))];
    build_particle<D>(i, n, k.p, Visit{k.m, k.cell_base, f_offset, w_offset}, f, w, in, wl, max_counts);
}

__global__ void k_b_density(size_t n, const float *__restrict__ drho_sum, float *__restrict__ drho)
{
    size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i < n)
        drho[i] = fmaxf(drho_sum[i], 0.0f);
}

// Start of an advection step, per instance: advection dt from the last 2nd-half maximum,
// the first acoustic dt from the last 1st-half maximum, both maxima reset.
__global__ void k_b_begin(int count, const BInst *__restrict__ inst, BRun *run)
{
    int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= count)
        return;
    const BInst &k = inst[b];
    BRun &r = run[b];
    double adv = from_ordered_bits(r.adv), ac = from_ordered_bits(r.ac);
    r.Dt = k.advection_cfl * k.p.h / (fmax(sqrt(adv), k.U_ref) + kTinyReal);
    r.dt = k.acoustic_cfl * k.p.h / (ac + kTinyReal);
    r.relax = 0.0;
    r.active = 1;
    r.substeps = 0;
    r.iter = 0;
    r.error = 0;
    r.ac = 0ull;
    r.adv = 0ull;
}

// ---------------------------------------------------------------- acoustic sub-step
__global__ void k_b_init1(size_t n, const uint32_t *__restrict__ starts, int count,
                          const BInst *__restrict__ inst, const BRun *__restrict__ run, float *__restrict__ drho,
                          const float *__restrict__ drho_dt, float4 *__restrict__ dyn, float *__restrict__ pres)
{
    size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    int b = find_instance(starts, count, uint32_t(i));
    if (!run[b].active)
        return;
    float r = drho[i] + drho_dt[i] * float(0.5 * run[b].dt);
    drho[i] = r;
    const float p = inst[b].p.p0_over_rho0 * r;
    reinterpret_cast<float *>(dyn)[4 * i + 3] = p;
    pres[i] = p;
}

// Blocks of 256 threads per SM the batch's 1st half is compiled to fit (4: 64 registers
// with spills; 3, at 80 registers without, measured 2 % slower).
#ifndef SPHX_BATCH_FIRST_MINB
#define SPHX_BATCH_FIRST_MINB 4
#endif
template <int D>
__global__ void __launch_bounds__(256, SPHX_BATCH_FIRST_MINB) k_b_first(size_t n, const uint32_t *__restrict__ starts, int count, const BInst *__restrict__ inst, BRun *run,
              MPState f, MPWallData w, MPNeighbors in, MPNeighbors wl)
{
    size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    int b = find_instance(starts, count, uint32_t(i < n ? i : n - 1));
    bool active = i < n && run[b].active;
    double vmax = -1.0e300;
    if (active)
    {
        const BInst &k = inst[b];
        vmax = first_particle<D, true>(i, n, k.p, Visit{k.m, k.cell_base, nullptr, nullptr}, run[b].dt, f, w, in,
                                       wl);
    }
    instance_max(run, b, active, vmax, false);
}

// held to 64 registers like the single-case 2nd half (its packed x / y arithmetic would
// otherwise take more, and fewer warps fit)
template <int D>
__global__ void __launch_bounds__(256, 4) k_b_second(size_t n, const uint32_t *__restrict__ starts, int count, const BInst *__restrict__ inst, BRun *run,
               MPState f, MPWallData w, MPNeighbors in, MPNeighbors wl)
{
    size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    int b = find_instance(starts, count, uint32_t(i < n ? i : n - 1));
    bool active = i < n && run[b].active;
    double amax = -1.0e300;
    if (active)
    {
        const BInst &k = inst[b];
        amax = second_particle<D, true>(i, n, k.p, Visit{k.m, k.cell_base, nullptr, nullptr}, run[b].dt, f, w, in,
                                        wl);
    }
    instance_max(run, b, active, amax, true);
}

// After each sub-step: per instance advance the relaxation time, take the next acoustic dt
// from the 1st-half maximum and decide whether another sub-step follows; sets the loop
// condition (graph) or the flag the host reads.
__global__ void k_b_control(int count, const BInst *__restrict__ inst, BRun *run, int *any_out,
                            const int *__restrict__ cap, cudaGraphConditionalHandle handle, int use_graph)
{
    const int max_substeps = *cap;
    __shared__ int any;
    if (threadIdx.x == 0)
        any = 0;
    __syncthreads();
    for (int b = threadIdx.x; b < count; b += blockDim.x)
    {
        BRun &r = run[b];
        if (!r.active)
            continue;
        const BInst &k = inst[b];
        r.relax += r.dt;
        r.time += r.dt;
        r.substeps += 1;
        r.iter += 1;
        bool more = r.relax < r.Dt;
        if (more && r.iter >= max_substeps) // needs another sub-step beyond the cap
        {
            more = false;
            r.error = 1;
        }
        if (more)
        {
            r.dt = k.acoustic_cfl * k.p.h / (from_ordered_bits(r.ac) + kTinyReal);
            r.ac = 0ull;
            r.adv = 0ull;
            atomicOr(&any, 1);
        }
        r.active = more ? 1 : 0;
    }
    __syncthreads();
    if (threadIdx.x == 0)
    {
        if (use_graph)
            cudaGraphSetConditional(handle, any ? 1u : 0u);
        else
            *any_out = any;
    }
}

// Initial maxima for the first time steps (all instances).
template <int D>
__global__ void k_b_initial_max(size_t n, const uint32_t *__restrict__ starts, int count,
                                const BInst *__restrict__ inst, BRun *run, MPState f)
{
    size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    int b = find_instance(starts, count, uint32_t(i));
    double vm, am;
    initial_max<D>(i, n, inst[b].p, inst[b].gd, f, &vm, &am);
    atomicMax(&run[b].ac, ordered_bits(vm));
    atomicMax(&run[b].adv, ordered_bits(am));
}

template <int D>
__global__ void k_b_download(size_t n, const uint32_t *__restrict__ starts, int count,
                             const BInst *__restrict__ inst, MPState f, double *__restrict__ out, size_t stride)
{
    // out rows (SoA, stride = total particles): pos (D), vel (D), rho, p; row index = the
    // instance's first particle + the particle's index in the instance's input order
    size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    int b = find_instance(starts, count, uint32_t(i));
    const BInst &k = inst[b];
    size_t o = size_t(k.p_start) + f.id[i];
    int c[3];
    unpack_cell<D>(__float_as_uint(f.geo0[i].w), c);
    float4 di = f.dyn[i];
    const float v[3] = {di.x, di.y, di.z};
#pragma unroll
    for (int d = 0; d < D; ++d)
    {
        out[d * stride + o] = cell_corner(k.m, d, c[d]) + offset_of(f, n, i, d);
        out[(D + d) * stride + o] = v[d];
    }
    out[(2 * D) * stride + o] = double(k.p.rho0) + double(f.drho[i]);
    out[(2 * D + 1) * stride + o] = di.w;
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

struct sphx_batch_s
{
    sphx_ctx ctx = nullptr;
    int dim = 3, count = 0;
    size_t n = 0, nw = 0, ncells = 0;
    std::vector<BInst> h_inst;
    BInst *inst = nullptr;
    BRun *run = nullptr;
    BRun *h_run = nullptr; // pinned mirror, refreshed after every advection step
    uint32_t *starts = nullptr, *wstarts = nullptr;
    // two state buffers: the configuration update gathers st[parity] into st[parity ^ 1]
    MPState st[2]{};
    int parity = 0;
    MPWallData w{};
    uint32_t *f_offset = nullptr, *w_offset = nullptr, *cnt = nullptr, *scan_tiles = nullptr;
    uint32_t *key = nullptr, *rank = nullptr, *perm = nullptr, *ncell = nullptr;
    float *noff = nullptr;
    MPNeighbors in{}, wl{};
    unsigned int *d_max = nullptr, *h_max = nullptr;
    int *d_any = nullptr, *h_any = nullptr;
    // cap of acoustic sub-steps per instance and advection step (device copy read by the
    // control kernel, so a captured graph sees a new value without being rebuilt)
    int *d_cap = nullptr;
    int max_substeps = kMaxSubsteps;
    int block = 128;
    // one executable graph per state parity: [density + step start] -> WHILE(sub-step) ->
    // [re-hash, sort, gather, neighbour lists, counter read-back]
    cudaStream_t capture = nullptr;
    cudaGraphExec_t graph_exec[2] = {nullptr, nullptr};
    uint64_t graph_launches = 0;
    std::vector<void *> owned;
    MPState &cur() { return st[parity]; }
    void invalidate_graphs()
    {
        for (int q = 0; q < 2; ++q)
            if (graph_exec[q])
            {
                cudaGraphExecDestroy(graph_exec[q]);
                graph_exec[q] = nullptr;
            }
    }
    template <typename T>
    T *alloc(size_t c)
    {
        T *p = dalloc<T>(c);
        if (p)
            owned.push_back(p);
        return p;
    }
};

namespace
{
// kernels enqueued by one configuration update (re-hash, 3-pass scan, total, scatter, segment
// sort, gather, build) and by the start of an advection step (density, step start)
constexpr uint64_t kConfigLaunches = 9, kBeginLaunches = 2, kSubstepLaunches = 4;

int b_alloc_state(sphx_batch bt, MPState &s)
{
    size_t n = bt->n, D = size_t(bt->dim);
    s.geo0 = bt->alloc<float4>(n);
    s.dyn = bt->alloc<float4>(n);
    s.off = bt->alloc<float>(D * n);
    s.off_lo = bt->alloc<float>(D * n);
    s.force = bt->alloc<float>(D * n);
    s.drho = bt->alloc<float>(n);
    s.drho_dt = bt->alloc<float>(n);
    s.drho_sum = bt->alloc<float>(n);
    s.pres = bt->alloc<float>(n);
    s.id = bt->alloc<uint32_t>(n);
    if (!s.geo0 || !s.dyn || !s.off || !s.off_lo || !s.force || !s.drho || !s.drho_dt || !s.drho_sum || !s.pres ||
        !s.id)
        return fail(SPHX_ERR_OUT_OF_MEMORY, "batch state allocation failed");
    return SPHX_OK;
}

int b_alloc_lists(sphx_batch bt, MPNeighbors &l, unsigned cap)
{
    if (l.J)
    {
        cudaFree(l.J);
        bt->owned.erase(std::remove(bt->owned.begin(), bt->owned.end(), (void *)l.J), bt->owned.end());
        l.J = nullptr;
    }
    l.J = bt->alloc<uint32_t>(size_t(cap) * std::max<size_t>(bt->n, 1));
    if (!l.J)
        return fail(SPHX_ERR_OUT_OF_MEMORY, "batch neighbour list allocation failed (%u slots)", cap);
    l.cap = cap;
    l.limit = uint32_t(&l == &bt->wl ? bt->nw : bt->n); // records the entries index
    bt->invalidate_graphs(); // the graphs hold the old list pointer
    return SPHX_OK;
}

// Offsets and cell-ordered permutation of n hashed particles (key/rank/cnt filled).
int b_enqueue_sort(sphx_batch bt, cudaStream_t s, size_t n, uint32_t *offset)
{
    SPHX_TRY(exclusive_scan_into(s, bt->cnt, offset, bt->ncells, bt->scan_tiles));
    k_b_set_total<<<1, 1, 0, s>>>(offset, bt->ncells, uint32_t(n));
    SPHX_CUDA(cudaGetLastError());
    if (n == 0)
        return SPHX_OK;
    k_b_scatter<<<grid_for(n, 256), 256, 0, s>>>(n, bt->key, bt->rank, offset, bt->perm);
    SPHX_CUDA(cudaGetLastError());
    k_b_sort_segments<<<grid_for(bt->ncells, 256), 256, 0, s>>>(bt->ncells, offset, bt->perm);
    SPHX_CUDA(cudaGetLastError());
    return SPHX_OK;
}

template <int D>
int b_enqueue_build(sphx_batch bt, cudaStream_t s, const MPState &dst)
{
    SPHX_CUDA(cudaMemsetAsync(bt->d_max, 0, 2 * sizeof(unsigned int), s));
    k_b_build<D><<<grid_for(bt->n, 256), 256, 0, s>>>(bt->n, bt->starts, bt->count, bt->inst, dst, bt->f_offset,
                                                     bt->w, bt->w_offset, bt->in, bt->wl, bt->d_max);
    SPHX_CUDA(cudaGetLastError());
    SPHX_CUDA(cudaMemcpyAsync(bt->h_max, bt->d_max, 2 * sizeof(unsigned int), cudaMemcpyDeviceToHost, s));
    return SPHX_OK;
}

// Configuration update from src into dst: re-hash (or the hash left by creation), sort,
// gather, neighbour lists and density sums.  Enqueues only.
template <int D>
int b_enqueue_configuration(sphx_batch bt, cudaStream_t s, const MPState &src, const MPState &dst, bool rehash)
{
    size_t n = bt->n;
    if (rehash)
    {
        SPHX_CUDA(cudaMemsetAsync(bt->cnt, 0, bt->ncells * sizeof(uint32_t), s));
        k_b_rehash<D><<<grid_for(n, 256), 256, 0, s>>>(n, src, bt->starts, bt->count, bt->inst,
                                                       bt->ncell, bt->noff, bt->key, bt->rank, bt->cnt);
        SPHX_CUDA(cudaGetLastError());
    }
    SPHX_TRY(b_enqueue_sort(bt, s, n, bt->f_offset));
    k_b_gather<D><<<grid_for(n, 256), 256, 0, s>>>(n, bt->perm, bt->ncell, bt->noff, src, dst);
    SPHX_CUDA(cudaGetLastError());
    return b_enqueue_build<D>(bt, s, dst);
}

// After a completed configuration update (h_max read back): grows the neighbour lists and
// rebuilds them when a particle had more neighbours than slots.
template <int D>
int b_check_lists(sphx_batch bt)
{
    cudaStream_t s = bt->ctx->stream;
    for (int attempt = 0; attempt < 3; ++attempt)
    {
        bool grow = false;
        if (bt->h_max[0] > bt->in.cap)
        {
            SPHX_TRY(b_alloc_lists(bt, bt->in, bt->h_max[0] + bt->h_max[0] / 4 + 4));
            grow = true;
        }
        if (bt->h_max[1] > bt->wl.cap)
        {
            SPHX_TRY(b_alloc_lists(bt, bt->wl, bt->h_max[1] + bt->h_max[1] / 4 + 4));
            grow = true;
        }
        if (!grow)
            return SPHX_OK;
        SPHX_TRY(b_enqueue_build<D>(bt, s, bt->cur()));
        bt->ctx->launches += 1;
        SPHX_CUDA(cudaStreamSynchronize(s));
    }
    return fail(SPHX_ERR_CAPACITY, "batch neighbour lists overflowed after growing");
}

template <int D>
int b_enqueue_begin(sphx_batch bt, cudaStream_t s, const MPState &cur)
{
    size_t n = bt->n;
    k_b_density<<<grid_for(n, 256), 256, 0, s>>>(n, cur.drho_sum, cur.drho);
    SPHX_CUDA(cudaGetLastError());
    k_b_begin<<<grid_for(size_t(bt->count), 64), 64, 0, s>>>(bt->count, bt->inst, bt->run);
    SPHX_CUDA(cudaGetLastError());
    return SPHX_OK;
}

template <int D>
int b_enqueue_substep(sphx_batch bt, cudaStream_t s, const MPState &cur, int use_graph,
                      cudaGraphConditionalHandle handle)
{
    size_t n = bt->n;
    unsigned blk = unsigned(bt->block);
    k_b_init1<<<grid_for(n, 256), 256, 0, s>>>(n, bt->starts, bt->count, bt->inst, bt->run, cur.drho, cur.drho_dt,
                                               cur.dyn, cur.pres);
    SPHX_CUDA(cudaGetLastError());
    k_b_first<D><<<grid_for(n, blk), blk, 0, s>>>(n, bt->starts, bt->count, bt->inst, bt->run, cur, bt->w, bt->in,
                                                  bt->wl);
    SPHX_CUDA(cudaGetLastError());
    k_b_second<D><<<grid_for(n, blk), blk, 0, s>>>(n, bt->starts, bt->count, bt->inst, bt->run, cur, bt->w, bt->in,
                                                   bt->wl);
    SPHX_CUDA(cudaGetLastError());
    k_b_control<<<1, 256, 0, s>>>(bt->count, bt->inst, bt->run, bt->d_any, bt->d_cap, handle, use_graph);
    SPHX_CUDA(cudaGetLastError());
    return SPHX_OK;
}

template <class F>
int capture_into(cudaStream_t s, cudaGraph_t *out, F &&enqueue)
{
    SPHX_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    int st = enqueue();
    cudaError_t e = cudaStreamEndCapture(s, out);
    SPHX_TRY(st);
    SPHX_CUDA(e);
    return SPHX_OK;
}

// Builds the executable graph of one advection step for state parity q.
template <int D>
int b_build_graph(sphx_batch bt, int q)
{
    const MPState src = bt->st[q], dst = bt->st[q ^ 1];
    cudaStream_t s = bt->capture;
    cudaGraph_t g = nullptr, pre = nullptr, post = nullptr;
    auto done = [&](int code) {
        if (pre)
            cudaGraphDestroy(pre);
        if (post)
            cudaGraphDestroy(post);
        if (g)
            cudaGraphDestroy(g);
        return code;
    };
    int st = capture_into(s, &pre, [&] { return b_enqueue_begin<D>(bt, s, src); });
    if (st == SPHX_OK)
        st = capture_into(s, &post, [&] {
            SPHX_TRY(b_enqueue_configuration<D>(bt, s, src, dst, true));
            SPHX_CUDA(cudaMemcpyAsync(bt->h_run, bt->run, size_t(bt->count) * sizeof(BRun), cudaMemcpyDeviceToHost, s));
            return int(SPHX_OK);
        });
    if (st != SPHX_OK)
        return done(st);
    cudaGraphConditionalHandle handle = 0;
    cudaGraphNode_t n_pre, n_loop, n_post;
    cudaGraphNodeParams params = {};
    if (cudaGraphCreate(&g, 0) != cudaSuccess ||
        // the loop condition is 1 at every launch: each instance takes at least one sub-step
        cudaGraphConditionalHandleCreate(&handle, g, 1, cudaGraphCondAssignDefault) != cudaSuccess ||
        cudaGraphAddChildGraphNode(&n_pre, g, nullptr, 0, pre) != cudaSuccess)
        return done(fail(SPHX_ERR_CUDA, "batch graph assembly failed: %s", cudaGetErrorString(cudaGetLastError())));
    params.type = cudaGraphNodeTypeConditional;
    params.conditional.handle = handle;
    params.conditional.type = cudaGraphCondTypeWhile;
    params.conditional.size = 1;
    if (cudaGraphAddNode(&n_loop, g, &n_pre, nullptr, 1, &params) != cudaSuccess)
        return done(fail(SPHX_ERR_CUDA, "batch graph: conditional node: %s", cudaGetErrorString(cudaGetLastError())));
    cudaGraph_t body = params.conditional.phGraph_out[0];
    SPHX_CUDA(cudaStreamBeginCaptureToGraph(s, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
    st = b_enqueue_substep<D>(bt, s, src, 1, handle);
    cudaGraph_t captured = nullptr;
    cudaError_t e = cudaStreamEndCapture(s, &captured);
    if (st != SPHX_OK)
        return done(st);
    if (e != cudaSuccess)
        return done(fail(SPHX_ERR_CUDA, "batch graph: loop body capture: %s", cudaGetErrorString(e)));
    if (cudaGraphAddChildGraphNode(&n_post, g, &n_loop, 1, post) != cudaSuccess)
        return done(fail(SPHX_ERR_CUDA, "batch graph: configuration node: %s", cudaGetErrorString(cudaGetLastError())));
    e = cudaGraphInstantiate(&bt->graph_exec[q], g, 0);
    if (e != cudaSuccess)
    {
        bt->graph_exec[q] = nullptr;
        return done(fail(SPHX_ERR_CUDA, "batch graph instantiation: %s", cudaGetErrorString(e)));
    }
    return done(SPHX_OK);
}

template <int D>
int b_advection_step(sphx_batch bt, int use_graph)
{
    sphx_ctx ctx = bt->ctx;
    cudaStream_t s = ctx->stream;
    const int q = bt->parity;
    const MPState src = bt->st[q], dst = bt->st[q ^ 1];
    uint64_t loops = 0;
    if (use_graph)
    {
        if (!bt->graph_exec[q])
            SPHX_TRY(b_build_graph<D>(bt, q));
        SPHX_CUDA(cudaGraphLaunch(bt->graph_exec[q], s));
        ++bt->graph_launches;
        SPHX_CUDA(cudaStreamSynchronize(s));
        for (int b = 0; b < bt->count; ++b)
            loops = std::max<uint64_t>(loops, uint64_t(bt->h_run[b].iter));
    }
    else
    {
        SPHX_TRY(b_enqueue_begin<D>(bt, s, src));
        for (int it = 0; it <= bt->max_substeps; ++it)
        {
            SPHX_TRY(b_enqueue_substep<D>(bt, s, src, 0, 0));
            ++loops;
            SPHX_CUDA(cudaMemcpyAsync(bt->h_any, bt->d_any, sizeof(int), cudaMemcpyDeviceToHost, s));
            SPHX_CUDA(cudaStreamSynchronize(s));
            if (!*bt->h_any)
                break;
        }
        SPHX_TRY(b_enqueue_configuration<D>(bt, s, src, dst, true));
        SPHX_CUDA(cudaMemcpyAsync(bt->h_run, bt->run, size_t(bt->count) * sizeof(BRun), cudaMemcpyDeviceToHost, s));
        SPHX_CUDA(cudaStreamSynchronize(s));
    }
    ctx->launches += kBeginLaunches + kSubstepLaunches * loops + kConfigLaunches;
    bt->parity ^= 1;
    for (int b = 0; b < bt->count; ++b)
        if (bt->h_run[b].error)
            return fail(SPHX_ERR_TIMEOUT, "instance %d reached the cap of %d acoustic sub-steps in one advection step",
                        b, bt->max_substeps);
    return b_check_lists<D>(bt);
}

template <int D>
int b_setup(sphx_batch bt, const double *d_fpos, const double *d_wpos, const double *d_wnrm)
{
    sphx_ctx ctx = bt->ctx;
    cudaStream_t s = ctx->stream;
    size_t n = bt->n, nw = bt->nw;
    // walls: sorted once into their cells
    SPHX_CUDA(cudaMemsetAsync(bt->cnt, 0, bt->ncells * sizeof(uint32_t), s));
    if (nw > 0)
    {
        k_b_wall_hash<D><<<grid_for(nw, 256), 256, 0, s>>>(nw, d_wpos, bt->wstarts, bt->count, bt->inst, bt->key,
                                                           bt->rank, bt->cnt);
        SPHX_LAUNCHED(ctx);
    }
    SPHX_TRY(b_enqueue_sort(bt, s, nw, bt->w_offset));
    ctx->launches += nw > 0 ? 6 : 4;
    if (nw > 0)
    {
        k_b_wall_load<D><<<grid_for(nw, 256), 256, 0, s>>>(nw, bt->perm, d_wpos, d_wnrm, bt->wstarts, bt->count,
                                                           bt->inst, bt->w.geo, bt->w.n);
        SPHX_LAUNCHED(ctx);
    }
    // fluid: hashed from the FP64 positions, then ordered with lists and density sums
    SPHX_CUDA(cudaMemsetAsync(bt->cnt, 0, bt->ncells * sizeof(uint32_t), s));
    k_b_from_fp64<D><<<grid_for(n, 256), 256, 0, s>>>(n, d_fpos, bt->starts, bt->count, bt->inst, bt->ncell,
                                                      bt->noff, bt->key, bt->rank, bt->cnt);
    SPHX_LAUNCHED(ctx);
    SPHX_TRY(b_enqueue_configuration<D>(bt, s, bt->st[0], bt->st[1], false));
    ctx->launches += kConfigLaunches - 1;
    SPHX_CUDA(cudaStreamSynchronize(s));
    bt->parity = 1;
    SPHX_TRY(b_check_lists<D>(bt));
    k_b_initial_max<D><<<grid_for(n, 256), 256, 0, s>>>(n, bt->starts, bt->count, bt->inst, bt->run, bt->cur());
    SPHX_LAUNCHED(ctx);
    SPHX_CUDA(cudaStreamSynchronize(s));
    return SPHX_OK;
}
} // namespace

extern "C" int sphx_batch_create(sphx_ctx ctx, int dim, int count, const sphx_batch_instance *desc,
                                 sphx_batch *out)
{
    if (!ctx || !desc || !out || (dim != 2 && dim != 3) || count < 1 || count > 4096)
        return fail(SPHX_ERR_INVALID_ARG, "invalid batch arguments (dim 2 or 3, 1..4096 instances)");
    *out = nullptr;
    sphx_batch bt = new sphx_batch_s();
    bt->ctx = ctx;
    ctx->retain();
    bt->dim = dim;
    bt->count = count;
    auto bail = [&](int code) {
        sphx_batch_destroy(bt);
        return code;
    };
    const int D = dim;
    size_t n = 0, nw = 0, nc = 0;
    std::vector<uint32_t> starts(count + 1), wstarts(count + 1);
    bt->h_inst.resize(count);
    for (int q = 0; q < count; ++q)
    {
        const sphx_batch_instance &d = desc[q];
        if (d.mesh.dim != dim || d.n_fluid < 1 || !d.fluid_pos || (d.n_wall && (!d.wall_pos || !d.wall_normal)) ||
            !(d.h > 0) || !(d.fluid_mass > 0) || !(d.fluid_vol > 0) || !(d.sigma0 > 0) || !(d.rho0 > 0) ||
            !(d.c0 > 0) || !(d.wall_rho0 > 0) || (d.n_wall && !(d.wall_vol > 0)))
            return bail(fail(SPHX_ERR_INVALID_ARG, "instance %d: invalid description", q));
        if (std::abs(d.mesh.grid_spacing - 2.0 * d.h) > 1e-12 * d.mesh.grid_spacing)
            return bail(fail(SPHX_ERR_INVALID_ARG, "instance %d: grid spacing must equal the cut-off radius 2h", q));
        const sphx_mesh_desc mesh = sub_mesh(d.mesh);
        size_t cells = 1;
        for (int a = 0; a < D; ++a)
        {
            int lim = D == 2 ? CellLanes<2>::max_cells : CellLanes<3>::max_cells;
            if (mesh.all_cells[a] < 1 || mesh.all_cells[a] > lim)
                return bail(fail(SPHX_ERR_INVALID_ARG, "instance %d: %d cells on axis %d (at most %d)", q,
                                 mesh.all_cells[a], a, lim));
            cells *= size_t(mesh.all_cells[a]);
        }
        BInst &k = bt->h_inst[q];
        k = BInst{};
        k.m = mesh_dev(mesh);
        k.inv_gs = 1.0 / mesh.grid_spacing;
        k.cell_base = uint32_t(nc);
        k.ncells = uint32_t(cells);
        k.p_start = uint32_t(n);
        k.p_count = uint32_t(d.n_fluid);
        k.w_start = uint32_t(nw);
        k.w_count = uint32_t(d.n_wall);
        for (int a = 0; a < 3; ++a)
            k.gd[a] = a < D ? d.gravity[a] : 0.0;
        k.p = make_params(D, mesh.grid_spacing, d.h, d.rho0, d.c0, d.fluid_vol, d.fluid_mass, d.sigma0,
                          1.0 / d.wall_rho0 * d.wall_mass, d.wall_vol, 3.0, k.gd);
        k.acoustic_cfl = 0.6;
        k.advection_cfl = 0.25;
        k.U_ref = d.U_ref;
        starts[q] = uint32_t(n);
        wstarts[q] = uint32_t(nw);
        n += d.n_fluid;
        nw += d.n_wall;
        nc += cells;
        if (n >= 0xffffffffull || nw >= 0xffffffffull || nc >= 0xffffffffull)
            return bail(fail(SPHX_ERR_INVALID_ARG, "batch exceeds 32-bit particle or cell indices"));
    }
    starts[count] = uint32_t(n);
    wstarts[count] = uint32_t(nw);
    bt->n = n;
    bt->nw = nw;
    bt->ncells = nc;
    // device allocations
    bt->inst = bt->alloc<BInst>(count);
    bt->run = bt->alloc<BRun>(count);
    bt->starts = bt->alloc<uint32_t>(count + 1);
    bt->wstarts = bt->alloc<uint32_t>(count + 1);
    bt->f_offset = bt->alloc<uint32_t>(nc + 1);
    bt->w_offset = bt->alloc<uint32_t>(nc + 1);
    bt->cnt = bt->alloc<uint32_t>(nc);
    bt->scan_tiles = bt->alloc<uint32_t>(scan_scratch_entries(nc));
    size_t big = std::max(n, nw);
    bt->key = bt->alloc<uint32_t>(big);
    bt->rank = bt->alloc<uint32_t>(big);
    bt->perm = bt->alloc<uint32_t>(big);
    bt->ncell = bt->alloc<uint32_t>(n);
    bt->noff = bt->alloc<float>(6 * n);
    bt->w.geo = bt->alloc<float4>(nw);
    bt->w.n = bt->alloc<float4>(nw);
    bt->in.count = bt->alloc<uint32_t>(n);
    bt->wl.count = bt->alloc<uint32_t>(n);
    bt->d_max = bt->alloc<unsigned int>(2);
    bt->d_any = bt->alloc<int>(1);
    bt->d_cap = bt->alloc<int>(1);
    int st;
    if (!bt->inst || !bt->run || !bt->starts || !bt->wstarts || !bt->f_offset || !bt->w_offset || !bt->cnt ||
        !bt->scan_tiles || !bt->key || !bt->rank || !bt->perm || !bt->ncell || !bt->noff || !bt->w.geo || !bt->w.n ||
        !bt->in.count || !bt->wl.count || !bt->d_max || !bt->d_any || !bt->d_cap)
        return bail(fail(SPHX_ERR_OUT_OF_MEMORY, "batch allocation failed"));
    if ((st = b_alloc_state(bt, bt->st[0])) != SPHX_OK || (st = b_alloc_state(bt, bt->st[1])) != SPHX_OK)
        return bail(st);
    if (cudaMallocHost(&bt->h_max, 2 * sizeof(unsigned int)) != cudaSuccess ||
        cudaMallocHost(&bt->h_any, sizeof(int)) != cudaSuccess ||
        cudaMallocHost(&bt->h_run, size_t(count) * sizeof(BRun)) != cudaSuccess)
        return bail(fail(SPHX_ERR_OUT_OF_MEMORY, "pinned allocation failed"));
    if (cudaStreamCreateWithFlags(&bt->capture, cudaStreamNonBlocking) != cudaSuccess)
        return bail(fail(SPHX_ERR_CUDA, "capture stream creation failed"));
    if ((st = b_alloc_lists(bt, bt->in, D == 2 ? 24 : 96)) != SPHX_OK ||
        (st = b_alloc_lists(bt, bt->wl, D == 2 ? 16 : 64)) != SPHX_OK)
        return bail(st);
    for (int q = 0; q < count; ++q)
        bt->h_run[q] = BRun{};
    if (cudaMemcpy(bt->d_cap, &bt->max_substeps, sizeof(int), cudaMemcpyHostToDevice) != cudaSuccess)
        return bail(fail(SPHX_ERR_CUDA, "sub-step cap upload failed"));
    // host staging: FP64 SoA of fluid positions, wall positions and normals
    std::vector<double> fpos(size_t(D) * n), wpos(size_t(D) * nw), wnrm(size_t(D) * nw);
    std::vector<uint32_t> ids(n);
    for (int q = 0; q < count; ++q)
    {
        const sphx_batch_instance &d = desc[q];
        for (size_t i = 0; i < d.n_fluid; ++i)
        {
            ids[starts[q] + i] = uint32_t(i);
            for (int a = 0; a < D; ++a)
                fpos[size_t(a) * n + starts[q] + i] = d.fluid_pos[i * D + a];
        }
        for (size_t i = 0; i < d.n_wall; ++i)
            for (int a = 0; a < D; ++a)
            {
                wpos[size_t(a) * nw + wstarts[q] + i] = d.wall_pos[i * D + a];
                wnrm[size_t(a) * nw + wstarts[q] + i] = d.wall_normal[i * D + a];
            }
    }
    double *d_fpos = nullptr, *d_wpos = nullptr, *d_wnrm = nullptr;
    auto cleanup = [&]() {
        cudaFree(d_fpos);
        cudaFree(d_wpos);
        cudaFree(d_wnrm);
    };
    if (cudaMalloc(&d_fpos, std::max<size_t>(fpos.size(), 1) * 8) != cudaSuccess ||
        cudaMalloc(&d_wpos, std::max<size_t>(wpos.size(), 1) * 8) != cudaSuccess ||
        cudaMalloc(&d_wnrm, std::max<size_t>(wnrm.size(), 1) * 8) != cudaSuccess)
    {
        cleanup();
        return bail(fail(SPHX_ERR_OUT_OF_MEMORY, "staging allocation failed"));
    }
    cudaStream_t s = ctx->stream;
    const MPState &a0 = bt->st[0];
    bool ok =
        cudaMemcpy(d_fpos, fpos.data(), fpos.size() * 8, cudaMemcpyHostToDevice) == cudaSuccess &&
        (wpos.empty() || cudaMemcpy(d_wpos, wpos.data(), wpos.size() * 8, cudaMemcpyHostToDevice) == cudaSuccess) &&
        (wnrm.empty() || cudaMemcpy(d_wnrm, wnrm.data(), wnrm.size() * 8, cudaMemcpyHostToDevice) == cudaSuccess) &&
        cudaMemcpy(bt->inst, bt->h_inst.data(), count * sizeof(BInst), cudaMemcpyHostToDevice) == cudaSuccess &&
        cudaMemcpy(bt->run, bt->h_run, count * sizeof(BRun), cudaMemcpyHostToDevice) == cudaSuccess &&
        cudaMemcpy(bt->starts, starts.data(), starts.size() * 4, cudaMemcpyHostToDevice) == cudaSuccess &&
        cudaMemcpy(bt->wstarts, wstarts.data(), wstarts.size() * 4, cudaMemcpyHostToDevice) == cudaSuccess &&
        cudaMemcpy(a0.id, ids.data(), n * 4, cudaMemcpyHostToDevice) == cudaSuccess &&
        // fluid at rest with rho = rho0 and no pressure force yet
        cudaMemset(a0.dyn, 0, n * sizeof(float4)) == cudaSuccess &&
        cudaMemset(a0.force, 0, size_t(D) * n * 4) == cudaSuccess &&
        cudaMemset(a0.drho, 0, n * 4) == cudaSuccess && cudaMemset(a0.drho_dt, 0, n * 4) == cudaSuccess;
    if (!ok)
    {
        cleanup();
        return bail(fail(SPHX_ERR_CUDA, "batch upload failed"));
    }
    st = D == 2 ? b_setup<2>(bt, d_fpos, d_wpos, d_wnrm) : b_setup<3>(bt, d_fpos, d_wpos, d_wnrm);
    cudaStreamSynchronize(s);
    cleanup();
    if (st != SPHX_OK)
        return bail(st);
    *out = bt;
    return SPHX_OK;
}

extern "C" int sphx_batch_destroy(sphx_batch bt)
{
    if (!bt)
        return SPHX_OK;
    sphx_ctx ctx = bt->ctx;
    cudaStreamSynchronize(ctx->stream);
    bt->invalidate_graphs();
    if (bt->capture)
        cudaStreamDestroy(bt->capture);
    for (void *p : bt->owned)
        cudaFree(p);
    if (bt->h_max)
        cudaFreeHost(bt->h_max);
    if (bt->h_any)
        cudaFreeHost(bt->h_any);
    if (bt->h_run)
        cudaFreeHost(bt->h_run);
    delete bt;
    release(ctx);
    return SPHX_OK;
}

extern "C" int sphx_batch_advection_step(sphx_batch bt, int use_graph, int *substeps, double *physical_time)
{
    if (!bt)
        return fail(SPHX_ERR_INVALID_ARG, "null batch");
    SPHX_TRY(bt->dim == 2 ? b_advection_step<2>(bt, use_graph) : b_advection_step<3>(bt, use_graph));
    for (int q = 0; q < bt->count; ++q)
    {
        if (substeps)
            substeps[q] = bt->h_run[q].substeps;
        if (physical_time)
            physical_time[q] = bt->h_run[q].time;
    }
    return SPHX_OK;
}

extern "C" int sphx_batch_set_tuning(sphx_batch bt, int block)
{
    if (!bt || block < 64 || block > 256 || block % 32 != 0)
        return fail(SPHX_ERR_INVALID_ARG, "block must be 64..256 in steps of 32");
    bt->block = block;
    bt->invalidate_graphs();
    return SPHX_OK;
}

extern "C" int sphx_batch_set_substep_cap(sphx_batch bt, int max_substeps)
{
    if (!bt || max_substeps < 1 || max_substeps > kMaxSubsteps)
        return fail(SPHX_ERR_INVALID_ARG, "the sub-step cap must lie in 1..%d", kMaxSubsteps);
    // ordered on the stream after every step already enqueued
    SPHX_CUDA(cudaMemcpyAsync(bt->d_cap, &max_substeps, sizeof(int), cudaMemcpyHostToDevice, bt->ctx->stream));
    SPHX_CUDA(cudaStreamSynchronize(bt->ctx->stream));
    bt->max_substeps = max_substeps;
    return SPHX_OK;
}

extern "C" int sphx_batch_graph_launches(sphx_batch bt, uint64_t *out)
{
    if (!bt || !out)
        return fail(SPHX_ERR_INVALID_ARG, "null argument");
    *out = bt->graph_launches;
    return SPHX_OK;
}

extern "C" int sphx_batch_download(sphx_batch bt, int instance, double *pos, double *vel, double *rho, double *p)
{
    if (!bt || instance < 0 || instance >= bt->count)
        return fail(SPHX_ERR_INVALID_ARG, "invalid instance");
    const int D = bt->dim;
    size_t n = bt->n;
    size_t rows = size_t(2 * D + 2);
    sphx_ctx ctx = bt->ctx;
    SPHX_TRY(ctx->ensure_scratch(rows * n * sizeof(double)));
    double *out = static_cast<double *>(ctx->d_scratch);
    if (D == 2)
        k_b_download<2><<<grid_for(n, 256), 256, 0, ctx->stream>>>(n, bt->starts, bt->count, bt->inst, bt->cur(),
                                                                    out, n);
    else
        k_b_download<3><<<grid_for(n, 256), 256, 0, ctx->stream>>>(n, bt->starts, bt->count, bt->inst, bt->cur(),
                                                                    out, n);
    SPHX_LAUNCHED(ctx);
    const BInst &k = bt->h_inst[instance];
    size_t cnt = k.p_count;
    std::vector<double> h(rows * cnt);
    for (size_t r = 0; r < rows; ++r)
        SPHX_CUDA(cudaMemcpyAsync(h.data() + r * cnt, out + r * n + k.p_start, cnt * sizeof(double),
                                  cudaMemcpyDeviceToHost, ctx->stream));
    SPHX_CUDA(cudaStreamSynchronize(ctx->stream));
    for (size_t i = 0; i < cnt; ++i)
    {
        for (int d = 0; d < D; ++d)
        {
            if (pos)
                pos[i * D + d] = h[size_t(d) * cnt + i];
            if (vel)
                vel[i * D + d] = h[size_t(D + d) * cnt + i];
        }
        if (rho)
            rho[i] = h[size_t(2 * D) * cnt + i];
        if (p)
            p[i] = h[size_t(2 * D + 1) * cnt + i];
    }
    return SPHX_OK;
}

extern "C" int sphx_batch_size(sphx_batch bt, size_t *fluid_particles, size_t *wall_particles)
{
    if (!bt)
        return fail(SPHX_ERR_INVALID_ARG, "null batch");
    if (fluid_particles)
        *fluid_particles = bt->n;
    if (wall_particles)
        *wall_particles = bt->nw;
    return SPHX_OK;
}
