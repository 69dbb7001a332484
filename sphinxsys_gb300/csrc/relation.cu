// Neighbour relations (configuration update) with the Wendland C2 kernel.
//
// Reference: InnerRelation::updateConfiguration (src/shared/body_relations/
// inner_body_relation.cpp:14-20) and ContactRelation::updateConfiguration
// (contact_body_relation.cpp:22-32) -> BaseCellLinkedList::searchNeighborsByMesh
// (src/shared/meshes/cell_linked_list.hpp:20-46) -> NeighborBuilderInner / Contact
// (src/shared/particle_neighborhood/neighborhood.cpp:26-46,85-98,144-160) with
// KernelWendlandC2 (src/shared/kernels/kernel_wendland_c2.cpp:8-45, base_kernel.cpp:6-76).
//
// Storage is ELL, slot-major: entry s of source particle i sits at s * n_src + i, so a
// warp of consecutive particles reads slot s of all its lanes in one coalesced access.
// Per entry: neighbour index j, dW_ij, e_ij (dim components), and r_ij / W_ij when the
// relation needs them.  Inner relations also keep sigma_i = W0 + sum_j W_ij and contact
// relations sum_j W_ij m_j / rho0_j, the two sums DensitySummation needs
// (density_summation.cpp:74-82,113-122).
//
// Membership test: |x_i - x_j|^2 < (2h)^2 in FP64 with the canonical association
// ((dx*dx + dy*dy) + dz*dz) and no fused multiply-add, so the pair set equals the
// oracle's bit for bit.  An FP32 test on cell-relative offsets first rejects candidates
// clearly outside the cut-off.
#include <algorithm>

#include "sphx_device.cuh"
#include "sphx_internal.cuh"

using namespace sphx;

namespace
{
constexpr unsigned kBlock = 128;

struct BuildArgs
{
    size_t n_src, n_tgt;
    const double *src_pos;       // SoA, stride n_src
    const uint32_t *cell_offset; // target cell list
    const uint32_t *pidx;
    const double *spos; // target positions in cell order, SoA stride n_tgt
    const float *soff;  // FP32 offsets from each cell corner, SoA stride n_tgt
    MeshDev m;
    WendlandC2 k;
    int depth, cap;
    uint32_t *count, *J;
    double *DW, *E, *R, *W; // E: dim arrays of cap * n_src
    double *wsum;
    const double *tgt_mass;
    double tgt_inv_rho0;
    unsigned int *max_count;
};

// Two passes per source particle.  Pass 1 walks the candidate cells with the FP32
// pre-filter only and writes the cell-list entry index of every candidate that passes
// into the particle's list slots.  Pass 2 walks that short list: the exact FP64 membership
// test, then W, dW, e (and r) in FP64 for the accepted pairs, compacted in place.  The FP64
// work of pass 2 runs with nearly all lanes of a warp busy; in one pass it ran for the
// whole warp whenever any lane accepted a candidate.  Entries, order and values are those
// of the one-pass form.  The capacity check uses the pass-1 count (a superset).
template <int D, bool INNER>
__global__ void __launch_bounds__(kBlock) k_build(BuildArgs a)
{
    size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= a.n_src)
        return;
    double xi[3] = {0, 0, 0};
#pragma unroll
    for (int d = 0; d < D; ++d)
        xi[d] = a.src_pos[d * a.n_src + i];
    int c[3] = {0, 0, 0}, lo[3] = {0, 0, 0}, hi[3] = {1, 1, 1};
    cell_index<D>(a.m, xi, c);
#pragma unroll
    for (int d = 0; d < D; ++d)
    {
        lo[d] = max(0, c[d] - a.depth);
        hi[d] = min(a.m.all_cells[d], c[d] + a.depth + 1);
    }
    const size_t stride = size_t(a.cap) * a.n_src;
    // pass 1: FP32 pre-filter, candidate entries into the list slots
    unsigned cand = 0;
    int cc[3] = {0, 0, 0};
    for (cc[0] = lo[0]; cc[0] < hi[0]; ++cc[0])
    {
        float o0 = float(xi[0] - cell_corner(a.m, 0, cc[0]));
        for (cc[1] = lo[1]; cc[1] < hi[1]; ++cc[1])
        {
            float o1 = float(xi[1] - cell_corner(a.m, 1, cc[1]));
            for (cc[2] = lo[2]; cc[2] < hi[2]; ++cc[2])
            {
                float o2 = D == 3 ? float(xi[2] - cell_corner(a.m, 2, cc[2])) : 0.0f;
                uint32_t lc = linear_cell<D>(a.m, cc);
                uint32_t kb = a.cell_offset[lc], ke = a.cell_offset[lc + 1];
                if (!SPHX_CHECKED(kb <= ke && ke <= a.n_tgt, kCheckCellRange, (uint64_t(kb) << 32) | ke))
                    ke = kb;
                for (uint32_t kk = kb; kk < ke; ++kk)
                {
                    float f0 = o0 - a.soff[kk], f1 = o1 - a.soff[a.n_tgt + kk];
                    float d2f = f0 * f0 + f1 * f1;
                    if (D == 3)
                    {
                        float f2 = o2 - a.soff[2 * a.n_tgt + kk];
                        d2f += f2 * f2;
                    }
                    if (d2f > a.k.prefilter_sqr)
                        continue;
                    if (INNER && a.pidx[kk] == uint32_t(i))
                        continue;
                    if (cand < unsigned(a.cap))
                        a.J[size_t(cand) * a.n_src + i] = kk;
                    ++cand;
                }
                if (D == 2)
                    break;
            }
        }
    }
    // pass 2: exact test and kernel values over the candidates, in place
    const unsigned stored = min(cand, unsigned(a.cap));
    unsigned cnt = 0;
    double ws = INNER ? a.k.factor_W : 0.0;
    for (unsigned s = 0; s < stored; ++s)
    {
        const uint32_t kk = a.J[size_t(s) * a.n_src + i];
        if (!SPHX_CHECKED(kk < a.n_tgt && a.pidx[kk] < a.n_tgt, kCheckListEntry, kk))
            continue;
        double dx[3] = {0, 0, 0};
#pragma unroll
        for (int d = 0; d < D; ++d)
            dx[d] = __dsub_rn(xi[d], a.spos[d * a.n_tgt + kk]);
        double r2 = __dadd_rn(__dmul_rn(dx[0], dx[0]), __dmul_rn(dx[1], dx[1]));
        if (D == 3)
            r2 = __dadd_rn(r2, __dmul_rn(dx[2], dx[2]));
        if (!(r2 < a.k.rc_sqr))
            continue;
        const uint32_t j = a.pidx[kk];
        // one reciprocal square root gives r and 1/r; e = dx / (r + TinyReal) of the
        // reference differs from dx / r by TinyReal / r relative, far below one rounding,
        // except for coincident particles where e is zero
        double ri = rsqrt(r2);
        double r = r2 > 0.0 ? r2 * ri : 0.0;
        double inv = r2 > 0.0 ? ri : 1.0 / kTinyReal;
        double q = r * a.k.inv_h;
        // Wendland C2 with t = 1 - q/2: W ~ t^4 (1 + 2q), dW ~ 0.625 (q - 2)^3 q = -5 t^3 q
        double t = 1.0 - 0.5 * q;
        double t2 = t * t, t3 = t2 * t;
        double W = a.k.factor_W * (t2 * t2 * (1.0 + 2.0 * q));
        double dW = a.k.factor_dW * (-5.0 * t3 * q);
        size_t slot = size_t(cnt) * a.n_src + i;
        a.J[slot] = j;
        a.DW[slot] = dW;
#pragma unroll
        for (int d = 0; d < D; ++d)
            a.E[d * stride + slot] = dx[d] * inv;
        if (a.R)
            a.R[slot] = r;
        if (a.W)
            a.W[slot] = W;
        if (INNER)
            ws += W;
        else
            ws += (W * a.tgt_inv_rho0) * a.tgt_mass[j];
        ++cnt;
    }
    a.count[i] = cnt;
    a.wsum[i] = ws;
    warp_atomic_max(a.max_count, cand);
}
} // namespace

void sphx_relation_s::release()
{
    cudaFree(count);
    cudaFree(j);
    cudaFree(dW);
    cudaFree(W);
    cudaFree(r);
    cudaFree(e);
    cudaFree(wsum);
    count = j = nullptr;
    dW = W = r = e = wsum = nullptr;
    cap = 0;
    n_src = 0;
}

int sphx_relation_s::allocate(int new_cap, size_t n)
{
    cudaStreamSynchronize(ctx->stream);
    release();
    size_t nn = std::max<size_t>(n, 1);
    size_t slots = size_t(new_cap) * nn;
    int dim = src->dim;
    SPHX_CUDA(cudaMalloc(&count, nn * sizeof(uint32_t)));
    SPHX_CUDA(cudaMalloc(&wsum, nn * sizeof(double)));
    SPHX_CUDA(cudaMalloc(&j, slots * sizeof(uint32_t)));
    SPHX_CUDA(cudaMalloc(&dW, slots * sizeof(double)));
    SPHX_CUDA(cudaMalloc(&e, slots * dim * sizeof(double)));
    if (store_r)
        SPHX_CUDA(cudaMalloc(&r, slots * sizeof(double)));
    if (store_W)
        SPHX_CUDA(cudaMalloc(&W, slots * sizeof(double)));
    SPHX_CUDA(cudaMemsetAsync(count, 0, nn * sizeof(uint32_t), ctx->stream));
    cap = new_cap;
    n_src = n;
    return SPHX_OK;
}

extern "C" int sphx_relation_keep_distances(sphx_relation rel)
{
    if (!rel)
        return fail(SPHX_ERR_INVALID_ARG, "null relation");
    if (!rel->store_r)
    {
        rel->store_r = true;
        rel->n_src = size_t(-1); // storage is reallocated with distances at the next update
    }
    return SPHX_OK;
}

static int initial_capacity(int dim, bool inner) { return dim == 2 ? (inner ? 24 : 16) : (inner ? 96 : 64); }

extern "C" int sphx_inner_relation_create(sphx_body body, sphx_cell_list cl, double h, sphx_relation *out)
{
    if (!body || !cl || !out || !(h > 0) || body->dim != cl->mesh.dim)
        return fail(SPHX_ERR_INVALID_ARG, "invalid inner relation arguments");
    sphx_relation r = new sphx_relation_s();
    r->ctx = body->ctx;
    r->ctx->retain();
    r->inner = true;
    r->src = r->tgt = body;
    r->cl = cl;
    r->h = h;
    r->depth = 1; // SearchDepthSingleResolution
    r->store_W = false;
    r->store_r = false;
    *out = r;
    return SPHX_OK;
}

extern "C" int sphx_contact_relation_create(sphx_body body, sphx_body target, sphx_cell_list target_cl, double h,
                                            int search_depth, double target_rho0, sphx_relation *out)
{
    if (!body || !target || !target_cl || !out || !(h > 0) || search_depth < 1 || !(target_rho0 > 0) ||
        body->dim != target->dim || target->dim != target_cl->mesh.dim)
        return fail(SPHX_ERR_INVALID_ARG, "invalid contact relation arguments");
    sphx_relation r = new sphx_relation_s();
    r->ctx = body->ctx;
    r->ctx->retain();
    r->inner = false;
    r->src = body;
    r->tgt = target;
    r->cl = target_cl;
    r->h = h;
    r->depth = search_depth;
    r->tgt_inv_rho0 = 1.0 / target_rho0;
    r->store_W = true; // observers interpolate with W; walls need r_ij
    r->store_r = true;
    *out = r;
    return SPHX_OK;
}

extern "C" int sphx_relation_destroy(sphx_relation r)
{
    if (!r)
        return SPHX_OK;
    sphx_ctx ctx = r->ctx;
    cudaStreamSynchronize(ctx->stream);
    r->release();
    delete r;
    release(ctx);
    return SPHX_OK;
}

static int launch_build(sphx_relation rel, unsigned int *d_max)
{
    sphx_ctx ctx = rel->ctx;
    sphx_body src = rel->src, tgt = rel->tgt;
    sphx_cell_list cl = rel->cl;
    Field *spos, *tmass = nullptr;
    SPHX_TRY(src->need("Position", SPHX_F64, src->dim, &spos));
    if (!rel->inner)
        SPHX_TRY(tgt->need("Mass", SPHX_F64, 1, &tmass));
    BuildArgs a{};
    a.n_src = src->n;
    a.n_tgt = cl->n_entries; // stride of the cell-ordered entry arrays (images included)
    a.src_pos = static_cast<const double *>(spos->dev);
    a.cell_offset = cl->cell_offset;
    a.pidx = cl->particle_index;
    a.spos = cl->sorted_pos;
    a.soff = cl->sorted_off;
    a.m = mesh_dev(cl->mesh);
    a.k = wendland(src->dim, rel->h);
    a.depth = rel->depth;
    a.cap = rel->cap;
    a.count = rel->count;
    a.J = rel->j;
    a.DW = rel->dW;
    a.E = rel->e;
    a.R = rel->r;
    a.W = rel->W;
    a.wsum = rel->wsum;
    a.tgt_mass = tmass ? static_cast<const double *>(tmass->dev) : nullptr;
    a.tgt_inv_rho0 = rel->tgt_inv_rho0;
    a.max_count = d_max;
    unsigned grid = grid_for(a.n_src, kBlock);
    if (src->dim == 2)
    {
        if (rel->inner)
            k_build<2, true><<<grid, kBlock, 0, ctx->stream>>>(a);
        else
            k_build<2, false><<<grid, kBlock, 0, ctx->stream>>>(a);
    }
    else
    {
        if (rel->inner)
            k_build<3, true><<<grid, kBlock, 0, ctx->stream>>>(a);
        else
            k_build<3, false><<<grid, kBlock, 0, ctx->stream>>>(a);
    }
    SPHX_LAUNCHED(ctx);
    return SPHX_OK;
}

extern "C" int sphx_relation_update(sphx_relation rel)
{
    if (!rel)
        return fail(SPHX_ERR_INVALID_ARG, "null relation");
    if (rel->cl->n != rel->tgt->n)
        return fail(SPHX_ERR_INVALID_ARG, "target cell list holds %zu particles but the target body has %zu; update "
                                          "the cell linked list first", rel->cl->n, rel->tgt->n);
    sphx_ctx ctx = rel->ctx;
    size_t n = rel->src->n;
    if (rel->cap == 0 || rel->n_src != n)
        SPHX_TRY(rel->allocate(rel->cap ? rel->cap : initial_capacity(rel->src->dim, rel->inner), n));
    if (n == 0)
        return SPHX_OK;
    unsigned int *d_max = reinterpret_cast<unsigned int *>(ctx->d_red);
    for (int attempt = 0; attempt < 2; ++attempt)
    {
        SPHX_CUDA(cudaMemsetAsync(d_max, 0, sizeof(unsigned int), ctx->stream));
        SPHX_TRY(launch_build(rel, d_max));
        SPHX_CUDA(cudaMemcpyAsync(ctx->h_red, d_max, sizeof(unsigned int), cudaMemcpyDeviceToHost, ctx->stream));
        SPHX_CUDA(cudaStreamSynchronize(ctx->stream));
        unsigned int maxc = *reinterpret_cast<unsigned int *>(ctx->h_red);
        if (maxc <= unsigned(rel->cap))
            return SPHX_OK;
        // grow with head room and search again
        SPHX_TRY(rel->allocate(int(maxc + maxc / 4 + 4), n));
    }
    return fail(SPHX_ERR_CAPACITY, "neighbour lists overflowed after growing the storage");
}

extern "C" int sphx_relation_download(sphx_relation rel, uint32_t *counts, uint32_t *j, double *W, double *dW,
                                      double *r, double *e, size_t *total)
{
    if (!rel)
        return fail(SPHX_ERR_INVALID_ARG, "null relation");
    size_t n = rel->n_src;
    int dim = rel->src->dim;
    cudaStream_t s = rel->ctx->stream;
    std::vector<uint32_t> cnt(n);
    if (n)
        SPHX_CUDA(cudaMemcpyAsync(cnt.data(), rel->count, n * sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
    size_t slots = size_t(rel->cap) * n;
    std::vector<uint32_t> hj(j ? slots : 0);
    std::vector<double> hW(W && rel->W ? slots : 0), hdW(dW ? slots : 0), hr(r && rel->r ? slots : 0),
        he(e ? slots * dim : 0);
    if (j && slots)
        SPHX_CUDA(cudaMemcpyAsync(hj.data(), rel->j, slots * sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
    if (!hW.empty())
        SPHX_CUDA(cudaMemcpyAsync(hW.data(), rel->W, slots * sizeof(double), cudaMemcpyDeviceToHost, s));
    if (!hdW.empty())
        SPHX_CUDA(cudaMemcpyAsync(hdW.data(), rel->dW, slots * sizeof(double), cudaMemcpyDeviceToHost, s));
    if (!hr.empty())
        SPHX_CUDA(cudaMemcpyAsync(hr.data(), rel->r, slots * sizeof(double), cudaMemcpyDeviceToHost, s));
    if (!he.empty())
        SPHX_CUDA(cudaMemcpyAsync(he.data(), rel->e, slots * dim * sizeof(double), cudaMemcpyDeviceToHost, s));
    SPHX_CUDA(cudaStreamSynchronize(s));
    size_t t = 0;
    for (size_t i = 0; i < n; ++i)
    {
        if (counts)
            counts[i] = cnt[i];
        for (uint32_t k = 0; k < cnt[i] && k < uint32_t(rel->cap); ++k, ++t)
        {
            size_t slot = size_t(k) * n + i;
            if (j)
                j[t] = hj[slot];
            if (!hW.empty())
                W[t] = hW[slot];
            if (!hdW.empty())
                dW[t] = hdW[slot];
            if (!hr.empty())
                r[t] = hr[slot];
            if (!he.empty())
                for (int d = 0; d < dim; ++d)
                    e[t * dim + d] = he[d * slots + slot];
        }
    }
    if (total)
        *total = t;
    return SPHX_OK;
}
