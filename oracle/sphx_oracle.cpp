// sphx_oracle.cpp -- TEST INFRASTRUCTURE ONLY.
//
// FP64 CPU restatement (C++17 + OpenMP) of SPHinXsys' classic weakly-compressible
// fluid step, used as the parity oracle for the CUDA library and as the timed CPU
// baseline.  Only the test suite, the smoke check and the benchmark's CPU legs load
// this library; the product path never does.
//
// Each routine names the reference file:line it restates (paths relative to the
// SPHinXsys source tree).  Where the reference is order-nondeterministic (TBB
// concurrent_vector insertion into cells, TBB parallel quicksort) the oracle pins a
// canonical order: particles inside a cell ascend by index, neighbours are listed in
// mesh_for_each cell order then by ascending index, and the Morton re-sort is stable.
//
// Build: see oracle/Makefile (g++ -O2 -fopenmp -ffp-contract=off).

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <numeric>
#include <string>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace orc
{
using Real = double;
using UInt = uint32_t;
// src/shared/common/base_data_type.h:204-208
constexpr Real Pi = Real(M_PI);
constexpr Real TinyReal = Real(2.71051e-20);
constexpr Real MinReal = std::numeric_limits<Real>::lowest();

struct V3
{
    Real v[3] = {0, 0, 0};
    Real &operator[](int i) { return v[i]; }
    const Real &operator[](int i) const { return v[i]; }
};

// Canonical 2/3-component dot and squared norm: ((x0*y0 + x1*y1) + x2*y2).
inline Real dotd(const V3 &a, const V3 &b, int D)
{
    Real s = a[0] * b[0] + a[1] * b[1];
    if (D == 3)
        s = s + a[2] * b[2];
    return s;
}
inline Real sqnorm(const V3 &a, int D) { return dotd(a, a, D); }

//------------------------------------------------------------------------------
// Mesh: src/shared/meshes/base_mesh.cpp:6-16, base_mesh.hxx:9-26,68-99
//------------------------------------------------------------------------------
struct Mesh
{
    int D = 3;
    V3 lower;
    Real gs = 1;
    int grid_points[3] = {1, 1, 1};
    int all_cells[3] = {1, 1, 1};

    static Mesh fromBounds(int D, const V3 &blo, const V3 &bup, Real gs, int buffer_width)
    {
        Mesh m;
        m.D = D;
        m.gs = gs;
        Real buffer = Real(buffer_width) * gs;
        for (int a = 0; a < D; ++a)
        {
            m.lower[a] = blo[a] - buffer;
            Real tentative = bup[a] + buffer - m.lower[a];
            m.grid_points[a] = int(std::ceil(tentative / gs)) + 1;
            m.all_cells[a] = m.grid_points[a] - 1;
        }
        return m;
    }
    void cellIndex(const V3 &x, int c[3]) const
    {
        for (int a = 0; a < D; ++a)
        {
            int k = int(std::floor((x[a] - lower[a]) / gs));
            k = std::max(k, 0);
            k = std::min(k, grid_points[a] - 2);
            c[a] = k;
        }
    }
    UInt linear(const int c[3]) const
    {
        if (D == 2)
            return UInt(c[0]) * UInt(all_cells[1]) + UInt(c[1]);
        return UInt(c[0]) * UInt(all_cells[1]) * UInt(all_cells[2]) + UInt(c[1]) * UInt(all_cells[2]) + UInt(c[2]);
    }
    size_t numCells() const
    {
        size_t n = 1;
        for (int a = 0; a < D; ++a)
            n *= size_t(all_cells[a]);
        return n;
    }
    V3 cellCentre(const int c[3]) const
    {
        V3 p;
        for (int a = 0; a < D; ++a)
            p[a] = (lower[a] + Real(c[a]) * gs) + 0.5 * gs;
        return p;
    }
    static UInt morton(UInt i)
    {
        UInt x = i & 0x3ff;
        x = (x | x << 16) & 0x30000ff;
        x = (x | x << 8) & 0x300f00f;
        x = (x | x << 4) & 0x30c30c3;
        x = (x | x << 2) & 0x9249249;
        return x;
    }
    UInt mortonKey(const V3 &x) const
    {
        int c[3];
        cellIndex(x, c);
        if (D == 2)
            return morton(UInt(c[0])) | (morton(UInt(c[1])) << 1);
        return morton(UInt(c[0])) | (morton(UInt(c[1])) << 1) | (morton(UInt(c[2])) << 2);
    }
};

//------------------------------------------------------------------------------
// Wendland C2: src/shared/kernels/kernel_wendland_c2.cpp:8-45, base_kernel.cpp:6-76
//------------------------------------------------------------------------------
struct Kernel
{
    int D = 3;
    Real h, inv_h, rc, rc_sqr, factor_W, factor_dW;
    Kernel(int D_, Real h_) : D(D_), h(h_)
    {
        inv_h = 1.0 / h;
        rc = 2.0 * h;
        rc_sqr = rc * rc;
        if (D == 2)
            factor_W = inv_h * inv_h * 7.0 / (4.0 * Pi);
        else
            factor_W = inv_h * inv_h * inv_h * 21.0 / (16.0 * Pi);
        factor_dW = inv_h * factor_W;
    }
    Real W(Real r) const
    {
        Real q = r * inv_h;
        return factor_W * (std::pow(1.0 - 0.5 * q, 4) * (1.0 + 2.0 * q));
    }
    Real dW(Real r) const
    {
        Real q = r * inv_h;
        return factor_dW * (0.625 * std::pow(q - 2.0, 3) * q);
    }
    Real W0() const { return factor_W; }
};

// SPHAdaptation::computeLatticeNumberDensity: src/shared/adaptations/adaptation.cpp:25-58
Real latticeNumberDensity(const Kernel &k, Real dp)
{
    Real sigma = 0;
    int depth = int(k.rc / dp) + 1;
    if (k.D == 2)
    {
        for (int j = -depth; j <= depth; ++j)
            for (int i = -depth; i <= depth; ++i)
            {
                Real x = i * dp, y = j * dp;
                Real d = std::sqrt(x * x + y * y);
                if (d < k.rc)
                    sigma += k.W(d);
            }
    }
    else
    {
        for (int kk = -depth; kk <= depth; ++kk)
            for (int j = -depth; j <= depth; ++j)
                for (int i = -depth; i <= depth; ++i)
                {
                    Real x = i * dp, y = j * dp, z = kk * dp;
                    Real d = std::sqrt((x * x + y * y) + z * z);
                    if (d < k.rc)
                        sigma += k.W(d);
                }
    }
    return sigma;
}

//------------------------------------------------------------------------------
// Box shapes: geometric_element.cpp:19-55 (closest point), geometric_element.h:43-55
// (contain, boundary included), base_geometry.cpp:45-58,84-137 (binary shapes, normal)
//------------------------------------------------------------------------------
struct Box
{
    V3 c, hs;
    bool contain(const V3 &x, int D) const
    {
        for (int a = 0; a < D; ++a)
            if (std::abs(x[a] - c[a]) > hs[a])
                return false;
        return true;
    }
    V3 closest(const V3 &x, int D) const
    {
        V3 p;
        for (int a = 0; a < D; ++a)
            p[a] = x[a] - c[a];
        bool inside = true;
        for (int a = 0; a < D; ++a)
        {
            if (p[a] < -hs[a])
            {
                p[a] = -hs[a];
                inside = false;
            }
            else if (p[a] > hs[a])
            {
                p[a] = hs[a];
                inside = false;
            }
        }
        if (inside)
        {
            int which = 0;
            Real mind = hs[0] - std::abs(p[0]);
            for (int a = 1; a < D; ++a)
            {
                Real d = hs[a] - std::abs(p[a]);
                if (d < mind)
                {
                    which = a;
                    mind = d;
                }
            }
            p[which] = p[which] < 0 ? -hs[which] : hs[which];
        }
        V3 out;
        for (int a = 0; a < D; ++a)
            out[a] = p[a] + c[a];
        return out;
    }
};

// Wall = outer box minus inner box (Dambreak.cpp:39-47).
struct WallShape
{
    Box outer, inner;
    bool contain(const V3 &x, int D) const { return outer.contain(x, D) && !inner.contain(x, D); }
    V3 closest(const V3 &x, int D) const
    {
        V3 best;
        Real dmin = std::numeric_limits<Real>::max();
        const Box *boxes[2] = {&outer, &inner};
        for (const Box *b : boxes)
        {
            V3 p = b->closest(x, D);
            V3 d;
            for (int a = 0; a < D; ++a)
                d[a] = x[a] - p[a];
            Real dist = std::sqrt(sqnorm(d, D));
            if (dist <= dmin)
            {
                dmin = dist;
                best = p;
            }
        }
        return best;
    }
    V3 normal(const V3 &x, int D) const
    {
        bool in = contain(x, D);
        V3 p = closest(x, D), d;
        for (int a = 0; a < D; ++a)
            d[a] = p[a] - x[a];
        Real n = std::sqrt(sqnorm(d, D));
        V3 out;
        for (int a = 0; a < D; ++a)
            out[a] = (in ? 1.0 : -1.0) * (d[a] / n);
        return out;
    }
};

//------------------------------------------------------------------------------
// Particles and neighbourhoods
//------------------------------------------------------------------------------
struct Body
{
    size_t n = 0;
    std::vector<V3> pos, vel, force, force_prior, prev_gravity, normal, acc_ave, vel_ave;
    std::vector<Real> rho, p, drho_dt, mass, Vol, rho_sum, observed;
    std::vector<UInt> original_id, sorted_id;
    void resize(size_t n_)
    {
        n = n_;
        pos.resize(n);
        vel.assign(n, V3());
        force.assign(n, V3());
        force_prior.assign(n, V3());
        prev_gravity.assign(n, V3());
        normal.assign(n, V3());
        acc_ave.assign(n, V3());
        vel_ave.assign(n, V3());
        rho.assign(n, 0);
        p.assign(n, 0);
        drho_dt.assign(n, 0);
        mass.assign(n, 0);
        Vol.assign(n, 0);
        rho_sum.assign(n, 0);
        observed.assign(n, 0);
        original_id.resize(n);
        sorted_id.resize(n);
        std::iota(original_id.begin(), original_id.end(), 0u);
        std::iota(sorted_id.begin(), sorted_id.end(), 0u);
    }
};

// Neighborhood SoA lists: src/shared/particle_neighborhood/neighborhood.h:49-80
struct Neighborhood
{
    std::vector<UInt> j;
    std::vector<Real> W, dW, r;
    std::vector<V3> e;
    void clear()
    {
        j.clear();
        W.clear();
        dW.clear();
        r.clear();
        e.clear();
    }
    size_t size() const { return j.size(); }
};

// Periodic images of PeriodicConditionUsingCellLinkedList (domain_bounding.cpp:16-60): along
// each periodic axis in turn, every entry (particle or an image of an earlier axis) with
// lower < x_a < lower + rc gets an image at x_a + L in the cell list, every entry with
// upper - rc < x_a < upper one at x_a - L.  Canonical order: per axis all lower-side images
// in entry order, then all upper-side ones (the reference inserts them concurrently).
struct Periodicity
{
    bool on[3] = {false, false, false};
    Real lower[3] = {0, 0, 0}, upper[3] = {0, 0, 0};
    Real rc = 0;
    bool any() const { return on[0] || on[1] || on[2]; }
};

// Cell lists: cell_linked_list.cpp:22-101; canonical ascending-index order.  Entries are
// the particles (entry e = particle e) followed by periodic images; particle_index[k] is
// the particle of the k-th entry in cell order, entry_sorted[k] that entry.
struct CellList
{
    Mesh mesh;
    std::vector<UInt> cell_offset, particle_index, entry_sorted, entry_index;
    std::vector<V3> entry_pos;
    void update(const Body &b, const Periodicity *per = nullptr)
    {
        entry_pos.assign(b.pos.begin(), b.pos.end());
        entry_index.resize(b.n);
        std::iota(entry_index.begin(), entry_index.end(), 0u);
        if (per && per->any())
            for (int a = 0; a < mesh.D; ++a)
            {
                if (!per->on[a])
                    continue;
                size_t n_cur = entry_pos.size();
                Real L = per->upper[a] - per->lower[a];
                for (int side = 0; side < 2; ++side)
                    for (size_t e = 0; e < n_cur; ++e)
                    {
                        Real x = entry_pos[e][a];
                        bool take = side == 0 ? (x > per->lower[a] && x < per->lower[a] + per->rc)
                                              : (x < per->upper[a] && x > per->upper[a] - per->rc);
                        if (!take)
                            continue;
                        V3 p = entry_pos[e];
                        p[a] = side == 0 ? x + L : x - L;
                        entry_pos.push_back(p);
                        entry_index.push_back(entry_index[e]);
                    }
            }
        size_t ne = entry_pos.size();
        size_t nc = mesh.numCells();
        std::vector<UInt> cell(ne);
        cell_offset.assign(nc + 1, 0);
#pragma omp parallel for schedule(static)
        for (long e = 0; e < (long)ne; ++e)
        {
            int c[3];
            mesh.cellIndex(entry_pos[e], c);
            cell[e] = mesh.linear(c);
        }
        for (size_t e = 0; e < ne; ++e)
            cell_offset[cell[e] + 1]++;
        for (size_t c = 0; c < nc; ++c)
            cell_offset[c + 1] += cell_offset[c];
        std::vector<UInt> fill(cell_offset.begin(), cell_offset.end() - 1);
        entry_sorted.assign(std::max(ne, nc), 0);
        particle_index.assign(std::max(ne, nc), 0);
        for (size_t e = 0; e < ne; ++e)
        {
            UInt k = fill[cell[e]]++;
            entry_sorted[k] = UInt(e);
            particle_index[k] = entry_index[e];
        }
    }
};

//------------------------------------------------------------------------------
// CK numerics: KernelTabulatedCK (kernel_tabulated_ck.h:37-62, .cpp:5-25) evaluated as
// Neighbor<SPHAdaptation, SPHAdaptation>::SmoothingKernel does (neighbor_method.hpp:66-142)
//------------------------------------------------------------------------------
struct TabKernel
{
    static constexpr int resolution = 20, size = resolution + 4;
    int D = 2;
    Real inv_h = 1, inv_h2 = 1, inv_h3 = 1, inv_h4 = 1, dim_factor = 1;
    Real dq = 0.1, d0 = 1, d1 = 1, d2 = 1, d3 = 1;
    Real w[size], dw[size];
    TabKernel() = default;
    TabKernel(int D_, Real h) : D(D_)
    {
        // KernelWendlandC2 (kernel_wendland_c2.cpp): W_1D, dW_1D; kernel size 2
        Real kinv_h = 1.0 / h;
        Real fW2 = kinv_h * kinv_h * 7.0 / (4.0 * Pi), fW3 = kinv_h * kinv_h * kinv_h * 21.0 / (16.0 * Pi);
        dim_factor = D == 2 ? fW2 * h * h : fW3 * h * h * h; // Kernel::DimensionFactor2D/3D
        dq = 2.0 / Real(resolution);
        for (int i = 0; i < size; ++i)
        {
            Real q = Real(i - 1) * dq;
            w[i] = std::pow(1.0 - 0.5 * q, 4) * (1.0 + 2.0 * q);
            dw[i] = 0.625 * std::pow(q - 2.0, 3) * q;
        }
        d0 = (-1.0 * dq) * (-2.0 * dq) * (-3.0 * dq);
        d1 = dq * (-1.0 * dq) * (-2.0 * dq);
        d2 = (2.0 * dq) * dq * (-1.0 * dq);
        d3 = (3.0 * dq) * (2.0 * dq) * dq;
        inv_h = 1.0 / h;
        inv_h2 = inv_h * inv_h;
        inv_h3 = inv_h2 * inv_h;
        inv_h4 = inv_h3 * inv_h;
    }
    Real cubic(const Real *data, Real q) const
    {
        int location = (int)std::floor(q / dq);
        int i = location + 1;
        Real f1 = q - Real(location) * dq, f0 = f1 + dq, f2 = f1 - dq, f3 = f1 - 2 * dq;
        return (f1 * f2 * f3) / d0 * data[i - 1] + (f0 * f2 * f3) / d1 * data[i] + (f0 * f1 * f3) / d2 * data[i + 1] +
               (f0 * f1 * f2) / d3 * data[i + 2];
    }
    Real W(Real r) const { return (D == 2 ? inv_h2 : inv_h3) * dim_factor * cubic(w, r * inv_h); }
    Real dW(Real r) const { return (D == 2 ? inv_h3 : inv_h4) * dim_factor * cubic(dw, r * inv_h); }
    Real W0() const { return (D == 2 ? inv_h2 : inv_h3) * dim_factor * cubic(w, 0.0); }
};

// Row-major D x D matrix in a 3 x 3 array.
struct M3
{
    Real m[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    Real &operator()(int r, int c) { return m[r * 3 + c]; }
    Real operator()(int r, int c) const { return m[r * 3 + c]; }
    static M3 identity(int D)
    {
        M3 I;
        for (int a = 0; a < D; ++a)
            I(a, a) = 1.0;
        return I;
    }
};
inline V3 mul(const M3 &A, const V3 &x, int D)
{
    V3 y;
    for (int r = 0; r < D; ++r)
    {
        Real s = 0;
        for (int c = 0; c < D; ++c)
            s += A(r, c) * x[c];
        y[r] = s;
    }
    return y;
}
inline Real det(const M3 &A, int D)
{
    if (D == 2)
        return A(0, 0) * A(1, 1) - A(0, 1) * A(1, 0);
    return A(0, 0) * (A(1, 1) * A(2, 2) - A(1, 2) * A(2, 1)) - A(0, 1) * (A(1, 0) * A(2, 2) - A(1, 2) * A(2, 0)) +
           A(0, 2) * (A(1, 0) * A(2, 1) - A(1, 1) * A(2, 0));
}
// Inverse by the adjugate (small fixed-size matrices).
inline M3 inverse(const M3 &A, int D)
{
    M3 R;
    Real d = det(A, D);
    if (D == 2)
    {
        R(0, 0) = A(1, 1) / d;
        R(0, 1) = -A(0, 1) / d;
        R(1, 0) = -A(1, 0) / d;
        R(1, 1) = A(0, 0) / d;
        return R;
    }
    R(0, 0) = (A(1, 1) * A(2, 2) - A(1, 2) * A(2, 1)) / d;
    R(0, 1) = (A(0, 2) * A(2, 1) - A(0, 1) * A(2, 2)) / d;
    R(0, 2) = (A(0, 1) * A(1, 2) - A(0, 2) * A(1, 1)) / d;
    R(1, 0) = (A(1, 2) * A(2, 0) - A(1, 0) * A(2, 2)) / d;
    R(1, 1) = (A(0, 0) * A(2, 2) - A(0, 2) * A(2, 0)) / d;
    R(1, 2) = (A(0, 2) * A(1, 0) - A(0, 0) * A(1, 2)) / d;
    R(2, 0) = (A(1, 0) * A(2, 1) - A(1, 1) * A(2, 0)) / d;
    R(2, 1) = (A(0, 1) * A(2, 0) - A(0, 0) * A(2, 1)) / d;
    R(2, 2) = (A(0, 0) * A(1, 1) - A(0, 1) * A(1, 0)) / d;
    return R;
}

// CK fluid state beside the classic Body: Compression, CompressionRate, Displacement,
// LinearCorrectionMatrix, VolumetricMeasureRef, CompressionSummation.
struct CKState
{
    std::vector<Real> compression, compression_rate, Vol_ref, compression_sum, wall_Vol_ref;
    std::vector<V3> dpos;
    std::vector<M3> B;
    std::vector<Real> pos_div;              // "PositionDivergence"
    std::vector<int> indicator, prev_indicator; // "Indicator", "PreviousSurfaceIndicator" (initial 1)
    Real present_time = 0, interval = 0; // TimeStepper::TriggerByInterval of the advection step
    long advection_steps = 0;
    bool ready = false;
};

struct Case
{
    int D = 2;
    Real dp = 0.025, h = 0.0325;
    Real rho0 = 1, c0 = 20, U_ref = 2, p0 = 400, wall_rho0 = 1;
    V3 gravity;
    Kernel kernel{2, 0.0325};
    Real sigma0 = 1, inv_sigma0 = 1, W0 = 0;
    Real h_min = 0.0325;
    Real acoustic_cfl = 0.6, advection_cfl = 0.25;
    // acoustic Riemann solver: riemann_solver.h:55-124, common_functors.h:82-94
    Real rho0c0, inv_rho0c0_ave, rho0c0_geo_ave, inv_c0_ave, limiter_slope = 3.0;
    Body fluid, wall, observer;
    CellList fluid_cells, wall_cells;
    int contact_depth = 2;
    std::vector<Neighborhood> inner, contact, obs;
    Box water_box;
    WallShape wall_shape;
    TabKernel tk;
    CKState ck;
    // Taylor-Green set-up (taylor_green.cpp): periodic box, viscosity, plain DensitySummation
    Periodicity periodic;
    Real mu = 0;
    bool free_surface = true;
    std::vector<V3> viscous_force, prev_viscous;
    V3 sys_lo, sys_up;
    Mesh sort_mesh;

    Real PJump(Real u) const
    {
        return rho0c0_geo_ave * u * std::min(limiter_slope * (inv_c0_ave * std::max(u, Real(0))), Real(1));
    }
    Real UJump(Real dp_) const { return dp_ * inv_rho0c0_ave; }
    Real getPressure(Real rho) const { return p0 * (rho / rho0 - 1.0); }
};

//------------------------------------------------------------------------------
// Neighbour search: cell_linked_list.hpp:20-46 with NeighborBuilderInner
// (neighborhood.cpp:85-98) and NeighborBuilderContact (neighborhood.cpp:144-160)
//------------------------------------------------------------------------------
template <bool INNER>
void searchNeighbors(const Case &cs, const Body &src, const Body &tgt, const CellList &cl, int depth,
                     std::vector<Neighborhood> &config)
{
    const int D = cs.D;
    const Mesh &m = cl.mesh;
    config.resize(src.n);
#pragma omp parallel for schedule(dynamic, 256)
    for (long i = 0; i < (long)src.n; ++i)
    {
        Neighborhood &nb = config[i];
        nb.clear();
        int c[3] = {0, 0, 0}, lo[3] = {0, 0, 0}, hi[3] = {1, 1, 1};
        m.cellIndex(src.pos[i], c);
        for (int a = 0; a < D; ++a)
        {
            lo[a] = std::max(0, c[a] - depth);
            hi[a] = std::min(m.all_cells[a], c[a] + depth + 1);
        }
        int cc[3] = {0, 0, 0};
        for (cc[0] = lo[0]; cc[0] < hi[0]; ++cc[0])
            for (cc[1] = lo[1]; cc[1] < hi[1]; ++cc[1])
                for (cc[2] = lo[2]; cc[2] < hi[2]; ++cc[2])
                {
                    UInt lc = m.linear(cc);
                    for (UInt k = cl.cell_offset[lc]; k < cl.cell_offset[lc + 1]; ++k)
                    {
                        UInt j = cl.particle_index[k];
                        const V3 &xj = cl.entry_pos[cl.entry_sorted[k]]; // the particle or its image
                        V3 d;
                        for (int a = 0; a < D; ++a)
                            d[a] = src.pos[i][a] - xj[a];
                        Real r2 = sqnorm(d, D);
                        if (r2 < cs.kernel.rc_sqr && (!INNER || UInt(i) != j))
                        {
                            Real r = std::sqrt(r2);
                            nb.j.push_back(j);
                            nb.W.push_back(cs.kernel.W(r));
                            nb.dW.push_back(cs.kernel.dW(r));
                            nb.r.push_back(r);
                            V3 e;
                            for (int a = 0; a < D; ++a)
                                e[a] = d[a] / (r + TinyReal);
                            nb.e.push_back(e);
                        }
                    }
                }
    }
}

void updateConfiguration(Case &cs)
{
    searchNeighbors<true>(cs, cs.fluid, cs.fluid, cs.fluid_cells, 1, cs.inner);
    searchNeighbors<false>(cs, cs.fluid, cs.wall, cs.wall_cells, cs.contact_depth, cs.contact);
}
void updateObserverConfiguration(Case &cs)
{
    // observer contact relation: same kernel (equal smoothing lengths), depth 1+floor(rc/gs)
    searchNeighbors<false>(cs, cs.observer, cs.fluid, cs.fluid_cells, cs.contact_depth, cs.obs);
}

//------------------------------------------------------------------------------
// DensitySummationComplexFreeSurface: density_summation.cpp:74-82,113-144,
// density_summation.hpp:28-32 (FreeSurface update; Vol is not updated)
//------------------------------------------------------------------------------
void densitySummation(Case &cs)
{
    Body &f = cs.fluid;
    const Real inv_rho0_wall = 1.0 / cs.wall_rho0; // Solid() default reference density is 1
#pragma omp parallel for schedule(static)
    for (long i = 0; i < (long)f.n; ++i)
    {
        Real sigma = cs.W0;
        const Neighborhood &nb = cs.inner[i];
        for (size_t n = 0; n < nb.size(); ++n)
            sigma += nb.W[n];
        Real rho_sum = sigma * cs.rho0 * cs.inv_sigma0;
        Real sigma_c = 0;
        const Neighborhood &wn = cs.contact[i];
        for (size_t n = 0; n < wn.size(); ++n)
            sigma_c += wn.W[n] * inv_rho0_wall * cs.wall.mass[wn.j[n]];
        rho_sum += sigma_c * cs.rho0 * cs.rho0 * cs.inv_sigma0 / f.mass[i];
        f.rho_sum[i] = rho_sum;
    }
    // DensitySummation<Inner<FreeSurface>>: max(rho_sum, rho0); <Inner<>>: rho_sum
#pragma omp parallel for schedule(static)
    for (long i = 0; i < (long)f.n; ++i)
        f.rho[i] = cs.free_surface ? std::max(f.rho_sum[i], cs.rho0) : f.rho_sum[i];
}

//------------------------------------------------------------------------------
// Integration1stHalfWithWallRiemann: fluid_integration.hpp:49-113
//------------------------------------------------------------------------------
void integration1stHalf(Case &cs, Real dt)
{
    const int D = cs.D;
    Body &f = cs.fluid;
    const Body &w = cs.wall;
#pragma omp parallel for schedule(static)
    for (long i = 0; i < (long)f.n; ++i)
    {
        f.rho[i] += f.drho_dt[i] * dt * 0.5;
        f.p[i] = cs.getPressure(f.rho[i]);
        for (int a = 0; a < D; ++a)
            f.pos[i][a] += f.vel[i][a] * dt * 0.5;
    }
#pragma omp parallel for schedule(static)
    for (long i = 0; i < (long)f.n; ++i)
    {
        // inner (fluid_integration.hpp:63-80)
        V3 force;
        Real rho_dissipation = 0;
        const Neighborhood &nb = cs.inner[i];
        for (size_t n = 0; n < nb.size(); ++n)
        {
            UInt j = nb.j[n];
            Real dW_ijV_j = nb.dW[n] * f.Vol[j];
            Real s = (f.p[i] + f.p[j]) * dW_ijV_j;
            for (int a = 0; a < D; ++a)
                force[a] -= s * nb.e[n][a];
            rho_dissipation += cs.UJump(f.p[i] - f.p[j]) * dW_ijV_j;
        }
        for (int a = 0; a < D; ++a)
            f.force[i][a] += force[a] * f.Vol[i];
        f.drho_dt[i] = rho_dissipation * f.rho[i];
        // wall contact (fluid_integration.hpp:88-113)
        V3 wforce;
        Real wrho = 0;
        const Neighborhood &wn = cs.contact[i];
        for (size_t n = 0; n < wn.size(); ++n)
        {
            UInt j = wn.j[n];
            const V3 &e = wn.e[n];
            Real dW_ijV_j = wn.dW[n] * w.Vol[j];
            Real r_ij = wn.r[n];
            V3 acc, me;
            for (int a = 0; a < D; ++a)
            {
                acc[a] = f.force_prior[i][a] / f.mass[i] - w.acc_ave[j][a];
                me[a] = -e[a];
            }
            Real face_acc = dotd(acc, me, D);
            Real p_j_in_wall = f.p[i] + f.rho[i] * r_ij * std::max(Real(0), face_acc);
            Real s = (f.p[i] + p_j_in_wall) * dW_ijV_j;
            for (int a = 0; a < D; ++a)
                wforce[a] -= s * e[a];
            wrho += cs.UJump(f.p[i] - p_j_in_wall) * dW_ijV_j;
        }
        for (int a = 0; a < D; ++a)
            f.force[i][a] += wforce[a] * f.Vol[i];
        f.drho_dt[i] += wrho * f.rho[i];
    }
#pragma omp parallel for schedule(static)
    for (long i = 0; i < (long)f.n; ++i)
        for (int a = 0; a < D; ++a)
            f.vel[i][a] += (f.force_prior[i][a] + f.force[i][a]) / f.mass[i] * dt;
}

//------------------------------------------------------------------------------
// Integration2ndHalfWithWallRiemann: fluid_integration.hpp:166-231
//------------------------------------------------------------------------------
void integration2ndHalf(Case &cs, Real dt)
{
    const int D = cs.D;
    Body &f = cs.fluid;
    const Body &w = cs.wall;
#pragma omp parallel for schedule(static)
    for (long i = 0; i < (long)f.n; ++i)
        for (int a = 0; a < D; ++a)
            f.pos[i][a] += f.vel[i][a] * dt * 0.5;
#pragma omp parallel for schedule(static)
    for (long i = 0; i < (long)f.n; ++i)
    {
        Real density_change_rate = 0;
        V3 p_dissipation;
        const Neighborhood &nb = cs.inner[i];
        for (size_t n = 0; n < nb.size(); ++n)
        {
            UInt j = nb.j[n];
            const V3 &e = nb.e[n];
            Real dW_ijV_j = nb.dW[n] * f.Vol[j];
            V3 dv;
            for (int a = 0; a < D; ++a)
                dv[a] = f.vel[i][a] - f.vel[j][a];
            Real u_jump = dotd(dv, e, D);
            density_change_rate += u_jump * dW_ijV_j;
            Real s = cs.PJump(u_jump) * dW_ijV_j;
            for (int a = 0; a < D; ++a)
                p_dissipation[a] += s * e[a];
        }
        f.drho_dt[i] += density_change_rate * f.rho[i];
        for (int a = 0; a < D; ++a)
            f.force[i][a] = p_dissipation[a] * f.Vol[i];
        // wall contact
        Real wrate = 0;
        V3 wdiss;
        const Neighborhood &wn = cs.contact[i];
        for (size_t n = 0; n < wn.size(); ++n)
        {
            UInt j = wn.j[n];
            const V3 &e = wn.e[n];
            Real dW_ijV_j = wn.dW[n] * w.Vol[j];
            const V3 &nj = w.normal[j];
            Real sg = dotd(e, nj, D);
            Real sgn = sg < 0 ? -1.0 : (sg > 0 ? 1.0 : 0.0);
            V3 n_star, vin_wall, dv, dv2;
            for (int a = 0; a < D; ++a)
            {
                n_star[a] = sgn * nj[a];
                vin_wall[a] = 2.0 * w.vel_ave[j][a] - f.vel[i][a];
                dv[a] = f.vel[i][a] - vin_wall[a];
                dv2[a] = f.vel[i][a] - w.vel_ave[j][a];
            }
            wrate += dotd(dv, e, D) * dW_ijV_j;
            Real u_jump = 2.0 * dotd(dv2, n_star, D);
            Real s = cs.PJump(u_jump) * dW_ijV_j;
            for (int a = 0; a < D; ++a)
                wdiss[a] += s * n_star[a];
        }
        f.drho_dt[i] += wrate * f.rho[i];
        for (int a = 0; a < D; ++a)
            f.force[i][a] += wdiss[a] * f.Vol[i];
    }
#pragma omp parallel for schedule(static)
    for (long i = 0; i < (long)f.n; ++i)
        f.rho[i] += f.drho_dt[i] * dt * 0.5;
}

//------------------------------------------------------------------------------
// Time steps: fluid_time_step.cpp:21-31 (acoustic), :54-65 (advection); ReduceMax
// starting at MinReal (reduce_functors.h:73-82)
//------------------------------------------------------------------------------
Real acousticTimeStep(const Case &cs)
{
    const Body &f = cs.fluid;
    Real m = MinReal;
#pragma omp parallel for reduction(max : m) schedule(static)
    for (long i = 0; i < (long)f.n; ++i)
        m = std::max(m, cs.c0 + std::sqrt(sqnorm(f.vel[i], cs.D)));
    return cs.acoustic_cfl * cs.h_min / (m + TinyReal);
}
Real advectionTimeStep(const Case &cs)
{
    const Body &f = cs.fluid;
    const int D = cs.D;
    Real m = MinReal;
#pragma omp parallel for reduction(max : m) schedule(static)
    for (long i = 0; i < (long)f.n; ++i)
    {
        V3 ft;
        for (int a = 0; a < D; ++a)
            ft[a] = f.force[i][a] + f.force_prior[i][a];
        Real acc = 4.0 * cs.h_min * std::sqrt(sqnorm(ft, D)) / f.mass[i];
        m = std::max(m, std::max(sqnorm(f.vel[i], D), acc));
    }
    Real speed_max = std::sqrt(m);
    return cs.advection_cfl * cs.h_min / (std::max(speed_max, cs.U_ref) + TinyReal);
}

//------------------------------------------------------------------------------
// ParticleSorting: particle_sorting.cpp:25-58 (Morton sequence of the finest mesh,
// base_mesh.hxx:80-99); the oracle uses a stable sort.
//------------------------------------------------------------------------------
template <typename T>
void permute(std::vector<T> &v, const std::vector<UInt> &perm)
{
    std::vector<T> tmp(v.size());
    for (size_t k = 0; k < perm.size(); ++k)
        tmp[k] = v[perm[k]];
    v.swap(tmp);
}
void particleSorting(Case &cs)
{
    Body &f = cs.fluid;
    std::vector<UInt> key(f.n), perm(f.n);
    for (size_t i = 0; i < f.n; ++i)
        key[i] = cs.sort_mesh.mortonKey(f.pos[i]);
    std::iota(perm.begin(), perm.end(), 0u);
    std::stable_sort(perm.begin(), perm.end(), [&](UInt a, UInt b) { return key[a] < key[b]; });
    permute(f.pos, perm);
    permute(f.vel, perm);
    permute(f.force, perm);
    permute(f.force_prior, perm);
    permute(f.prev_gravity, perm);
    permute(f.rho, perm);
    permute(f.p, perm);
    permute(f.drho_dt, perm);
    permute(f.mass, perm);
    permute(f.Vol, perm);
    permute(f.original_id, perm);
    for (size_t i = 0; i < f.n; ++i)
        f.sorted_id[f.original_id[i]] = UInt(i);
}

// ObservedQuantityRecording<Real>("Pressure"): general_interpolation.h:58-78
void observePressure(Case &cs)
{
    Body &o = cs.observer;
    for (size_t i = 0; i < o.n; ++i)
    {
        Real q = 0, ttl = 0;
        const Neighborhood &nb = cs.obs[i];
        for (size_t n = 0; n < nb.size(); ++n)
        {
            Real w = nb.W[n] * cs.fluid.Vol[nb.j[n]];
            q += w * cs.fluid.p[nb.j[n]];
            ttl += w;
        }
        o.observed[i] = q / (ttl + TinyReal);
    }
}

// TotalMechanicalEnergy: general_reduce.cpp:75-79, external_force.h:53-56 (zero reference 0)
Real totalMechanicalEnergy(const Case &cs)
{
    const Body &f = cs.fluid;
    Real e = 0;
    for (size_t i = 0; i < f.n; ++i)
    {
        V3 mx;
        for (int a = 0; a < cs.D; ++a)
            mx[a] = -f.pos[i][a];
        e += 0.5 * f.mass[i] * sqnorm(f.vel[i], cs.D) + f.mass[i] * dotd(cs.gravity, mx, cs.D);
    }
    return e;
}

// UpperFrontInAxisDirection over a gauge box region: general_reduce.h:82-99
Real upperFront(const Case &cs, int axis, const V3 &lo, const V3 &up)
{
    const Body &f = cs.fluid;
    Real m = MinReal;
    for (size_t i = 0; i < f.n; ++i)
    {
        bool in = true;
        for (int a = 0; a < cs.D; ++a)
            if (f.pos[i][a] < lo[a] || f.pos[i][a] > up[a])
                in = false;
        if (in)
            m = std::max(m, f.pos[i][axis]);
    }
    return m;
}

//------------------------------------------------------------------------------
// CK dam-break numerics (tests/tests_sycl/2d_examples/test_2d_dambreak_sycl/dambreak_sycl.cpp):
// pair geometry from the current Position (moved once per advection step by
// UpdateParticlePosition), the tabulated kernel, the neighbour lists of the configuration.
//------------------------------------------------------------------------------
inline V3 sub3(const V3 &a, const V3 &b, int D)
{
    V3 r;
    for (int k = 0; k < D; ++k)
        r[k] = a[k] - b[k];
    return r;
}
// Eigen normalized(): x / |x| for a non-zero x, x itself otherwise
inline V3 normalized(const V3 &x, int D)
{
    Real n2 = sqnorm(x, D);
    V3 e = x;
    if (n2 > 0)
    {
        Real n = std::sqrt(n2);
        for (int k = 0; k < D; ++k)
            e[k] = x[k] / n;
    }
    return e;
}

void ckEnsureState(Case &cs)
{
    CKState &ck = cs.ck;
    size_t n = cs.fluid.n;
    if (ck.ready && ck.compression.size() == n && ck.wall_Vol_ref.size() == cs.wall.n)
        return;
    ck.compression.assign(n, 1.0);   // registerStateVariable("Compression", 1)
    ck.compression_rate.assign(n, 0.0);
    ck.compression_sum.assign(n, 1.0);
    ck.dpos.assign(n, V3());
    ck.B.assign(n, M3::identity(cs.D)); // "LinearCorrectionMatrix", identity
    ck.Vol_ref = cs.fluid.Vol;           // registerStateVariableFrom("VolumetricMeasureRef", ...)
    ck.wall_Vol_ref = cs.wall.Vol;
    ck.pos_div.assign(n, 0.0);
    ck.indicator.assign(n, 0);
    ck.prev_indicator.assign(n, 1);
    ck.ready = true;
}

// CompressionSummation<Inner, Contact> + DensityRegularization<FreeSurface>:
// density_regularization.hpp:40-118, density_regularization.h:164-180
void ckDensityRegularization(Case &cs)
{
    ckEnsureState(cs);
    const int D = cs.D;
    Body &f = cs.fluid;
    CKState &ck = cs.ck;
#pragma omp parallel for schedule(static)
    for (long i = 0; i < (long)f.n; ++i)
    {
        Real sum = cs.tk.W0() * ck.Vol_ref[i];
        const Neighborhood &nb = cs.inner[i];
        for (size_t k = 0; k < nb.size(); ++k)
        {
            UInt j = nb.j[k];
            Real r = std::sqrt(sqnorm(sub3(f.pos[i], f.pos[j], D), D));
            sum += cs.tk.W(r) * ck.Vol_ref[j];
        }
        const Neighborhood &nw = cs.contact[i];
        for (size_t k = 0; k < nw.size(); ++k)
        {
            UInt j = nw.j[k];
            Real r = std::sqrt(sqnorm(sub3(f.pos[i], cs.wall.pos[j], D), D));
            sum += cs.tk.W(r) * ck.wall_Vol_ref[j];
        }
        ck.compression_sum[i] = sum;
        ck.compression[i] = std::max(sum, Real(1));
        f.rho[i] = ck.compression[i] * cs.rho0;
    }
}

// AdvectionStepSetup: fluid_time_step_ck.h:145-149
void ckAdvectionStepSetup(Case &cs)
{
    ckEnsureState(cs);
    Body &f = cs.fluid;
    for (size_t i = 0; i < f.n; ++i)
    {
        f.Vol[i] = f.mass[i] / f.rho[i];
        cs.ck.dpos[i] = V3();
    }
}

// UpdateParticlePosition: fluid_time_step_ck.h:173-176
void ckUpdateParticlePosition(Case &cs)
{
    Body &f = cs.fluid;
    for (size_t i = 0; i < f.n; ++i)
        for (int a = 0; a < cs.D; ++a)
            f.pos[i][a] += cs.ck.dpos[i][a];
}

// LinearCorrectionMatrix<Inner<WithUpdate>> + <Contact>: kernel_correction_ck.hpp:25-80,
// inverseTikhonov (vector_functions.h:199-203) with SqrtEps = 1e-8
void ckLinearCorrectionMatrix(Case &cs, Real alpha)
{
    ckEnsureState(cs);
    const int D = cs.D;
    Body &f = cs.fluid;
    CKState &ck = cs.ck;
#pragma omp parallel for schedule(static)
    for (long i = 0; i < (long)f.n; ++i)
    {
        M3 B;
        auto add = [&](const V3 &xj, Real Vj) {
            V3 r = sub3(f.pos[i], xj, D);
            Real dW = cs.tk.dW(std::sqrt(sqnorm(r, D)));
            V3 e = normalized(r, D);
            for (int a = 0; a < D; ++a)
                for (int b = 0; b < D; ++b)
                    B(a, b) -= r[a] * (dW * e[b] * Vj);
        };
        const Neighborhood &nb = cs.inner[i];
        for (size_t k = 0; k < nb.size(); ++k)
            add(f.pos[nb.j[k]], f.Vol[nb.j[k]]);
        const Neighborhood &nw = cs.contact[i];
        for (size_t k = 0; k < nw.size(); ++k)
            add(cs.wall.pos[nw.j[k]], cs.wall.Vol[nw.j[k]]);
        Real determinant = det(B, D);
        Real det_sqr = std::max(alpha - determinant, Real(0));
        // inverseTikhonov: (B^T B + eps I)^-1 B^T
        M3 BtB;
        for (int a = 0; a < D; ++a)
            for (int b = 0; b < D; ++b)
            {
                Real sum = 0;
                for (int c = 0; c < D; ++c)
                    sum += B(c, a) * B(c, b);
                BtB(a, b) = sum + (a == b ? 1.0e-8 : 0.0);
            }
        M3 Inv = inverse(BtB, D), T;
        for (int a = 0; a < D; ++a)
            for (int b = 0; b < D; ++b)
            {
                Real sum = 0;
                for (int c = 0; c < D; ++c)
                    sum += Inv(a, c) * B(b, c);
                T(a, b) = sum;
            }
        Real weight = determinant / (determinant + det_sqr);
        M3 R;
        for (int a = 0; a < D; ++a)
            for (int b = 0; b < D; ++b)
                R(a, b) = weight * T(a, b) + (1.0 - weight) * (a == b ? 1.0 : 0.0);
        ck.B[i] = R;
    }
}

// AcousticStep1stHalf<Inner<OneLevel, AcousticRiemannSolverCK, LinearCorrectionCK>> +
// <Contact<Wall, ...>>: acoustic_step_1st_half.hpp:40-190; RiemannSolver AverageP /
// DissipativeUJump: riemann_solver_ck.hpp:14-50
void ckAcousticStep1stHalf(Case &cs, Real dt)
{
    const int D = cs.D;
    Body &f = cs.fluid;
    CKState &ck = cs.ck;
    const Real Z = cs.rho0c0, inv_Zsum = 1.0 / (Z + Z);
#pragma omp parallel for schedule(static)
    for (long i = 0; i < (long)f.n; ++i)
    {
        ck.compression[i] += 0.5 * dt * ck.compression_rate[i];
        f.rho[i] = ck.compression[i] * cs.rho0;
        f.p[i] = cs.getPressure(f.rho[i]);
        for (int a = 0; a < D; ++a)
            ck.dpos[i][a] += f.vel[i][a] * dt * 0.5;
    }
#pragma omp parallel for schedule(static)
    for (long i = 0; i < (long)f.n; ++i)
    {
        V3 force_sum;
        Real dissipation = 0;
        const Neighborhood &nb = cs.inner[i];
        for (size_t k = 0; k < nb.size(); ++k)
        {
            UInt j = nb.j[k];
            V3 r = sub3(f.pos[i], f.pos[j], D);
            Real dWV = cs.tk.dW(std::sqrt(sqnorm(r, D))) * f.Vol[j];
            V3 e = normalized(r, D);
            // AverageP(B_j p_i, B_i p_j) = (Z_j B_j p_i + Z_i B_i p_j) / (Z_i + Z_j)
            V3 bj = mul(ck.B[j], e, D), bi = mul(ck.B[i], e, D);
            for (int a = 0; a < D; ++a)
                force_sum[a] -= inv_Zsum * (f.p[i] * Z * bj[a] + f.p[j] * Z * bi[a]) * 2.0 * dWV;
            dissipation += (f.p[i] - f.p[j]) * cs.inv_rho0c0_ave * dWV;
        }
        for (int a = 0; a < D; ++a)
            f.force[i][a] += force_sum[a] * f.Vol[i];
        ck.compression_rate[i] = dissipation * ck.compression[i];
        // wall contact
        V3 wforce;
        Real wdis = 0;
        const Neighborhood &nw = cs.contact[i];
        for (size_t k = 0; k < nw.size(); ++k)
        {
            UInt j = nw.j[k];
            V3 r = sub3(f.pos[i], cs.wall.pos[j], D);
            Real rij = std::sqrt(sqnorm(r, D));
            Real dWV = cs.tk.dW(rij) * cs.wall.Vol[j];
            V3 e = normalized(r, D);
            V3 acc;
            for (int a = 0; a < D; ++a)
                acc[a] = -(f.force_prior[i][a] / f.mass[i] - cs.wall.acc_ave[j][a]);
            Real face = dotd(acc, e, D);
            Real p_wall = f.p[i] + f.rho[i] * rij * std::max(Real(0), face);
            V3 be = mul(ck.B[i], e, D);
            for (int a = 0; a < D; ++a)
                wforce[a] -= (f.p[i] + p_wall) * be[a] * dWV;
            wdis += (f.p[i] - p_wall) * cs.inv_rho0c0_ave * dWV;
        }
        for (int a = 0; a < D; ++a)
            f.force[i][a] += wforce[a] * f.Vol[i];
        ck.compression_rate[i] += wdis * ck.compression[i];
    }
#pragma omp parallel for schedule(static)
    for (long i = 0; i < (long)f.n; ++i)
        for (int a = 0; a < D; ++a)
            f.vel[i][a] += (f.force_prior[i][a] + f.force[i][a]) / f.mass[i] * dt;
}

// AcousticStep2ndHalf<Inner<...>> + <Contact<Wall, ...>>: acoustic_step_2nd_half.hpp:20-120;
// AverageV / DissipativePJump: riemann_solver_ck.hpp:20-45
void ckAcousticStep2ndHalf(Case &cs, Real dt)
{
    const int D = cs.D;
    Body &f = cs.fluid;
    CKState &ck = cs.ck;
    const Real Z = cs.rho0c0, inv_Zsum = 1.0 / (Z + Z);
#pragma omp parallel for schedule(static)
    for (long i = 0; i < (long)f.n; ++i)
        for (int a = 0; a < D; ++a)
            ck.dpos[i][a] += f.vel[i][a] * dt * 0.5;
#pragma omp parallel for schedule(static)
    for (long i = 0; i < (long)f.n; ++i)
    {
        Real divergence = 0;
        V3 p_dis;
        const Neighborhood &nb = cs.inner[i];
        for (size_t k = 0; k < nb.size(); ++k)
        {
            UInt j = nb.j[k];
            V3 r = sub3(f.pos[i], f.pos[j], D);
            Real dWV = cs.tk.dW(std::sqrt(sqnorm(r, D))) * f.Vol[j];
            V3 e = normalized(r, D);
            V3 be = mul(ck.B[i], e, D), dv;
            for (int a = 0; a < D; ++a)
            {
                Real v_ave = (f.vel[i][a] * Z + f.vel[j][a] * Z) * inv_Zsum;
                dv[a] = f.vel[i][a] - v_ave;
            }
            divergence += 2.0 * dotd(dv, be, D) * dWV;
            Real u_jump = dotd(sub3(f.vel[i], f.vel[j], D), e, D);
            Real pj = cs.PJump(u_jump) * dWV;
            for (int a = 0; a < D; ++a)
                p_dis[a] += pj * e[a];
        }
        ck.compression_rate[i] += divergence * ck.compression[i];
        for (int a = 0; a < D; ++a)
            f.force[i][a] = p_dis[a] * f.Vol[i];
        Real wdiv = 0;
        V3 wdis;
        const Neighborhood &nw = cs.contact[i];
        for (size_t k = 0; k < nw.size(); ++k)
        {
            UInt j = nw.j[k];
            V3 r = sub3(f.pos[i], cs.wall.pos[j], D);
            Real dWV = cs.tk.dW(std::sqrt(sqnorm(r, D))) * cs.wall.Vol[j];
            V3 e = normalized(r, D);
            V3 vel_diff, be = mul(ck.B[i], e, D);
            for (int a = 0; a < D; ++a)
                vel_diff[a] = 2.0 * (f.vel[i][a] - cs.wall.vel_ave[j][a]);
            wdiv += dotd(vel_diff, be, D) * dWV;
            Real en = dotd(e, cs.wall.normal[j], D);
            Real sgn = en > 0 ? 1.0 : (en < 0 ? -1.0 : 0.0);
            V3 n_star;
            for (int a = 0; a < D; ++a)
                n_star[a] = sgn * cs.wall.normal[j][a];
            Real pj = cs.PJump(dotd(vel_diff, n_star, D)) * dWV;
            for (int a = 0; a < D; ++a)
                wdis[a] += pj * n_star[a];
        }
        ck.compression_rate[i] += wdiv * ck.compression[i];
        for (int a = 0; a < D; ++a)
            f.force[i][a] += wdis[a] * f.Vol[i];
    }
#pragma omp parallel for schedule(static)
    for (long i = 0; i < (long)f.n; ++i)
    {
        ck.compression[i] += 0.5 * dt * ck.compression_rate[i];
        f.rho[i] = ck.compression[i] * cs.rho0;
    }
}

// AcousticTimeStepCK: fluid_time_step_ck.hpp:25-57 (sound speed c0 for this fluid)
Real ckAcousticTimeStep(const Case &cs)
{
    const Body &f = cs.fluid;
    Real m = 0;
    for (size_t i = 0; i < f.n; ++i)
    {
        V3 F;
        for (int a = 0; a < cs.D; ++a)
            F[a] = f.force[i][a] + f.force_prior[i][a];
        Real acc_scale = std::sqrt(4.0 * cs.h_min * std::sqrt(sqnorm(F, cs.D)) / f.mass[i]);
        m = std::max(m, std::max(cs.c0 + std::sqrt(sqnorm(f.vel[i], cs.D)), acc_scale));
    }
    return cs.acoustic_cfl * cs.h_min / (m + TinyReal);
}

// AdvectionTimeStepCK: fluid_time_step_ck.cpp:16-20, fluid_time_step_ck.h:106-109
Real ckAdvectionTimeStep(const Case &cs)
{
    const Body &f = cs.fluid;
    Real m = 0;
    for (size_t i = 0; i < f.n; ++i)
        m = std::max(m, sqnorm(f.vel[i], cs.D));
    return cs.advection_cfl * cs.h_min / (std::max(std::sqrt(m), cs.U_ref) + TinyReal);
}

// The observer pressure through the tabulated kernel with the current fluid volumes
// (Interpolation<Contact<Real>>: interpolation_dynamics.hpp:46-60)
void ckObservePressure(Case &cs)
{
    Body &o = cs.observer;
    for (size_t i = 0; i < o.n; ++i)
    {
        Real q = 0, ttl = 0;
        const Neighborhood &nb = cs.obs[i];
        for (size_t n = 0; n < nb.size(); ++n)
        {
            UInt j = nb.j[n];
            Real r = std::sqrt(sqnorm(sub3(o.pos[i], cs.fluid.pos[j], cs.D), cs.D));
            Real w = cs.tk.W(r) * cs.fluid.Vol[j];
            q += w * cs.fluid.p[j];
            ttl += w;
        }
        o.observed[i] = q / (ttl + TinyReal);
    }
}

// Set-up part of dambreak_sycl.cpp:138-169: the advection interval from the initial state,
// then density regularization, advection-step set-up and correction matrices.
void ckInitialize(Case &cs)
{
    ckEnsureState(cs);
    cs.ck.present_time = 0;
    cs.ck.interval = ckAdvectionTimeStep(cs);
    cs.ck.advection_steps = 0;
    ckDensityRegularization(cs);
    ckAdvectionStepSetup(cs);
    ckLinearCorrectionMatrix(cs, 0.5);
}

// One pass of the dambreak_sycl.cpp:181-198 loop body up to the advection trigger:
// acoustic dt, both halves, and on trigger the new interval and the position update.
// Returns 1 when an advection step is due (the caller then observes and calls
// ckConfiguration).
int ckAcousticStep(Case &cs, Real *physical_time)
{
    Real dt = ckAcousticTimeStep(cs);
    *physical_time += dt;
    cs.ck.present_time += dt;
    ckAcousticStep1stHalf(cs, dt);
    ckAcousticStep2ndHalf(cs, dt);
    if (cs.ck.present_time > cs.ck.interval)
    {
        cs.ck.present_time = 0;
        cs.ck.interval = ckAdvectionTimeStep(cs);
        cs.ck.advection_steps++;
        ckUpdateParticlePosition(cs);
        return 1;
    }
    return 0;
}

// FreeSurfaceIndicationCK<Inner<WithUpdate>, Contact<>> (surface_indication_ck.hpp:49-150;
// threshold 0.75 d, h the reference smoothing length): inner interaction with the
// spatial-temporal rule, contact interaction, then the update over all particles.
void ckFreeSurfaceIndication(Case &cs)
{
    ckEnsureState(cs);
    const int D = cs.D;
    Body &f = cs.fluid;
    CKState &ck = cs.ck;
    const Real thr = 0.75 * D;
#pragma omp parallel for schedule(static)
    for (long i = 0; i < (long)f.n; ++i)
    {
        Real pos_div = 0.0;
        const Neighborhood &nb = cs.inner[i];
        for (size_t k = 0; k < nb.size(); ++k)
        {
            UInt j = nb.j[k];
            Real r = std::sqrt(sqnorm(sub3(f.pos[i], f.pos[j], D), D));
            pos_div -= cs.tk.dW(r) * f.Vol[j] * r;
        }
        if (pos_div < thr && ck.prev_indicator[i] != 1)
        {
            bool near_previous = false;
            for (size_t k = 0; k < nb.size(); ++k)
                if (ck.prev_indicator[nb.j[k]] == 1)
                {
                    near_previous = true;
                    break;
                }
            if (!near_previous)
                pos_div = 2.0 * thr;
        }
        ck.pos_div[i] = pos_div;
    }
#pragma omp parallel for schedule(static)
    for (long i = 0; i < (long)f.n; ++i)
    {
        Real pos_div = 0.0;
        const Neighborhood &nw = cs.contact[i];
        for (size_t k = 0; k < nw.size(); ++k)
        {
            UInt j = nw.j[k];
            Real r = std::sqrt(sqnorm(sub3(f.pos[i], cs.wall.pos[j], D), D));
            pos_div -= cs.tk.dW(r) * cs.wall.Vol[j] * r;
        }
        ck.pos_div[i] += pos_div;
    }
#pragma omp parallel for schedule(static)
    for (long i = 0; i < (long)f.n; ++i)
    {
        int ind = 1;
        if (ck.pos_div[i] > thr)
        {
            bool very_near = false;
            const Neighborhood &nb = cs.inner[i];
            for (size_t k = 0; k < nb.size(); ++k)
            {
                UInt j = nb.j[k];
                Real r = std::sqrt(sqnorm(sub3(f.pos[i], f.pos[j], D), D));
                if (ck.pos_div[j] < thr && r < cs.h)
                {
                    very_near = true;
                    break;
                }
            }
            if (!very_near)
                ind = 0;
        }
        ck.indicator[i] = ind;
    }
    ck.prev_indicator = ck.indicator;
}

// One advection step of tests_sycl/3d_examples/test_3d_dambreak_sycl/dambreak.cpp:186-224:
// compression summation + regularization, advection-step set-up, advection dt,
// free-surface indication, correction matrices, the acoustic sub-steps (acoustic dt
// first), the position update, cell list and relations (the Morton re-sort of the driver
// only permutes particles and is not applied).  Returns the number of sub-steps.
int ckNestedAdvectionStep(Case &cs, Real *physical_time, Real *advection_dt)
{
    ckDensityRegularization(cs);
    ckAdvectionStepSetup(cs);
    Real Dt = ckAdvectionTimeStep(cs);
    ckFreeSurfaceIndication(cs);
    ckLinearCorrectionMatrix(cs, 0.5);
    Real relaxation = 0;
    int sub = 0;
    while (relaxation < Dt)
    {
        Real dt = ckAcousticTimeStep(cs);
        ckAcousticStep1stHalf(cs, dt);
        ckAcousticStep2ndHalf(cs, dt);
        relaxation += dt;
        *physical_time += dt;
        ++sub;
    }
    ckUpdateParticlePosition(cs);
    cs.ck.advection_steps++;
    cs.fluid_cells.update(cs.fluid, &cs.periodic);
    updateConfiguration(cs);
    if (advection_dt)
        *advection_dt = Dt;
    return sub;
}

// dambreak_sycl.cpp:230-245: cell list, relations, density regularization, advection-step
// set-up, correction matrices (the Morton re-sort of the driver only permutes particles and
// is not applied).
void ckConfiguration(Case &cs)
{
    cs.fluid_cells.update(cs.fluid, &cs.periodic);
    updateConfiguration(cs);
    ckDensityRegularization(cs);
    ckAdvectionStepSetup(cs);
    ckLinearCorrectionMatrix(cs, 0.5);
}

//------------------------------------------------------------------------------
// Taylor-Green vortex (tests/2d_examples/test_2d_taylor_green/taylor_green.cpp)
//------------------------------------------------------------------------------
// ViscousForce<Inner<>, FixedViscosity, NoKernelCorrection> (viscous_dynamics.hpp:25-53)
// with the ForcePrior update (force_prior.hpp:22-26)
void viscousForceInner(Case &cs)
{
    const int D = cs.D;
    Body &f = cs.fluid;
    cs.viscous_force.resize(f.n);
    cs.prev_viscous.resize(f.n);
#pragma omp parallel for schedule(static)
    for (long i = 0; i < (long)f.n; ++i)
    {
        V3 force;
        const Neighborhood &nb = cs.inner[i];
        for (size_t n = 0; n < nb.size(); ++n)
        {
            UInt j = nb.j[n];
            const V3 &e = nb.e[n];
            Real denom = nb.r[n] + 0.01 * cs.h;
            Real ee = 0;
            for (int a = 0; a < D; ++a)
                ee += e[a] * (2.0 * e[a]); // e . ((B_i + B_j) e) with B = 1
            for (int a = 0; a < D; ++a)
            {
                Real vd = (f.vel[i][a] - f.vel[j][a]) / denom;
                force[a] += ee * cs.mu * vd * nb.dW[n] * f.Vol[j];
            }
        }
        for (int a = 0; a < D; ++a)
            cs.viscous_force[i][a] = force[a] * f.Vol[i];
    }
    for (size_t i = 0; i < f.n; ++i)
        for (int a = 0; a < D; ++a)
        {
            f.force_prior[i][a] += cs.viscous_force[i][a] - cs.prev_viscous[i][a];
            cs.prev_viscous[i][a] = cs.viscous_force[i][a];
        }
}

// TransportVelocityCorrection<Inner<SPHAdaptation, TruncatedLinear>> with coefficient 0.2
// and the default limiter slope 100 (transport_velocity_correction.hpp:32-66,
// common_functors.h:82-94)
void transportVelocityCorrectionInner(Case &cs, Real coefficient)
{
    const int D = cs.D;
    Body &f = cs.fluid;
    std::vector<V3> inc(f.n);
#pragma omp parallel for schedule(static)
    for (long i = 0; i < (long)f.n; ++i)
    {
        V3 s;
        const Neighborhood &nb = cs.inner[i];
        for (size_t n = 0; n < nb.size(); ++n)
            for (int a = 0; a < D; ++a)
                s[a] -= (1.0 + 1.0) * nb.dW[n] * f.Vol[nb.j[n]] * nb.e[n][a];
        inc[i] = s;
    }
    Real h2 = cs.h * cs.h, scaling = coefficient * h2;
    for (size_t i = 0; i < f.n; ++i)
    {
        Real sq = sqnorm(inc[i], D);
        Real lim = std::min(100.0 * (h2 * sq), Real(1));
        for (int a = 0; a < D; ++a)
            f.pos[i][a] += scaling * lim * inc[i][a] * 1.0 * 1.0;
    }
}

// PeriodicBounding::checkLowerBound / checkUpperBound (domain_bounding.h:103-113)
void periodicBounding(Case &cs)
{
    Body &f = cs.fluid;
    for (int a = 0; a < cs.D; ++a)
    {
        if (!cs.periodic.on[a])
            continue;
        Real L = cs.periodic.upper[a] - cs.periodic.lower[a];
        for (size_t i = 0; i < f.n; ++i)
        {
            if (f.pos[i][a] < cs.periodic.lower[a])
                f.pos[i][a] += L;
            if (f.pos[i][a] > cs.periodic.upper[a])
                f.pos[i][a] -= L;
        }
    }
}

// One pass of the taylor_green.cpp:133-164 advection loop; returns the acoustic sub-steps.
int tgvAdvectionStep(Case &cs, Real *physical_time, Real *advection_dt)
{
    Real Dt = advectionTimeStep(cs);
    densitySummation(cs);
    viscousForceInner(cs);
    transportVelocityCorrectionInner(cs, 0.2);
    Real relaxation = 0;
    int sub = 0;
    while (relaxation < Dt)
    {
        Real dt = std::min(acousticTimeStep(cs), Dt);
        relaxation += dt;
        integration1stHalf(cs, dt);
        integration2ndHalf(cs, dt);
        *physical_time += dt;
        ++sub;
    }
    periodicBounding(cs);
    cs.fluid_cells.update(cs.fluid, &cs.periodic);
    updateConfiguration(cs);
    if (advection_dt)
        *advection_dt = Dt;
    return sub;
}

Real totalKineticEnergy(const Case &cs)
{
    const Body &f = cs.fluid;
    Real e = 0;
    for (size_t i = 0; i < f.n; ++i)
        e += 0.5 * f.mass[i] * sqnorm(f.vel[i], cs.D);
    return e;
}

Real maximumSpeed(const Case &cs)
{
    const Body &f = cs.fluid;
    Real m = 0;
    for (size_t i = 0; i < f.n; ++i)
        m = std::max(m, std::sqrt(sqnorm(f.vel[i], cs.D)));
    return m;
}

// Lattice generation: particle_generator_lattice_{2d,3d}.cpp:12-23
template <class Contain>
std::vector<V3> lattice(int D, const V3 &lo, const V3 &up, Real dp, Contain contain)
{
    Mesh m = Mesh::fromBounds(D, lo, up, dp, 0);
    std::vector<V3> out;
    int c[3] = {0, 0, 0};
    int n2 = D == 3 ? m.all_cells[2] : 1;
    for (c[0] = 0; c[0] < m.all_cells[0]; ++c[0])
        for (c[1] = 0; c[1] < m.all_cells[1]; ++c[1])
            for (c[2] = 0; c[2] < n2; ++c[2])
            {
                V3 p = m.cellCentre(c);
                if (contain(p))
                    out.push_back(p);
            }
    return out;
}
} // namespace orc

using namespace orc;

extern "C"
{
    // Case description shared with the Python side (ctypes.Structure of the same layout).
    struct OrcCaseDesc
    {
        int dim;
        int n_observers;
        double sys_lower[3], sys_upper[3];
        double dp, h_ratio;
        double water_center[3], water_halfsize[3];
        double outer_center[3], outer_halfsize[3];
        double inner_center[3], inner_halfsize[3];
        double rho0, c0, U_ref;
        double gravity[3];
        double observers[16][3];
    };

    void orc_set_num_threads(int n)
    {
#ifdef _OPENMP
        if (n > 0)
            omp_set_num_threads(n);
#endif
    }
    int orc_get_max_threads()
    {
#ifdef _OPENMP
        return omp_get_max_threads();
#else
        return 1;
#endif
    }

    // Builds the bodies of a dam-break case: Dambreak.cpp:56-73,124-127 (lattice particles,
    // Mass = rho0 Vol, Density = rho0, wall normals, gravity prior force, cell lists and
    // initial configurations).
    void *orc_case_create(const OrcCaseDesc *d)
    {
        Case *cs = new Case();
        const int D = d->dim;
        cs->D = D;
        cs->dp = d->dp;
        cs->h = d->h_ratio * d->dp;
        cs->h_min = cs->h;
        cs->kernel = Kernel(D, cs->h);
        cs->tk = TabKernel(D, cs->h);
        cs->rho0 = d->rho0;
        cs->c0 = d->c0;
        cs->U_ref = d->U_ref;
        cs->p0 = d->rho0 * d->c0 * d->c0;
        for (int a = 0; a < 3; ++a)
        {
            cs->gravity[a] = d->gravity[a];
            cs->sys_lo[a] = d->sys_lower[a];
            cs->sys_up[a] = d->sys_upper[a];
            cs->water_box.c[a] = d->water_center[a];
            cs->water_box.hs[a] = d->water_halfsize[a];
            cs->wall_shape.outer.c[a] = d->outer_center[a];
            cs->wall_shape.outer.hs[a] = d->outer_halfsize[a];
            cs->wall_shape.inner.c[a] = d->inner_center[a];
            cs->wall_shape.inner.hs[a] = d->inner_halfsize[a];
        }
        cs->sigma0 = latticeNumberDensity(cs->kernel, cs->dp);
        cs->inv_sigma0 = 1.0 / cs->sigma0;
        cs->W0 = cs->kernel.W0();
        Real Z = cs->rho0 * cs->c0;
        Real inv_sum = 1.0 / (Z + Z);
        cs->rho0c0 = Z;
        cs->inv_rho0c0_ave = (Z + Z) / (std::pow(Z, 2.0) + std::pow(Z, 2.0));
        cs->rho0c0_geo_ave = 2.0 * Z * Z * inv_sum;
        cs->inv_c0_ave = 0.5 * (cs->rho0 + cs->rho0) * cs->inv_rho0c0_ave;

        Real vol = D == 2 ? cs->dp * cs->dp : cs->dp * cs->dp * cs->dp;
        auto fpos = lattice(D, cs->sys_lo, cs->sys_up, cs->dp, [&](const V3 &p) { return cs->water_box.contain(p, D); });
        auto wpos = lattice(D, cs->sys_lo, cs->sys_up, cs->dp, [&](const V3 &p) { return cs->wall_shape.contain(p, D); });
        cs->fluid.resize(fpos.size());
        cs->wall.resize(wpos.size());
        for (size_t i = 0; i < fpos.size(); ++i)
        {
            cs->fluid.pos[i] = fpos[i];
            cs->fluid.Vol[i] = vol;
            cs->fluid.rho[i] = cs->rho0;
            cs->fluid.mass[i] = cs->rho0 * vol;
        }
        for (size_t i = 0; i < wpos.size(); ++i)
        {
            cs->wall.pos[i] = wpos[i];
            cs->wall.Vol[i] = vol;
            cs->wall.rho[i] = cs->wall_rho0;
            cs->wall.mass[i] = cs->wall_rho0 * vol;
            cs->wall.normal[i] = cs->wall_shape.normal(wpos[i], D);
        }
        cs->observer.resize(size_t(d->n_observers));
        for (int k = 0; k < d->n_observers; ++k)
            for (int a = 0; a < 3; ++a)
                cs->observer.pos[k][a] = d->observers[k][a];
        // GravityForce (force_prior.hpp:35-41, BaseForcePrior::update)
        for (size_t i = 0; i < cs->fluid.n; ++i)
            for (int a = 0; a < D; ++a)
            {
                Real g = cs->fluid.mass[i] * cs->gravity[a];
                cs->fluid.force_prior[i][a] += g - cs->fluid.prev_gravity[i][a];
                cs->fluid.prev_gravity[i][a] = g;
            }
        // cell linked lists (SPHAdaptation::createCellLinkedList, buffer width 2)
        Mesh m = Mesh::fromBounds(D, cs->sys_lo, cs->sys_up, cs->kernel.rc, 2);
        cs->fluid_cells.mesh = m;
        cs->wall_cells.mesh = m;
        cs->sort_mesh = m;
        // SearchDepthContact: base_body_relation.cpp:10-16
        cs->contact_depth = 1 + int(std::floor(cs->kernel.rc * (1.0 / m.gs)));
        cs->fluid_cells.update(cs->fluid, &cs->periodic);
        cs->wall_cells.update(cs->wall);
        updateConfiguration(*cs);
        updateObserverConfiguration(*cs);
        return cs;
    }
    void orc_case_destroy(void *h) { delete static_cast<Case *>(h); }

    static Body *body_of(Case *cs, int b) { return b == 0 ? &cs->fluid : (b == 1 ? &cs->wall : &cs->observer); }

    size_t orc_num_particles(void *h, int b) { return body_of(static_cast<Case *>(h), b)->n; }

    // Resizes a body to n particles with zeroed variables and ids 0..n-1 (the caller sets
    // every variable it needs with orc_set, then rebuilds cell lists and configurations):
    // lets a test hold an arbitrary particle set, e.g. one rank's slab plus ghosts.
    void orc_body_resize(void *h, int b, size_t n)
    {
        Case *cs = static_cast<Case *>(h);
        body_of(cs, b)->resize(n);
        cs->ck.ready = false;
        if (b == 0)
        {
            cs->inner.clear();
            cs->contact.clear();
        }
        if (b == 2)
            cs->obs.clear();
    }

    // Scalar case constants: 0 sigma0, 1 W0, 2 h, 3 rc, 4 contact depth, 5 inv_rho0c0_ave,
    // 6 rho0c0_geo_ave, 7 inv_c0_ave, 8 p0, 9 factor_W, 10 factor_dW
    double orc_constant(void *h, int which)
    {
        Case *cs = static_cast<Case *>(h);
        switch (which)
        {
        case 0: return cs->sigma0;
        case 1: return cs->W0;
        case 2: return cs->h;
        case 3: return cs->kernel.rc;
        case 4: return cs->contact_depth;
        case 5: return cs->inv_rho0c0_ave;
        case 6: return cs->rho0c0_geo_ave;
        case 7: return cs->inv_c0_ave;
        case 8: return cs->p0;
        case 9: return cs->kernel.factor_W;
        case 10: return cs->kernel.factor_dW;
        }
        return 0;
    }

    static int vec_field(Body *b, const char *name, std::vector<V3> **out)
    {
        std::string s(name);
        if (s == "Position") *out = &b->pos;
        else if (s == "Velocity") *out = &b->vel;
        else if (s == "Force") *out = &b->force;
        else if (s == "ForcePrior") *out = &b->force_prior;
        else if (s == "NormalDirection") *out = &b->normal;
        else if (s == "Acceleration") *out = &b->acc_ave;
        else if (s == "WallVelocity") *out = &b->vel_ave;
        else return 0;
        return 1;
    }
    static int scalar_field(Body *b, const char *name, std::vector<Real> **out)
    {
        std::string s(name);
        if (s == "Density") *out = &b->rho;
        else if (s == "Pressure") *out = &b->p;
        else if (s == "DensityChangeRate") *out = &b->drho_dt;
        else if (s == "Mass") *out = &b->mass;
        else if (s == "VolumetricMeasure") *out = &b->Vol;
        else if (s == "DensitySummation") *out = &b->rho_sum;
        else if (s == "Observed") *out = &b->observed;
        else return 0;
        return 1;
    }

    // Copies a field out as AoS (n x dim for vectors).  Returns components or 0 if unknown.
    int orc_get(void *h, int b, const char *name, double *out)
    {
        Case *cs = static_cast<Case *>(h);
        Body *bd = body_of(cs, b);
        std::vector<V3> *vf;
        std::vector<Real> *sf;
        if (vec_field(bd, name, &vf))
        {
            for (size_t i = 0; i < bd->n; ++i)
                for (int a = 0; a < cs->D; ++a)
                    out[i * cs->D + a] = (*vf)[i][a];
            return cs->D;
        }
        if (scalar_field(bd, name, &sf))
        {
            std::copy(sf->begin(), sf->end(), out);
            return 1;
        }
        return 0;
    }
    int orc_set(void *h, int b, const char *name, const double *in)
    {
        Case *cs = static_cast<Case *>(h);
        Body *bd = body_of(cs, b);
        std::vector<V3> *vf;
        std::vector<Real> *sf;
        if (vec_field(bd, name, &vf))
        {
            for (size_t i = 0; i < bd->n; ++i)
                for (int a = 0; a < cs->D; ++a)
                    (*vf)[i][a] = in[i * cs->D + a];
            return cs->D;
        }
        if (scalar_field(bd, name, &sf))
        {
            std::copy(in, in + bd->n, sf->begin());
            return 1;
        }
        return 0;
    }
    int orc_get_ids(void *h, int b, uint32_t *original_id, uint32_t *sorted_id)
    {
        Body *bd = body_of(static_cast<Case *>(h), b);
        if (original_id)
            std::copy(bd->original_id.begin(), bd->original_id.end(), original_id);
        if (sorted_id)
            std::copy(bd->sorted_id.begin(), bd->sorted_id.end(), sorted_id);
        return 0;
    }

    // Mesh of the cell linked list: lower[3], gs, all_cells[3]
    void orc_mesh(void *h, double *lower, double *gs, int *all_cells)
    {
        Case *cs = static_cast<Case *>(h);
        const Mesh &m = cs->fluid_cells.mesh;
        for (int a = 0; a < 3; ++a)
        {
            lower[a] = m.lower[a];
            all_cells[a] = a < cs->D ? m.all_cells[a] : 1;
        }
        *gs = m.gs;
    }
    size_t orc_num_cells(void *h) { return static_cast<Case *>(h)->fluid_cells.mesh.numCells(); }

    void orc_update_cell_linked_list(void *h, int b)
    {
        Case *cs = static_cast<Case *>(h);
        if (b == 0)
            cs->fluid_cells.update(cs->fluid, &cs->periodic);
        else
            cs->wall_cells.update(cs->wall);
    }
    void orc_get_cell_list(void *h, int b, uint32_t *cell_offset, uint32_t *particle_index)
    {
        Case *cs = static_cast<Case *>(h);
        CellList &cl = b == 0 ? cs->fluid_cells : cs->wall_cells;
        std::copy(cl.cell_offset.begin(), cl.cell_offset.end(), cell_offset);
        Body *bd = body_of(cs, b);
        std::copy(cl.particle_index.begin(), cl.particle_index.begin() + bd->n, particle_index);
    }
    void orc_update_configuration(void *h) { updateConfiguration(*static_cast<Case *>(h)); }
    void orc_update_observer_configuration(void *h) { updateObserverConfiguration(*static_cast<Case *>(h)); }

    // Neighbour lists (0 inner, 1 wall contact, 2 observer contact): counts[n_src]; the
    // other arrays are the concatenated lists (total = sum counts), any may be null.
    size_t orc_get_neighbors(void *h, int which, uint32_t *counts, uint32_t *j, double *W, double *dW, double *r,
                             double *e)
    {
        Case *cs = static_cast<Case *>(h);
        std::vector<Neighborhood> &cfg = which == 0 ? cs->inner : (which == 1 ? cs->contact : cs->obs);
        size_t total = 0;
        for (size_t i = 0; i < cfg.size(); ++i)
        {
            const Neighborhood &nb = cfg[i];
            if (counts)
                counts[i] = UInt(nb.size());
            for (size_t n = 0; n < nb.size(); ++n, ++total)
            {
                if (j) j[total] = nb.j[n];
                if (W) W[total] = nb.W[n];
                if (dW) dW[total] = nb.dW[n];
                if (r) r[total] = nb.r[n];
                if (e)
                    for (int a = 0; a < cs->D; ++a)
                        e[total * cs->D + a] = nb.e[n][a];
            }
        }
        return total;
    }

    void orc_density_summation(void *h) { densitySummation(*static_cast<Case *>(h)); }
    void orc_integration_1st_half(void *h, double dt) { integration1stHalf(*static_cast<Case *>(h), dt); }
    void orc_integration_2nd_half(void *h, double dt) { integration2ndHalf(*static_cast<Case *>(h), dt); }
    double orc_acoustic_time_step(void *h) { return acousticTimeStep(*static_cast<Case *>(h)); }
    double orc_advection_time_step(void *h) { return advectionTimeStep(*static_cast<Case *>(h)); }
    void orc_particle_sorting(void *h) { particleSorting(*static_cast<Case *>(h)); }
    void orc_observe_pressure(void *h, double *out)
    {
        Case *cs = static_cast<Case *>(h);
        observePressure(*cs);
        std::copy(cs->observer.observed.begin(), cs->observer.observed.end(), out);
    }
    double orc_total_mechanical_energy(void *h) { return totalMechanicalEnergy(*static_cast<Case *>(h)); }
    double orc_upper_front(void *h, int axis, const double *lo, const double *up)
    {
        Case *cs = static_cast<Case *>(h);
        V3 l, u;
        for (int a = 0; a < 3; ++a)
        {
            l[a] = lo[a];
            u[a] = up[a];
        }
        return upperFront(*cs, axis, l, u);
    }
    double orc_lattice_number_density(int dim, double h, double dp) { return latticeNumberDensity(Kernel(dim, h), dp); }

    // Taylor-Green vortex: a periodic box [0, L]^dim of lattice particles at rest density,
    // velocity kind 0 the 2D taylor_green.cpp field (-cos 2pi x sin 2pi y, sin 2pi x cos 2pi y)
    // on L = 1, kind 1 the 3D field (sin x cos y cos z, -cos x sin y cos z, 0) on L = 2 pi;
    // mu = rho0 U L / Re, the Riemann dissipation of the 2nd half off (NoRiemannSolver),
    // DensitySummation<Inner<>>, AdvectionViscousTimeStep reference speed max(U, mu/rho0/h).
    struct OrcTGVDesc
    {
        int dim, velocity_kind;
        double L, dp, h_ratio, rho0, U, c0, Re;
    };
    void *orc_tgv_create(const OrcTGVDesc *d)
    {
        Case *cs = new Case();
        const int D = d->dim;
        cs->D = D;
        cs->dp = d->dp;
        cs->h = d->h_ratio * d->dp;
        cs->h_min = cs->h;
        cs->kernel = Kernel(D, cs->h);
        cs->tk = TabKernel(D, cs->h);
        cs->rho0 = d->rho0;
        cs->c0 = d->c0;
        cs->p0 = d->rho0 * d->c0 * d->c0;
        cs->mu = d->rho0 * d->U * d->L / d->Re;
        cs->U_ref = std::max(d->U, cs->mu / d->rho0 / cs->h);
        cs->limiter_slope = 0.0; // NoRiemannSolver in the 2nd half: DissipativePJump = 0
        cs->free_surface = false;
        for (int a = 0; a < 3; ++a)
        {
            cs->sys_lo[a] = 0.0;
            cs->sys_up[a] = a < D ? d->L : 0.0;
            cs->periodic.on[a] = a < D;
            cs->periodic.lower[a] = 0.0;
            cs->periodic.upper[a] = a < D ? d->L : 0.0;
        }
        cs->periodic.rc = cs->kernel.rc;
        cs->sigma0 = latticeNumberDensity(cs->kernel, cs->dp);
        cs->inv_sigma0 = 1.0 / cs->sigma0;
        cs->W0 = cs->kernel.W0();
        Real Z = cs->rho0 * cs->c0;
        Real inv_sum = 1.0 / (Z + Z);
        cs->rho0c0 = Z;
        cs->inv_rho0c0_ave = (Z + Z) / (std::pow(Z, 2.0) + std::pow(Z, 2.0));
        cs->rho0c0_geo_ave = 2.0 * Z * Z * inv_sum;
        cs->inv_c0_ave = 0.5 * (cs->rho0 + cs->rho0) * cs->inv_rho0c0_ave;
        Real vol = D == 2 ? cs->dp * cs->dp : cs->dp * cs->dp * cs->dp;
        auto fpos = lattice(D, cs->sys_lo, cs->sys_up, cs->dp, [&](const V3 &) { return true; });
        cs->fluid.resize(fpos.size());
        cs->wall.resize(0);
        cs->observer.resize(0);
        for (size_t i = 0; i < fpos.size(); ++i)
        {
            const V3 &x = fpos[i];
            cs->fluid.pos[i] = x;
            cs->fluid.Vol[i] = vol;
            cs->fluid.rho[i] = cs->rho0;
            cs->fluid.mass[i] = cs->rho0 * vol;
            V3 &v = cs->fluid.vel[i];
            if (d->velocity_kind == 0)
            {
                v[0] = -std::cos(2.0 * Pi * x[0]) * std::sin(2.0 * Pi * x[1]);
                v[1] = std::sin(2.0 * Pi * x[0]) * std::cos(2.0 * Pi * x[1]);
            }
            else
            {
                v[0] = std::sin(x[0]) * std::cos(x[1]) * std::cos(x[2]);
                v[1] = -std::cos(x[0]) * std::sin(x[1]) * std::cos(x[2]);
                v[2] = 0.0;
            }
        }
        Mesh m = Mesh::fromBounds(D, cs->sys_lo, cs->sys_up, cs->kernel.rc, 2);
        cs->fluid_cells.mesh = m;
        cs->wall_cells.mesh = m;
        cs->sort_mesh = m;
        cs->contact_depth = 1 + int(std::floor(cs->kernel.rc * (1.0 / m.gs)));
        cs->fluid_cells.update(cs->fluid, &cs->periodic);
        cs->wall_cells.update(cs->wall);
        updateConfiguration(*cs);
        return cs;
    }
    int orc_tgv_advection_step(void *h, double *physical_time, double *advection_dt)
    {
        return tgvAdvectionStep(*static_cast<Case *>(h), physical_time, advection_dt);
    }
    double orc_total_kinetic_energy(void *h) { return totalKineticEnergy(*static_cast<Case *>(h)); }
    double orc_maximum_speed(void *h) { return maximumSpeed(*static_cast<Case *>(h)); }
    size_t orc_cell_entries(void *h, int b)
    {
        Case *cs = static_cast<Case *>(h);
        return (b == 0 ? cs->fluid_cells : cs->wall_cells).entry_pos.size();
    }

    // CK numerics (the tests_sycl dam-break drivers)
    double orc_ck_kernel(void *h, int which, double r)
    {
        Case *cs = static_cast<Case *>(h);
        return which == 0 ? cs->tk.W(r) : (which == 1 ? cs->tk.dW(r) : cs->tk.W0());
    }
    void orc_ck_initialize(void *h) { ckInitialize(*static_cast<Case *>(h)); }
    int orc_ck_acoustic_step(void *h, double *physical_time)
    {
        return ckAcousticStep(*static_cast<Case *>(h), physical_time);
    }
    void orc_ck_configuration(void *h) { ckConfiguration(*static_cast<Case *>(h)); }
    void orc_ck_free_surface_indication(void *h) { ckFreeSurfaceIndication(*static_cast<Case *>(h)); }
    int orc_ck_nested_advection_step(void *h, double *physical_time, double *advection_dt)
    {
        return ckNestedAdvectionStep(*static_cast<Case *>(h), physical_time, advection_dt);
    }
    void orc_ck_density_regularization(void *h) { ckDensityRegularization(*static_cast<Case *>(h)); }
    void orc_ck_advection_step_setup(void *h) { ckAdvectionStepSetup(*static_cast<Case *>(h)); }
    void orc_ck_linear_correction_matrix(void *h, double alpha)
    {
        ckLinearCorrectionMatrix(*static_cast<Case *>(h), alpha);
    }
    void orc_ck_acoustic_1st_half(void *h, double dt) { ckAcousticStep1stHalf(*static_cast<Case *>(h), dt); }
    void orc_ck_acoustic_2nd_half(void *h, double dt) { ckAcousticStep2ndHalf(*static_cast<Case *>(h), dt); }
    double orc_ck_acoustic_time_step(void *h) { return ckAcousticTimeStep(*static_cast<Case *>(h)); }
    double orc_ck_advection_time_step(void *h) { return ckAdvectionTimeStep(*static_cast<Case *>(h)); }
    void orc_ck_update_particle_position(void *h) { ckUpdateParticlePosition(*static_cast<Case *>(h)); }
    long orc_ck_advection_steps(void *h) { return static_cast<Case *>(h)->ck.advection_steps; }
    // The observer relation is searched on a cell list of the current positions (the
    // driver's relation update at observation time runs on the cell list of the previous
    // configuration; the fluid cell list is rebuilt right after it anyway).
    void orc_ck_observe_pressure(void *h, double *out)
    {
        Case *cs = static_cast<Case *>(h);
        cs->fluid_cells.update(cs->fluid, &cs->periodic);
        updateObserverConfiguration(*cs);
        ckObservePressure(*cs);
        std::copy(cs->observer.observed.begin(), cs->observer.observed.end(), out);
    }
    // CK variables of the fluid: 0 Compression, 1 CompressionRate, 2 VolumetricMeasureRef,
    // 3 CompressionSummation (n values); 4 Displacement (n x dim); 5 LinearCorrectionMatrix
    // (n x dim x dim, row-major); 6 PositionDivergence, 7 Indicator (n values).
    void orc_ck_get(void *h, int which, double *out)
    {
        Case *cs = static_cast<Case *>(h);
        ckEnsureState(*cs);
        CKState &ck = cs->ck;
        const int D = cs->D;
        size_t n = cs->fluid.n;
        const std::vector<Real> *v = which == 0 ? &ck.compression
                                     : which == 1 ? &ck.compression_rate
                                     : which == 2 ? &ck.Vol_ref
                                     : which == 3 ? &ck.compression_sum
                                     : which == 6 ? &ck.pos_div
                                                  : nullptr;
        if (v)
            std::copy(v->begin(), v->end(), out);
        else if (which == 7)
            for (size_t i = 0; i < n; ++i)
                out[i] = ck.indicator[i];
        else if (which == 4)
            for (size_t i = 0; i < n; ++i)
                for (int a = 0; a < D; ++a)
                    out[i * D + a] = ck.dpos[i][a];
        else
            for (size_t i = 0; i < n; ++i)
                for (int a = 0; a < D; ++a)
                    for (int b = 0; b < D; ++b)
                        out[(i * D + a) * D + b] = ck.B[i](a, b);
    }

    // One advection step of the dam-break loop (Dambreak.cpp:166-220 for loop_style 0;
    // test_3d_dambreak/dambreak.cpp:183-224 for loop_style 1, whose acoustic dt is taken
    // after the relaxation and starts from the previous one).  `iteration` is the number
    // of completed advection steps before this one; `acoustic_dt_io` carries the acoustic
    // dt between calls for loop_style 1.  When `observe` is set the observer pressures and
    // the total mechanical energy are sampled after the relaxation and before the
    // configuration update, where Dambreak.cpp:192-201 writes them.  Returns the number of
    // acoustic sub-steps.
    int orc_advection_step(void *h, int loop_style, long iteration, double *physical_time, double *acoustic_dt_io,
                           double *advection_dt_out, int observe, double *observed_out, double *energy_out)
    {
        Case *cs = static_cast<Case *>(h);
        Real Dt = advectionTimeStep(*cs);
        densitySummation(*cs);
        Real relaxation_time = 0;
        Real dt = acoustic_dt_io ? *acoustic_dt_io : 0.0;
        int substeps = 0;
        while (relaxation_time < Dt)
        {
            if (loop_style == 0)
                dt = acousticTimeStep(*cs);
            integration1stHalf(*cs, dt);
            integration2ndHalf(*cs, dt);
            if (loop_style == 1)
                dt = acousticTimeStep(*cs);
            relaxation_time += dt;
            *physical_time += dt;
            ++substeps;
        }
        if (acoustic_dt_io)
            *acoustic_dt_io = dt;
        if (advection_dt_out)
            *advection_dt_out = Dt;
        if (observe)
        {
            observePressure(*cs);
            if (observed_out)
                std::copy(cs->observer.observed.begin(), cs->observer.observed.end(), observed_out);
            if (energy_out)
                *energy_out = totalMechanicalEnergy(*cs);
        }
        long it = iteration + 1;
        if (it % 100 == 0 && it != 1)
            particleSorting(*cs);
        cs->fluid_cells.update(cs->fluid, &cs->periodic);
        updateConfiguration(*cs);
        updateObserverConfiguration(*cs);
        return substeps;
    }
}
