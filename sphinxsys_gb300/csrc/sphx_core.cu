// Context, particle-variable registry, mesh and kernel constants of libsphx_cuda.so.
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>

#include "sphx_internal.cuh"

namespace sphx
{
static thread_local char g_err[512] = "";

int fail(int code, const char *fmt, ...)
{
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof(g_err), fmt, ap);
    va_end(ap);
    return code;
}

int cuda_fail(cudaError_t e, const char *what, const char *file, int line)
{
    return fail(e == cudaErrorMemoryAllocation ? SPHX_ERR_OUT_OF_MEMORY : SPHX_ERR_CUDA, "%s failed at %s:%d: %s",
                what, file, line, cudaGetErrorString(e));
}

MeshDev mesh_dev(const sphx_mesh_desc &m)
{
    MeshDev d{};
    for (int a = 0; a < 3; ++a)
    {
        d.lower[a] = m.lower[a];
        d.all_cells[a] = a < m.dim ? m.all_cells[a] : 1;
        d.grid_points[a] = d.all_cells[a] + 1;
    }
    d.gs = m.grid_spacing;
    return d;
}

WendlandC2 wendland(int dim, double h)
{
    const double Pi = M_PI;
    WendlandC2 k{};
    k.h = h;
    k.inv_h = 1.0 / h;
    k.rc = 2.0 * h;
    k.rc_sqr = k.rc * k.rc;
    if (dim == 2)
        k.factor_W = k.inv_h * k.inv_h * 7.0 / (4.0 * Pi);
    else
        k.factor_W = k.inv_h * k.inv_h * k.inv_h * 21.0 / (16.0 * Pi);
    k.factor_dW = k.inv_h * k.factor_W;
    // FP32 pre-filter on offsets of at most a few cells: relative rounding error of the
    // squared distance stays far below 2^-10, so candidates above this bound are outside rc.
    k.prefilter_sqr = float(k.rc_sqr * (1.0 + 1.0 / 1024.0));
    return k;
}
} // namespace sphx

using namespace sphx;

int sphx_ctx_s::ensure_scratch(size_t bytes)
{
    if (bytes <= scratch_bytes)
        return SPHX_OK;
    if (d_scratch)
        cudaFree(d_scratch);
    d_scratch = nullptr;
    scratch_bytes = 0;
    size_t nb = bytes + bytes / 4 + 4096;
    SPHX_CUDA(cudaMalloc(&d_scratch, nb));
    scratch_bytes = nb;
    return SPHX_OK;
}

int sphx_body_s::require(const char *name, sphx_dtype dtype, int nc, Field **out)
{
    Field *f = find(name);
    if (f)
    {
        if (f->dtype != dtype || f->ncomp != nc)
            return fail(SPHX_ERR_INVALID_ARG, "variable %s exists with another type or component count", name);
        *out = f;
        return SPHX_OK;
    }
    Field nf;
    nf.dtype = dtype;
    nf.ncomp = nc;
    size_t bytes = std::max<size_t>(1, n) * size_t(nc) * dtype_size(dtype);
    SPHX_CUDA(cudaMalloc(&nf.dev, bytes));
    SPHX_CUDA(cudaMemsetAsync(nf.dev, 0, bytes, ctx->stream));
    fields[name] = nf;
    *out = &fields[name];
    return SPHX_OK;
}

int sphx_body_s::need(const char *name, sphx_dtype dtype, int nc, Field **out)
{
    Field *f = find(name);
    if (!f)
        return fail(SPHX_ERR_NOT_FOUND, "variable %s is not registered on this body", name);
    if (f->dtype != dtype || f->ncomp != nc)
        return fail(SPHX_ERR_INVALID_ARG, "variable %s has another type or component count", name);
    *out = f;
    return SPHX_OK;
}

extern "C" const char *sphx_last_error(void) { return g_err; }
extern "C" const char *sphx_version(void) { return "sphx-gb300 0.1 (sm_103a)"; }

namespace sphx
{
static std::vector<CheckReader> &check_readers()
{
    static std::vector<CheckReader> readers;
    return readers;
}

int check_register(CheckReader reader)
{
    check_readers().push_back(reader);
    return int(check_readers().size());
}
} // namespace sphx

extern "C" int sphx_checked_build(void)
{
#ifdef SPHX_CHECK
    return 1;
#else
    return 0;
#endif
}

extern "C" int sphx_check_violations(uint64_t *count, uint64_t *first, int reset)
{
    SPHX_CUDA(cudaDeviceSynchronize());
    unsigned long long total = 0, first_seen = 0;
    for (CheckReader read : check_readers())
    {
        unsigned long long c = 0, f = 0;
        if (read(&c, &f, reset != 0) != 0)
            return fail(SPHX_ERR_CUDA, "reading the bounds-check record failed");
        if (c && !total)
            first_seen = f;
        total += c;
    }
    if (count)
        *count = total;
    if (first)
        *first = first_seen;
    if (total)
        return fail(SPHX_ERR_BOUNDS, "%llu failed index tests; first: site %llu, value %llu", total,
                    first_seen >> 48, first_seen & 0xffffffffffffull);
    return SPHX_OK;
}

extern "C" int sphx_ctx_create(int device, void *stream, sphx_ctx *out)
{
    if (!out)
        return fail(SPHX_ERR_INVALID_ARG, "null output handle");
    int ndev = 0;
    cudaError_t e = cudaGetDeviceCount(&ndev);
    if (e != cudaSuccess || ndev == 0)
        return fail(SPHX_ERR_NO_DEVICE, "no CUDA device available (%s)", cudaGetErrorString(e));
    if (device < 0 || device >= ndev)
        return fail(SPHX_ERR_INVALID_ARG, "device %d out of range (%d devices)", device, ndev);
    SPHX_CUDA(cudaSetDevice(device));
    sphx_ctx c = new sphx_ctx_s();
    c->device = device;
    SPHX_CUDA(cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, device));
    if (stream)
        c->stream = static_cast<cudaStream_t>(stream);
    else
    {
        SPHX_CUDA(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
        c->own_stream = true;
    }
    SPHX_CUDA(cudaMalloc(&c->d_red, 64 * sizeof(unsigned long long)));
    SPHX_CUDA(cudaMallocHost(&c->h_red, 64 * sizeof(unsigned long long)));
    *out = c;
    return SPHX_OK;
}

void sphx::release(sphx_ctx c)
{
    if (--c->refs > 0)
        return;
    cudaSetDevice(c->device);
    cudaStreamSynchronize(c->stream);
    if (c->d_red)
        cudaFree(c->d_red);
    if (c->h_red)
        cudaFreeHost(c->h_red);
    if (c->d_scratch)
        cudaFree(c->d_scratch);
    if (c->own_stream)
        cudaStreamDestroy(c->stream);
    delete c;
}

extern "C" int sphx_ctx_destroy(sphx_ctx c)
{
    if (c)
        release(c);
    return SPHX_OK;
}

extern "C" int sphx_ctx_synchronize(sphx_ctx c)
{
    if (!c)
        return fail(SPHX_ERR_INVALID_ARG, "null context");
    SPHX_CUDA(cudaStreamSynchronize(c->stream));
    return SPHX_OK;
}

extern "C" int sphx_ctx_launch_count(sphx_ctx c, uint64_t *count)
{
    if (!c || !count)
        return fail(SPHX_ERR_INVALID_ARG, "null argument");
    *count = c->launches;
    return SPHX_OK;
}

extern "C" int sphx_ctx_stream(sphx_ctx c, void **stream)
{
    if (!c || !stream)
        return fail(SPHX_ERR_INVALID_ARG, "null argument");
    *stream = c->stream;
    return SPHX_OK;
}

extern "C" int sphx_body_create(sphx_ctx ctx, int dim, size_t n, sphx_body *out)
{
    if (!ctx || !out || (dim != 2 && dim != 3))
        return fail(SPHX_ERR_INVALID_ARG, "invalid body arguments (dim=%d)", dim);
    if (n > 0xffffffffull)
        return fail(SPHX_ERR_INVALID_ARG, "body size %zu exceeds 32-bit particle indices", n);
    sphx_body b = new sphx_body_s();
    b->ctx = ctx;
    ctx->retain();
    b->dim = dim;
    b->n = n;
    *out = b;
    return SPHX_OK;
}

extern "C" int sphx_body_destroy(sphx_body b)
{
    if (!b)
        return SPHX_OK;
    sphx_ctx ctx = b->ctx;
    cudaStreamSynchronize(ctx->stream);
    for (auto &kv : b->fields)
        cudaFree(kv.second.dev);
    delete b;
    release(ctx);
    return SPHX_OK;
}

extern "C" int sphx_body_size(sphx_body b, size_t *n)
{
    if (!b || !n)
        return fail(SPHX_ERR_INVALID_ARG, "null argument");
    *n = b->n;
    return SPHX_OK;
}

extern "C" int sphx_body_register(sphx_body b, const char *name, sphx_dtype dtype, int ncomp)
{
    if (!b || !name || ncomp < 1 || ncomp > 3)
        return fail(SPHX_ERR_INVALID_ARG, "invalid register arguments");
    Field *f;
    return b->require(name, dtype, ncomp, &f);
}

namespace
{
// AoS (count x nc) <-> rows [first, first + count) of an SoA array with row stride
// `stride` (component c of row r at soa[c * stride + r]); 4- or 8-byte elements.
template <typename T>
__global__ void k_aos_to_soa(size_t count, int nc, const T *__restrict__ aos, T *__restrict__ soa, size_t stride,
                             size_t first)
{
    size_t k = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (k >= count * size_t(nc))
        return;
    size_t c = k / count, i = k - c * count;
    soa[c * stride + first + i] = aos[i * size_t(nc) + c];
}
template <typename T>
__global__ void k_soa_to_aos(size_t count, int nc, const T *__restrict__ soa, size_t stride, size_t first,
                             T *__restrict__ aos)
{
    size_t k = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (k >= count * size_t(nc))
        return;
    size_t i = k / size_t(nc), c = k - i * size_t(nc);
    aos[k] = soa[c * stride + first + i];
}

int transpose(sphx_ctx ctx, size_t es, size_t count, int nc, size_t stride, size_t first, const void *src, void *dst,
              bool to_soa)
{
    unsigned g = grid_for(count * size_t(nc), 256);
    cudaStream_t s = ctx->stream;
    if (es == 8)
    {
        if (to_soa)
            k_aos_to_soa<<<g, 256, 0, s>>>(count, nc, static_cast<const double *>(src), static_cast<double *>(dst),
                                           stride, first);
        else
            k_soa_to_aos<<<g, 256, 0, s>>>(count, nc, static_cast<const double *>(src), stride, first,
                                           static_cast<double *>(dst));
    }
    else
    {
        if (to_soa)
            k_aos_to_soa<<<g, 256, 0, s>>>(count, nc, static_cast<const uint32_t *>(src),
                                           static_cast<uint32_t *>(dst), stride, first);
        else
            k_soa_to_aos<<<g, 256, 0, s>>>(count, nc, static_cast<const uint32_t *>(src), stride, first,
                                           static_cast<uint32_t *>(dst));
    }
    SPHX_LAUNCHED(ctx);
    return SPHX_OK;
}

// Host AoS rows -> device SoA rows [first, first + count): one copy of the host buffer (at
// full link speed when the caller's buffer is pinned), then the transpose on the device.
// Synchronous: the host buffer may be reused when the call returns.
int upload_rows(sphx_body b, Field *f, const void *host, size_t first, size_t count)
{
    if (count == 0)
        return SPHX_OK;
    sphx_ctx ctx = b->ctx;
    size_t es = dtype_size(f->dtype), bytes = count * size_t(f->ncomp) * es;
    if (f->ncomp == 1)
        SPHX_CUDA(cudaMemcpyAsync(static_cast<unsigned char *>(f->dev) + first * es, host, bytes,
                                  cudaMemcpyHostToDevice, ctx->stream));
    else
    {
        SPHX_TRY(ctx->ensure_scratch(bytes));
        SPHX_CUDA(cudaMemcpyAsync(ctx->d_scratch, host, bytes, cudaMemcpyHostToDevice, ctx->stream));
        SPHX_TRY(transpose(ctx, es, count, f->ncomp, b->n, first, ctx->d_scratch, f->dev, true));
    }
    SPHX_CUDA(cudaStreamSynchronize(ctx->stream));
    return SPHX_OK;
}

// Device SoA rows -> host AoS: transpose on the device, then one copy (synchronises).
int download_rows(sphx_body b, const Field *f, void *host, size_t first, size_t count)
{
    if (count == 0)
        return SPHX_OK;
    sphx_ctx ctx = b->ctx;
    size_t es = dtype_size(f->dtype), bytes = count * size_t(f->ncomp) * es;
    if (f->ncomp == 1)
        SPHX_CUDA(cudaMemcpyAsync(host, static_cast<const unsigned char *>(f->dev) + first * es, bytes,
                                  cudaMemcpyDeviceToHost, ctx->stream));
    else
    {
        SPHX_TRY(ctx->ensure_scratch(bytes));
        SPHX_TRY(transpose(ctx, es, count, f->ncomp, b->n, first, f->dev, ctx->d_scratch, false));
        SPHX_CUDA(cudaMemcpyAsync(host, ctx->d_scratch, bytes, cudaMemcpyDeviceToHost, ctx->stream));
    }
    SPHX_CUDA(cudaStreamSynchronize(ctx->stream));
    return SPHX_OK;
}
} // namespace

extern "C" int sphx_body_upload(sphx_body b, const char *name, sphx_dtype dtype, int ncomp, const void *host,
                                size_t n)
{
    if (!b || !name || !host || ncomp < 1 || ncomp > 3)
        return fail(SPHX_ERR_INVALID_ARG, "invalid upload arguments");
    if (n != b->n)
        return fail(SPHX_ERR_INVALID_ARG, "upload of %s: %zu values for a body of %zu particles", name, n, b->n);
    Field *f;
    SPHX_TRY(b->require(name, dtype, ncomp, &f));
    return upload_rows(b, f, host, 0, n);
}

extern "C" int sphx_body_download(sphx_body b, const char *name, void *host, size_t n)
{
    if (!b || !name || !host)
        return fail(SPHX_ERR_INVALID_ARG, "invalid download arguments");
    Field *f = b->find(name);
    if (!f)
        return fail(SPHX_ERR_NOT_FOUND, "variable %s is not registered", name);
    if (n != b->n)
        return fail(SPHX_ERR_INVALID_ARG, "download of %s: buffer for %zu of %zu particles", name, n, b->n);
    return download_rows(b, f, host, 0, n);
}

extern "C" int sphx_body_upload_rows(sphx_body b, const char *name, const void *host, size_t first, size_t count)
{
    if (!b || !name || (count && !host))
        return fail(SPHX_ERR_INVALID_ARG, "invalid upload arguments");
    Field *f = b->find(name);
    if (!f)
        return fail(SPHX_ERR_NOT_FOUND, "variable %s is not registered", name);
    if (first > b->n || count > b->n - first)
        return fail(SPHX_ERR_INVALID_ARG, "rows [%zu, %zu) of %s outside a body of %zu particles", first,
                    first + count, name, b->n);
    return upload_rows(b, f, host, first, count);
}

extern "C" int sphx_body_download_rows(sphx_body b, const char *name, void *host, size_t first, size_t count)
{
    if (!b || !name || (count && !host))
        return fail(SPHX_ERR_INVALID_ARG, "invalid download arguments");
    Field *f = b->find(name);
    if (!f)
        return fail(SPHX_ERR_NOT_FOUND, "variable %s is not registered", name);
    if (first > b->n || count > b->n - first)
        return fail(SPHX_ERR_INVALID_ARG, "rows [%zu, %zu) of %s outside a body of %zu particles", first,
                    first + count, name, b->n);
    return download_rows(b, f, host, first, count);
}

extern "C" int sphx_body_device_ptr(sphx_body b, const char *name, void **dev, sphx_dtype *dtype, int *ncomp)
{
    if (!b || !name || !dev)
        return fail(SPHX_ERR_INVALID_ARG, "invalid arguments");
    Field *f = b->find(name);
    if (!f)
        return fail(SPHX_ERR_NOT_FOUND, "variable %s is not registered", name);
    *dev = f->dev;
    if (dtype)
        *dtype = f->dtype;
    if (ncomp)
        *ncomp = f->ncomp;
    return SPHX_OK;
}

namespace
{
// Particles of an SoA variable (component c of particle i at v[c * n + i]) with a
// non-finite component; one atomic per particle found.
template <typename T>
__global__ void k_count_non_finite(size_t n, int ncomp, const T *__restrict__ v, unsigned long long *count)
{
    for (size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += size_t(gridDim.x) * blockDim.x)
    {
        bool fin = true;
        for (int c = 0; c < ncomp; ++c)
            fin = fin && isfinite(v[size_t(c) * n + i]);
        if (!fin)
            atomicAdd(count, 1ull);
    }
}
} // namespace

extern "C" int sphx_body_check_finite(sphx_body b, const char *name, uint64_t *non_finite)
{
    if (!b || !name)
        return fail(SPHX_ERR_INVALID_ARG, "invalid check arguments");
    Field *f = b->find(name);
    if (!f)
        return fail(SPHX_ERR_NOT_FOUND, "variable %s is not registered", name);
    if (f->dtype != SPHX_F64 && f->dtype != SPHX_F32)
        return fail(SPHX_ERR_INVALID_ARG, "variable %s is not a floating-point variable", name);
    sphx_ctx ctx = b->ctx;
    SPHX_TRY(ctx->ensure_scratch(sizeof(unsigned long long)));
    unsigned long long *d = static_cast<unsigned long long *>(ctx->d_scratch);
    SPHX_CUDA(cudaMemsetAsync(d, 0, sizeof(unsigned long long), ctx->stream));
    if (b->n > 0)
    {
        unsigned g = unsigned(std::max(1, std::min(ctx->num_sms * 4, int(grid_for(b->n, 256)))));
        if (f->dtype == SPHX_F64)
            k_count_non_finite<<<g, 256, 0, ctx->stream>>>(b->n, f->ncomp, static_cast<const double *>(f->dev), d);
        else
            k_count_non_finite<<<g, 256, 0, ctx->stream>>>(b->n, f->ncomp, static_cast<const float *>(f->dev), d);
        SPHX_LAUNCHED(ctx);
    }
    unsigned long long h = 0;
    SPHX_CUDA(cudaMemcpyAsync(&h, d, sizeof(h), cudaMemcpyDeviceToHost, ctx->stream));
    SPHX_CUDA(cudaStreamSynchronize(ctx->stream));
    if (non_finite)
        *non_finite = h;
    if (h)
        return fail(SPHX_ERR_NUMERIC, "variable %s: %llu particles with non-finite values", name, h);
    return SPHX_OK;
}

extern "C" int sphx_mesh_from_bounds(int dim, const double *lower, const double *upper, double gs, int buffer_width,
                                     sphx_mesh_desc *out)
{
    if (!lower || !upper || !out || (dim != 2 && dim != 3) || !(gs > 0) || buffer_width < 0)
        return fail(SPHX_ERR_INVALID_ARG, "invalid mesh arguments");
    sphx_mesh_desc m{};
    m.dim = dim;
    m.grid_spacing = gs;
    double buffer = double(buffer_width) * gs;
    for (int a = 0; a < 3; ++a)
    {
        if (a < dim)
        {
            m.lower[a] = lower[a] - buffer;
            double tentative = upper[a] + buffer - m.lower[a];
            double cells = std::ceil(tentative / gs);
            if (!(cells >= 1) || cells > 1.0e6)
                return fail(SPHX_ERR_INVALID_ARG, "mesh axis %d has %g cells", a, cells);
            m.all_cells[a] = int(cells) + 1 - 1;
        }
        else
        {
            m.lower[a] = 0;
            m.all_cells[a] = 1;
        }
    }
    *out = m;
    return SPHX_OK;
}

extern "C" int sphx_lattice_number_density(int dim, double h, double dp, double *sigma0)
{
    if ((dim != 2 && dim != 3) || !(h > 0) || !(dp > 0) || !sigma0)
        return fail(SPHX_ERR_INVALID_ARG, "invalid lattice arguments");
    WendlandC2 k = wendland(dim, h);
    auto W = [&](double r) {
        double q = r * k.inv_h;
        return k.factor_W * (std::pow(1.0 - 0.5 * q, 4) * (1.0 + 2.0 * q));
    };
    double sigma = 0;
    int depth = int(k.rc / dp) + 1;
    int kmax = dim == 3 ? depth : 0;
    for (int kk = -kmax; kk <= kmax; ++kk)
        for (int j = -depth; j <= depth; ++j)
            for (int i = -depth; i <= depth; ++i)
            {
                double x = i * dp, y = j * dp, z = kk * dp;
                double d = dim == 2 ? std::sqrt(x * x + y * y) : std::sqrt((x * x + y * y) + z * z);
                if (d < k.rc)
                    sigma += W(d);
            }
    *sigma0 = sigma;
    return SPHX_OK;
}
