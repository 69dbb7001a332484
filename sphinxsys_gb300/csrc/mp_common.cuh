// Device helpers shared by the mixed-precision solvers (single case and batch).
#pragma once

#include "sphx_device.cuh"

namespace sphx
{
namespace mpc
{
constexpr float kTinyF = 2.71051e-20f; // TinyReal of the reference, base_data_type.h:207
constexpr int kGroup = 8;             // neighbours per plain partial sum
constexpr int kUnroll = 4;            // neighbour records in flight per thread in list sweeps

struct Kahan
{
    float s = 0.f, c = 0.f;
    __device__ __forceinline__ void add(float x)
    {
        float y = x - c;
        float t = s + y;
        c = (t - s) - y;
        s = t;
    }
    __device__ __forceinline__ float value() const { return s - c; }
};

// Compensated neighbour sum: plain FP32 partials over groups, Kahan across groups.
struct Acc
{
    float part = 0.f;
    Kahan k;
    __device__ __forceinline__ void add(float x) { part += x; }
    __device__ __forceinline__ void flush()
    {
        k.add(part);
        part = 0.f;
    }
    __device__ __forceinline__ float value() const { return k.value(); }
};

// Warp max of the order-preserving bits of v, one atomicMax per warp.
__device__ __forceinline__ void warp_max_to(unsigned long long *slot, double v)
{
    unsigned long long b = ordered_bits(v);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
    {
        unsigned long long y = __shfl_down_sync(0xffffffffu, b, o);
        b = y > b ? y : b;
    }
    if ((threadIdx.x & 31u) == 0)
        atomicMax(slot, b);
}

// Wendland C2 in FP32 with t = 1 - q/2: W = fW t^4 (1 + 2q), dW = fdW 0.625 (q - 2)^3 q.
__device__ __forceinline__ float wc2_W(float fW, float inv_h, float r)
{
    float q = r * inv_h;
    float t = 1.0f - 0.5f * q;
    float t2 = t * t;
    return fW * (t2 * t2 * (1.0f + 2.0f * q));
}
__device__ __forceinline__ float wc2_dW(float fdW, float inv_h, float r)
{
    float q = r * inv_h;
    float t = q - 2.0f;
    return fdW * (0.625f * (t * t * t) * q);
}

// DissipativePJump of AcousticRiemannSolver with the TruncatedLinear limiter.
__device__ __forceinline__ float p_jump(float zgeo, float inv_c0, float slope, float u)
{
    return zgeo * u * fminf(slope * (inv_c0 * fmaxf(u, 0.0f)), 1.0f);
}
} // namespace mpc
} // namespace sphx
