// Device helpers shared by the USFFT gather/scatter kernels.
#pragma once

#include <cuda_runtime.h>

#include "rectv_internal.cuh"

namespace rectv {

__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
    return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

// (a.x b.x + c.x, a.y b.y + c.y) as one packed FP32x2 FMA (each lane an IEEE
// fma.rn, so results equal two fmaf calls).
__device__ __forceinline__ float2 ffma2(float2 a, float2 b, float2 c) {
    unsigned long long d;
    asm("fma.rn.f32x2 %0, %1, %2, %3;"
        : "=l"(d)
        : "l"(*reinterpret_cast<const unsigned long long *>(&a)), "l"(*reinterpret_cast<const unsigned long long *>(&b)),
          "l"(*reinterpret_cast<const unsigned long long *>(&c)));
    return *reinterpret_cast<const float2 *>(&d);
}

// Position of polar sample (theta, k): identical float operation sequence to
// the host plan (plan.cpp) and to takexy (kernels_radonusfft.cuh:73-78).
__device__ __forceinline__ void sample_pos(int k, float2 sc, const UsGeo &g, float &x0, float &y0, int &fx,
                                           int &fy) {
    const float q = __fdiv_rn((float)(k - g.n / 2), (float)g.n);
    x0 = __fmul_rn(q, sc.x);
    y0 = __fmul_rn(q, sc.y);
    if (x0 >= 0.5f) x0 = 0.5f - 1e-5f;
    if (y0 >= 0.5f) y0 = 0.5f - 1e-5f;
    fx = (int)floorf(__fmul_rn(g.tn, x0));
    fy = (int)floorf(__fmul_rn(g.tn, y0));
}

// Gaussian weight exp(-pi^2/mu d^2) of tap i of the 9 taps per axis
// (gather, kernels_radonusfft.cuh:116-118; pi/mu and 1/n are applied once).
__device__ __forceinline__ float tap_weight(int f, int i, float p0, const UsGeo &g) {
    const float d = (float)(f - kR + i) * g.inv2n - p0;
    return __expf(-g.wexp * d * d);
}

__device__ __forceinline__ void tap_weights(int f, float p0, const UsGeo &g, float (&e)[kTaps]) {
#pragma unroll
    for (int i = 0; i < kTaps; ++i) e[i] = tap_weight(f, i, p0, g);
}

}  // namespace rectv
