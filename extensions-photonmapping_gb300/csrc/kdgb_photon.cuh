// Photon sampling for the incoherent tracing workload: a counter-based
// Philox4x32-10 stream and the direction samplers, written so every operation
// is an IEEE-rounded add, multiply, divide or square root in a fixed order
// (no library sin/cos), which makes the photon paths reproducible bit for bit
// on any IEEE machine.
#pragma once

#include "kdgb_internal.cuh"

namespace kdgb {

// Philox4x32 with 10 rounds (Salmon, Moraes, Dror, Shaw, "Parallel random
// numbers: as easy as 1, 2, 3", SC 2011): multipliers 0xD2511F53 and
// 0xCD9E8D57, Weyl key increments 0x9E3779B9 and 0xBB67AE85.
__device__ __forceinline__ uint4 philox4x32_10(uint4 c, uint2 k)
{
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        if (r > 0) {
            k.x += 0x9E3779B9u;
            k.y += 0xBB67AE85u;
        }
        const unsigned lo0 = 0xD2511F53u * c.x, hi0 = __umulhi(0xD2511F53u, c.x);
        const unsigned lo1 = 0xCD9E8D57u * c.z, hi1 = __umulhi(0xCD9E8D57u, c.z);
        c = make_uint4(hi1 ^ c.y ^ k.x, lo1, hi0 ^ c.w ^ k.y, lo0);
    }
    return c;
}

// Top 24 bits to a float in [0, 1) (exact).
__device__ __forceinline__ float u24(unsigned x) { return (float)(x >> 8) * 0x1p-24f; }

// sin and cos of 2*pi*u for u in [0, 1): quadrant reduction on u (exact),
// then Taylor polynomials on [-pi/4, pi/4] (|error| < 4e-7).
__device__ __forceinline__ void sincos_2pi(float u, float &s, float &c)
{
    const float u4 = __fmul_rn(u, 4.0f);
    const float k = floorf(__fadd_rn(u4, 0.5f));
    const float x = __fmul_rn(__fsub_rn(u4, k), 1.57079632679489662f);
    const float x2 = __fmul_rn(x, x);
    // sin x = x (1 - x^2/6 (1 - x^2/20 (1 - x^2/42)))
    float ps = __fsub_rn(1.0f, __fmul_rn(x2, 0.0238095238095238095f));
    ps = __fsub_rn(1.0f, __fmul_rn(__fmul_rn(x2, 0.05f), ps));
    ps = __fsub_rn(1.0f, __fmul_rn(__fmul_rn(x2, 0.166666666666666667f), ps));
    const float sx = __fmul_rn(x, ps);
    // cos x = 1 - x^2/2 (1 - x^2/12 (1 - x^2/30 (1 - x^2/56)))
    float pc = __fsub_rn(1.0f, __fmul_rn(x2, 0.0178571428571428571f));
    pc = __fsub_rn(1.0f, __fmul_rn(__fmul_rn(x2, 0.0333333333333333333f), pc));
    pc = __fsub_rn(1.0f, __fmul_rn(__fmul_rn(x2, 0.0833333333333333333f), pc));
    const float cx = __fsub_rn(1.0f, __fmul_rn(__fmul_rn(x2, 0.5f), pc));
    const int q = ((int)k) & 3;
    s = q == 0 ? sx : (q == 1 ? cx : (q == 2 ? -sx : -cx));
    c = q == 0 ? cx : (q == 1 ? -sx : (q == 2 ? -cx : sx));
}

// Uniform direction on the unit sphere.
__device__ __forceinline__ float3 sample_sphere(float u0, float u1)
{
    const float z = __fsub_rn(1.0f, __fmul_rn(2.0f, u0));
    const float r = __fsqrt_rn(fmaxf(0.0f, __fsub_rn(1.0f, __fmul_rn(z, z))));
    float s, c;
    sincos_2pi(u1, s, c);
    return make_float3(__fmul_rn(r, c), __fmul_rn(r, s), z);
}

// Cosine-weighted direction around unit normal n, with the orthonormal basis
// of Duff et al., "Building an Orthonormal Basis, Revisited" (JCGT 2017).
__device__ __forceinline__ float3 sample_cosine(float3 n, float u0, float u1)
{
    const float r = __fsqrt_rn(u0);
    float s, c;
    sincos_2pi(u1, s, c);
    const float x = __fmul_rn(r, c), y = __fmul_rn(r, s);
    const float z = __fsqrt_rn(fmaxf(0.0f, __fsub_rn(1.0f, u0)));
    const float sign = copysignf(1.0f, n.z);
    const float a = __fdiv_rn(-1.0f, __fadd_rn(sign, n.z));
    const float b = __fmul_rn(__fmul_rn(n.x, n.y), a);
    const float3 t = make_float3(__fadd_rn(1.0f, __fmul_rn(__fmul_rn(__fmul_rn(sign, n.x), n.x), a)),
                                 __fmul_rn(sign, b), -__fmul_rn(sign, n.x));
    const float3 bt = make_float3(b, __fadd_rn(sign, __fmul_rn(__fmul_rn(n.y, n.y), a)), -n.y);
    return make_float3(__fadd_rn(__fadd_rn(__fmul_rn(t.x, x), __fmul_rn(bt.x, y)), __fmul_rn(n.x, z)),
                       __fadd_rn(__fadd_rn(__fmul_rn(t.y, x), __fmul_rn(bt.y, y)), __fmul_rn(n.y, z)),
                       __fadd_rn(__fadd_rn(__fmul_rn(t.z, x), __fmul_rn(bt.z, y)), __fmul_rn(n.z, z)));
}

}  // namespace kdgb
