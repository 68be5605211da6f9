// The CUDA-SDK vector helpers (cutil_math) that the reference uses but does
// not vendor, shared by the g++ and the nvcc stand-ins of Meta/CUDA.h.  TEST
// INFRASTRUCTURE ONLY.
//
// Evaluation order as the oracle and the kernels document it: dot left to
// right, standard cross components, every operation rounded separately
// (compile with -ffp-contract=off), normalize with an IEEE 1/sqrt (the SDK's
// host branch).  KDGB_PIN_HD is empty for g++ and __host__ __device__ for
// nvcc; the including header defines float3/float4 and make_float3(x, y, z)
// / make_float4(x, y, z, w) before this file.
#pragma once

KDGB_PIN_HD inline float3 make_float3(float4 a) { return make_float3(a.x, a.y, a.z); }
KDGB_PIN_HD inline float3 make_float3(float s) { return make_float3(s, s, s); }
KDGB_PIN_HD inline float4 make_float4(float3 a, float w) { return make_float4(a.x, a.y, a.z, w); }
KDGB_PIN_HD inline float4 make_float4(float3 a) { return make_float4(a.x, a.y, a.z, 0.0f); }
KDGB_PIN_HD inline float4 make_float4(float s) { return make_float4(s, s, s, s); }

KDGB_PIN_HD inline float3 operator+(float3 a, float3 b) { return make_float3(a.x + b.x, a.y + b.y, a.z + b.z); }
KDGB_PIN_HD inline float3 operator-(float3 a, float3 b) { return make_float3(a.x - b.x, a.y - b.y, a.z - b.z); }
KDGB_PIN_HD inline float3 operator*(float3 a, float3 b) { return make_float3(a.x * b.x, a.y * b.y, a.z * b.z); }
KDGB_PIN_HD inline float3 operator/(float3 a, float3 b) { return make_float3(a.x / b.x, a.y / b.y, a.z / b.z); }
KDGB_PIN_HD inline float3 operator*(float3 a, float s) { return make_float3(a.x * s, a.y * s, a.z * s); }
KDGB_PIN_HD inline float3 operator*(float s, float3 a) { return make_float3(s * a.x, s * a.y, s * a.z); }
KDGB_PIN_HD inline float3 operator-(float3 a) { return make_float3(-a.x, -a.y, -a.z); }
KDGB_PIN_HD inline void operator-=(float3 &a, float3 b) { a = a - b; }
KDGB_PIN_HD inline void operator+=(float3 &a, float3 b) { a = a + b; }
KDGB_PIN_HD inline float4 operator+(float4 a, float4 b) { return make_float4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w); }
KDGB_PIN_HD inline float4 operator*(float s, float4 a) { return make_float4(s * a.x, s * a.y, s * a.z, s * a.w); }
KDGB_PIN_HD inline float4 operator*(float4 a, float s) { return make_float4(a.x * s, a.y * s, a.z * s, a.w * s); }

KDGB_PIN_HD inline float dot(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
KDGB_PIN_HD inline float3 cross(float3 a, float3 b)
{
    return make_float3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
KDGB_PIN_HD inline float length(float3 v) { return sqrtf(dot(v, v)); }
KDGB_PIN_HD inline float3 normalize(float3 v)
{
    const float inv = 1.0f / sqrtf(dot(v, v));
    return v * inv;
}
KDGB_PIN_HD inline float clamp(float f, float a, float b) { return fmaxf(a, fminf(f, b)); }
KDGB_PIN_HD inline float3 clamp(float3 v, float a, float b)
{
    return make_float3(clamp(v.x, a, b), clamp(v.y, a, b), clamp(v.z, a, b));
}
