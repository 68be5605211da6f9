// Host-only stand-ins for what the reference's header-only intersection code
// (Utils/CUDA/IRayTracer.h, Utils/CUDA/IntersectionTests.h, Utils/CUDA/Utils.h,
// Scene/KDNode.h) takes from CUDA, OpenEngine core and extensions-CUDA, so that
// code compiles unmodified with g++ for the oracle's pin test.  TEST
// INFRASTRUCTURE ONLY: never part of the library.
//
// The CUDA-SDK vector helpers are not vendored by the reference; they come
// from kdgb_pin_vec.h in the evaluation order the oracle and the kernels
// document.
#pragma once
#include <cmath>
#include <cstddef>
#include <cstdint>
#include <cstring>
#include <sstream>
#include <string>

#define __host__
#define __device__
#define __global__
#define __forceinline__ inline

struct float2 { float x, y; };
struct float3 { float x, y, z; };
struct float4 { float x, y, z, w; };
struct int2 { int x, y; };
struct int4 { int x, y, z, w; };
struct uchar4 { unsigned char x, y, z, w; };
struct longlong2 { long long x, y; };
struct longlong4 { long long x, y, z, w; };

inline float3 make_float3(float x, float y, float z) { float3 r = {x, y, z}; return r; }
inline float4 make_float4(float x, float y, float z, float w) { float4 r = {x, y, z, w}; return r; }
inline int2 make_int2(int x, int y) { int2 r = {x, y}; return r; }
inline int4 make_int4(int x, int y, int z, int w) { int4 r = {x, y, z, w}; return r; }

// Scalar min/max as CUDA provides them for float (fminf/fmaxf).
inline float min(float a, float b) { return fminf(a, b); }
inline float max(float a, float b) { return fmaxf(a, b); }
inline int min(int a, int b) { return a < b ? a : b; }
inline int max(int a, int b) { return a < b ? b : a; }
inline unsigned min(unsigned a, unsigned b) { return a < b ? a : b; }
inline unsigned max(unsigned a, unsigned b) { return a < b ? b : a; }
// Mixed signedness, as CUDA's integer min/max overloads treat it.
inline unsigned min(unsigned a, int b) { return min(a, (unsigned)b); }
inline unsigned min(int a, unsigned b) { return min((unsigned)a, b); }
inline unsigned max(unsigned a, int b) { return max(a, (unsigned)b); }
inline unsigned max(int a, unsigned b) { return max((unsigned)a, b); }

#define KDGB_PIN_HD
#include <kdgb_pin_vec.h>

// Host copies as plain memory copies (the test keeps everything on the host).
enum cudaMemcpyKind { cudaMemcpyHostToHost, cudaMemcpyHostToDevice, cudaMemcpyDeviceToHost, cudaMemcpyDeviceToDevice };
typedef int cudaError_t;
inline cudaError_t cudaMemcpy(void *dst, const void *src, size_t n, cudaMemcpyKind) { memcpy(dst, src, n); return 0; }
template <class T>
inline cudaError_t cudaMemcpyFromSymbol(void *dst, const T &sym, size_t n) { memcpy(dst, &sym, n); return 0; }

// A logger that discards what it is given.
struct KdgbPinLogStream {
    template <class T>
    KdgbPinLogStream &operator<<(const T &) { return *this; }
};
struct KdgbPinLogger {
    KdgbPinLogStream info, warning, error;
    int end = 0;
};
static KdgbPinLogger logger;

// extensions-CUDA's description of the active device (only read by launch
// helpers the pinned functions do not call).
struct KdgbPinDeviceProp {
    int maxThreadsDim[3];
    int maxGridSize[3];
    size_t sharedMemPerBlock;
    int regsPerBlock;
    int warpSize;
};
static KdgbPinDeviceProp activeCudaDevice = {{1024, 1024, 64}, {2147483647, 65535, 65535}, 49152, 65536, 32};

// Kernel execution on the host, one thread at a time (pin tests of the
// reference's per-thread kernels): launch qualifiers vanish, the thread
// coordinates are globals set by the caller, and shared memory is a static
// host buffer.
#define __constant__
#define __shared__ static
#define __launch_bounds__(...)
struct uint3 { unsigned x, y, z; };
struct dim3 { unsigned x, y, z; };
extern uint3 threadIdx, blockIdx;
extern dim3 blockDim, gridDim;
inline void __syncthreads() {}
static const int warpSize = 32;
inline float2 make_float2(float x, float y) { float2 r = {x, y}; return r; }
inline float __int_as_float(int i) { float f; memcpy(&f, &i, sizeof f); return f; }
inline int __float_as_int(float f) { int i; memcpy(&i, &f, sizeof i); return i; }
