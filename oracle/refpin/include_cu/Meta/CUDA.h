// nvcc stand-ins for what the reference's tracer sources (Utils/CUDA/
// Raytracer.cu, ShortStack.cu, BruteTracer.cu) take from OpenEngine core,
// extensions-CUDA, cutil and the CUDA SDK, so that those files compile
// unmodified and their __host__ __device__ traversal functions can be called
// on the host.  TEST INFRASTRUCTURE ONLY: never part of the library.
//
// The host branches of the reference's fetch helpers (Utils/CUDA/Utils.h)
// read through cudaMemcpy / cudaMemcpyFromSymbol; refpin_runtime.cpp answers
// those with plain host copies, so the traversal runs on host arrays without
// a GPU.
#pragma once
#include <cuda_runtime.h>

#include <cmath>
#include <cstddef>
#include <cstdint>
#include <cstring>
#include <sstream>
#include <string>
#include <strings.h>

#define KDGB_PIN_HD __host__ __device__
#include <kdgb_pin_vec.h>

// Gone from CUDA 13 (same meaning; device code only ever compiled here,
// never run).
#define cudaThreadSynchronize cudaDeviceSynchronize
__device__ inline float saturate(float v) { return __saturatef(v); }
#define CHECK_FOR_CUDA_ERROR() ((void)0)

// cutil's timers (the timing lines of the host methods).
inline void cutCreateTimer(unsigned int *id) { *id = 0; }
inline void cutResetTimer(unsigned int) {}
inline void cutStartTimer(unsigned int) {}
inline void cutStopTimer(unsigned int) {}
inline float cutGetTimerValue(unsigned int) { return 0.0f; }

// extensions-CUDA's description of the active device (read by KernelConf1D).
struct KdgbPinDeviceProp {
    int maxThreadsDim[3];
    int maxGridSize[3];
    size_t sharedMemPerBlock;
    int regsPerBlock;
    int warpSize;
};
static KdgbPinDeviceProp activeCudaDevice = {{1024, 1024, 64}, {2147483647, 65535, 65535}, 49152, 65536, 32};

// OpenEngine's logger, as an observer of the reference's own CUDALogger lines
// (Utils/CUDA/Utils.h:36-38, host branch).  It keeps what the traversal
// reports after each leaf ("THit: " << tHit) and, in Raytracer.cu, the
// primitive of a hit ("Primary ray intersected " << primHit); everything
// else is dropped.
struct KdgbPinLogEnd {};
struct KdgbPinObserved {
    float3 last_thit;      // tHit after the latest leaf
    int have_thit;
    int first_prim;        // first "Primary ray intersected" of the ray
    float3 first_thit;     // tHit logged just before it
    int have_first;
};
static KdgbPinObserved kdgb_pin_observed;
static inline void kdgb_pin_observe_reset() { memset(&kdgb_pin_observed, 0, sizeof kdgb_pin_observed); }

struct KdgbPinLogStream {
    int state = 0;  // 1 after "THit: ", 2 after "Primary ray intersected "
    KdgbPinLogStream &operator<<(const char *s)
    {
        state = strcmp(s, "THit: ") == 0 ? 1 : (strcmp(s, "Primary ray intersected ") == 0 ? 2 : 0);
        return *this;
    }
    KdgbPinLogStream &operator<<(char *s) { return *this << (const char *)s; }
    KdgbPinLogStream &operator<<(const float3 &v)
    {
        if (state == 1) {
            kdgb_pin_observed.last_thit = v;
            kdgb_pin_observed.have_thit = 1;
        }
        state = 0;
        return *this;
    }
    KdgbPinLogStream &operator<<(int v)
    {
        if (state == 2 && !kdgb_pin_observed.have_first) {
            kdgb_pin_observed.first_prim = v;
            kdgb_pin_observed.first_thit = kdgb_pin_observed.last_thit;
            kdgb_pin_observed.have_first = 1;
        }
        state = 0;
        return *this;
    }
    KdgbPinLogStream &operator<<(const KdgbPinLogEnd &) { state = 0; return *this; }
    template <class T>
    KdgbPinLogStream &operator<<(const T &) { state = 0; return *this; }
};
struct KdgbPinLogger {
    KdgbPinLogStream info, warning, error;
    KdgbPinLogEnd end;
};
static KdgbPinLogger logger;

// The specular power of the shading loop (Utils/CUDA/Kernels/ColorKernels.h:28-32
// calls __powf on the device and powf on the host).  Declared in the namespace
// the tracer sources include ColorKernels.h into, so their host branch calls
// this one: the C library's powf unless ref_trace_set_pow installed another
// function (refpin_trace.h).
namespace OpenEngine {
namespace Utils {
namespace CUDA {
float powf(float x, float y);
}  // namespace CUDA
}  // namespace Utils
}  // namespace OpenEngine
