// kdgb_trace_brute_noalloc: brute-force first-hit tracing that allocates no
// device memory.
//
// kdgb_trace_brute converts the caller's T*9 triangles into a packed form in
// scratch memory it allocates per call.  This variant keeps that scratch in a
// file-scope device array of fixed size instead, so a caller that cannot
// allocate device memory while it runs can still trace.  The array lives in
// the library's module image: every GPU that loads this library holds it
// (KDGB_NOALLOC_MAX_TRIS * 48 bytes = 3 MiB) until the process exits.
//
// Host code cannot use the array's name as a device address; the address is
// fetched per device with cudaGetSymbolAddress, on the first call made with
// that device current, and cached together with the identity of the CUDA
// context it belongs to.  A context torn down and created again (after
// cudaDeviceReset) reloads the module, possibly elsewhere: the next call sees
// a different context id and fetches the address again.
#include <cuda.h>
#include <cuda_runtime.h>

#include <mutex>

#include "kdgb_internal.cuh"

namespace kdgb {
namespace {

constexpr int kNoAllocBlock = 128;
constexpr int kMaxDevices = 64;

// Packed triangle records {v0.xyz, e1.x} {e1.yz, e2.xy} {e2.z, id, 0, 0}.
static __device__ __align__(256) float4 g_noalloc_tris[3 * KDGB_NOALLOC_MAX_TRIS];

std::mutex g_noalloc_mu;
float4 *g_noalloc_addr[kMaxDevices] = {};
unsigned long long g_noalloc_ctx[kMaxDevices] = {};  // context id the address belongs to

// cuCtxGetCurrent / cuCtxGetId, fetched through the runtime so that the
// library does not link the driver library itself.
typedef CUresult (*CtxGetCurrentFn)(CUcontext *);
typedef CUresult (*CtxGetIdFn)(CUcontext, unsigned long long *);
CtxGetCurrentFn g_ctx_current = nullptr;
CtxGetIdFn g_ctx_id = nullptr;

// Id of the context current on this thread; 0 when there is none.
unsigned long long current_context_id()
{
    if (!g_ctx_current || !g_ctx_id) {
        void *f0 = nullptr, *f1 = nullptr;
        cudaDriverEntryPointQueryResult q0, q1;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f0, 12000, cudaEnableDefault, &q0) != cudaSuccess ||
            cudaGetDriverEntryPointByVersion("cuCtxGetId", &f1, 12000, cudaEnableDefault, &q1) != cudaSuccess ||
            q0 != cudaDriverEntryPointSuccess || q1 != cudaDriverEntryPointSuccess) {
            cudaGetLastError();
            return 0;
        }
        g_ctx_current = reinterpret_cast<CtxGetCurrentFn>(f0);
        g_ctx_id = reinterpret_cast<CtxGetIdFn>(f1);
    }
    CUcontext ctx = nullptr;
    unsigned long long id = 0;
    if (g_ctx_current(&ctx) != CUDA_SUCCESS || !ctx || g_ctx_id(ctx, &id) != CUDA_SUCCESS) return 0;
    return id;
}

// Device address of g_noalloc_tris on the current device, looked up on the
// first call with that device current and again whenever the device's
// context has changed since.  The lookup may load the library's module, which
// a stream capture does not allow: a call that needs it while `s` is
// capturing is refused.
int noalloc_scratch(float4 **out, cudaStream_t s)
{
    int dev = -1;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return fail(KDGB_ERR_NO_DEVICE, "kdgb_trace_brute_noalloc: no CUDA device");
    }
    if (dev < 0 || dev >= kMaxDevices) return fail(KDGB_ERR_UNSUPPORTED, "kdgb_trace_brute_noalloc: device id too large");
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    const unsigned long long ctx = current_context_id();
    if (!g_noalloc_addr[dev] || ctx == 0 || ctx != g_noalloc_ctx[dev]) {
        cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
        if (cudaStreamIsCapturing(s, &cap) == cudaSuccess && cap != cudaStreamCaptureStatusNone)
            return fail(KDGB_ERR_UNSUPPORTED,
                        "kdgb_trace_brute_noalloc: the first call on a device (or the first after its context was "
                        "reset) looks up the scratch array and must not be made during stream capture");
        cudaGetLastError();
        void *p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_tris);
        if (e != cudaSuccess) return cuda_fail(e, "kdgb_trace_brute_noalloc: cudaGetSymbolAddress");
        g_noalloc_addr[dev] = static_cast<float4 *>(p);
        g_noalloc_ctx[dev] = current_context_id();
    }
    *out = g_noalloc_addr[dev];
    return KDGB_OK;
}

__global__ void k_noalloc_pack(const float *__restrict__ tri, int32_t T, float4 *__restrict__ rec)
{
    const int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= T) return;
    const float *p = tri + 9 * (int64_t)i;
    const float3 v0 = make_float3(p[0], p[1], p[2]);
    const float3 e1 = sub3(make_float3(p[3], p[4], p[5]), v0);
    const float3 e2 = sub3(make_float3(p[6], p[7], p[8]), v0);
    rec[3 * (int64_t)i + 0] = make_float4(v0.x, v0.y, v0.z, e1.x);
    rec[3 * (int64_t)i + 1] = make_float4(e1.y, e1.z, e2.x, e2.y);
    rec[3 * (int64_t)i + 2] = make_float4(e2.z, __int_as_float(i), 0.0f, 0.0f);
}

// Moeller-Trumbore (IRayTracer.h:111-145) with the library's rounding: every
// product and sum separately rounded, IEEE reciprocal.
__device__ __forceinline__ void noalloc_mt(float4 a, float4 b, float4 c, float3 o, float3 d, int tie, int &hit,
                                           float &tb, float &ub, float &vb)
{
    const float3 v0 = make_float3(a.x, a.y, a.z), e1 = make_float3(a.w, b.x, b.y), e2 = make_float3(b.z, b.w, c.x);
    const int id = __float_as_int(c.y);
    const float3 p = cross3(d, e2);
    const float3 t = sub3(o, v0);
    const float3 q = cross3(t, e1);
    const float inv_det = __frcp_rn(dot3(p, e1));
    const float ht = __fmul_rn(inv_det, dot3(q, e2));
    if (0.0f <= ht && ht <= tb) {
        const float hu = __fmul_rn(inv_det, dot3(p, t));
        const float hv = __fmul_rn(inv_det, dot3(q, d));
        if (hu >= 0.0f && hv >= 0.0f && __fadd_rn(hu, hv) <= 1.0f) {
            if (tie == KDGB_TIE_REF_LAST || hit == -1 || ht < tb || id < hit) {
                hit = id; tb = ht; ub = hu; vb = hv;
            }
        }
    }
}

// BruteTracer.cu:54-96 over the packed records, staged through shared memory.
__global__ void __launch_bounds__(kNoAllocBlock) k_noalloc_brute(const float4 *__restrict__ rec, int32_t T, int tie,
                                                                const float *__restrict__ ro,
                                                                const float *__restrict__ rd, int64_t n,
                                                                int32_t *hit, float *ot, float *ou, float *ov)
{
    __shared__ float4 s[3 * kNoAllocBlock];
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const bool live = i < n;
    float3 o = make_float3(0.f, 0.f, 0.f), d = o;
    if (live) {
        o = make_float3(ro[3 * i], ro[3 * i + 1], ro[3 * i + 2]);
        d = make_float3(rd[3 * i], rd[3 * i + 1], rd[3 * i + 2]);
    }
    int h = -1;
    float tb = KDGB_FINF, ub = 0.0f, vb = 0.0f;
    for (int32_t base = 0; base < T; base += kNoAllocBlock) {
        const int m = min(kNoAllocBlock, T - base);
        for (int k = threadIdx.x; k < 3 * m; k += kNoAllocBlock) s[k] = rec[3 * (int64_t)base + k];
        __syncthreads();
        if (live)
            for (int k = 0; k < m; ++k) noalloc_mt(s[3 * k], s[3 * k + 1], s[3 * k + 2], o, d, tie, h, tb, ub, vb);
        __syncthreads();
    }
    if (!live) return;
    if (tb < KDGB_FINF) {
        hit[i] = h; ot[i] = tb; ou[i] = ub; ov[i] = vb;
    } else {
        hit[i] = -1; ot[i] = INFINITY; ou[i] = 0.0f; ov[i] = 0.0f;
    }
}

}  // namespace
}  // namespace kdgb

using namespace kdgb;

extern "C" int kdgb_trace_brute_noalloc(const float *tri_v_dev, int32_t n_tris, int32_t tie,
                                        const float *ray_o_dev, const float *ray_d_dev, int32_t n, int32_t *hit_dev,
                                        float *t_dev, float *u_dev, float *v_dev, kdgb_stream_t stream)
{
    if (n_tris < 0 || n < 0) return fail(KDGB_ERR_INVALID_ARGUMENT, "kdgb_trace_brute_noalloc: negative count");
    if (n_tris > KDGB_NOALLOC_MAX_TRIS)
        return fail(KDGB_ERR_CAPACITY, "kdgb_trace_brute_noalloc: n_tris " + std::to_string(n_tris) +
                                           " exceeds the static scratch of " + std::to_string(KDGB_NOALLOC_MAX_TRIS) +
                                           " triangles");
    if (tie != KDGB_TIE_LOWEST_ID && tie != KDGB_TIE_REF_LAST)
        return fail(KDGB_ERR_INVALID_ARGUMENT, "kdgb_trace_brute_noalloc: unknown tie rule");
    if (n_tris > 0 && !tri_v_dev) return fail(KDGB_ERR_INVALID_ARGUMENT, "kdgb_trace_brute_noalloc: NULL triangles");
    if (n == 0) return KDGB_OK;
    if (!ray_o_dev || !ray_d_dev || !hit_dev || !t_dev || !u_dev || !v_dev)
        return fail(KDGB_ERR_INVALID_ARGUMENT, "kdgb_trace_brute_noalloc: NULL ray or output buffer");
    cudaStream_t s = (cudaStream_t)stream;
    float4 *rec = nullptr;
    KDGB_CHECK(noalloc_scratch(&rec, s));
    if (n_tris > 0) {
        k_noalloc_pack<<<(n_tris + kNoAllocBlock - 1) / kNoAllocBlock, kNoAllocBlock, 0, s>>>(tri_v_dev, n_tris, rec);
        KDGB_LAUNCH_CHECK();
    }
    k_noalloc_brute<<<(unsigned)((n + kNoAllocBlock - 1) / kNoAllocBlock), kNoAllocBlock, 0, s>>>(
        rec, n_tris, tie, ray_o_dev, ray_d_dev, n, hit_dev, t_dev, u_dev, v_dev);
    KDGB_LAUNCH_CHECK();
    return KDGB_OK;
}
