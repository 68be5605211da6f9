// Adjoint of the first-hit Moeller-Trumbore outputs with respect to the
// vertex positions of an indexed mesh (no counterpart in the reference).
//
// For a ray o + t d hitting triangle (v0, v1, v2) at barycentrics (u, v):
//   o + t d = (1 - u - v) v0 + u v1 + v v2.
// Differentiating with o, d fixed gives J [dt du dv]^T = (1-u-v) dv0 + u dv1
// + v dv2 with J = [d, -e1, -e2].  For upstream gradients g = (gt, gu, gv),
//   lambda = J^-T g = (gt (e1 x e2) + gu (d x e2) - gv (d x e1)) / (d . (e1 x e2))
// and dL/dv0 = (1-u-v) lambda, dL/dv1 = u lambda, dL/dv2 = v lambda.
// The hit ids recorded by the forward trace are reused: nothing is
// re-traversed.  Contributions are summed per vertex with warp-aggregated
// atomics (lanes of a warp that touch the same vertex reduce first), so the
// summation order, and the last bits of the result, vary from run to run.
#include <cuda_runtime.h>

#include "kdgb_internal.cuh"

namespace kdgb {
namespace {

constexpr int kAdjBlock = 128;

__device__ __forceinline__ float3 fma3(float3 acc, float s, float3 v)
{
    return make_float3(__fadd_rn(acc.x, __fmul_rn(s, v.x)), __fadd_rn(acc.y, __fmul_rn(s, v.y)),
                       __fadd_rn(acc.z, __fmul_rn(s, v.z)));
}

// Adds `g` to vertex `vid` (vid < 0: nothing), aggregating lanes of the warp
// that add to the same vertex.
__device__ __forceinline__ void warp_add(float *grad, int vid, float3 g)
{
    const unsigned m = __match_any_sync(0xffffffffu, vid);
    if (vid < 0) return;
    const int leader = __ffs(m) - 1;
    float3 s = make_float3(0.f, 0.f, 0.f);
    for (unsigned mm = m; mm; mm &= mm - 1u) {
        const int src = __ffs(mm) - 1;
        const float x = __shfl_sync(m, g.x, src), y = __shfl_sync(m, g.y, src), z = __shfl_sync(m, g.z, src);
        s.x += x; s.y += y; s.z += z;
    }
    if ((int)(threadIdx.x & 31) == leader) {
        float *p = grad + 3 * (int64_t)vid;
        atomicAdd(p + 0, s.x);
        atomicAdd(p + 1, s.y);
        atomicAdd(p + 2, s.z);
    }
}

__global__ void __launch_bounds__(kAdjBlock) k_backward(const float *__restrict__ verts, int32_t n_verts,
                                                       const unsigned *__restrict__ idx, int32_t n_tris, const float *__restrict__ ro,
                                                       const float *__restrict__ rd, int64_t n,
                                                       const int32_t *__restrict__ hit, const float *__restrict__ gt,
                                                       const float *__restrict__ gu, const float *__restrict__ gv,
                                                       float *__restrict__ grad)
{
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    int h = -1;
    if (i < n) h = hit[i];
    if (h >= n_tris) h = -1;
    int i0 = -1, i1 = -1, i2 = -1;
    float3 g0 = make_float3(0.f, 0.f, 0.f), g1 = g0, g2 = g0;
    if (h >= 0) {
        i0 = (int)idx[3 * (int64_t)h];
        i1 = (int)idx[3 * (int64_t)h + 1];
        i2 = (int)idx[3 * (int64_t)h + 2];
        if ((unsigned)i0 >= (unsigned)n_verts || (unsigned)i1 >= (unsigned)n_verts || (unsigned)i2 >= (unsigned)n_verts)
            h = -1;  // malformed index buffer: skip the ray rather than read out of bounds
    }
    if (h >= 0) {
        const float3 v0 = make_float3(verts[3 * (int64_t)i0], verts[3 * (int64_t)i0 + 1], verts[3 * (int64_t)i0 + 2]);
        const float3 v1 = make_float3(verts[3 * (int64_t)i1], verts[3 * (int64_t)i1 + 1], verts[3 * (int64_t)i1 + 2]);
        const float3 v2 = make_float3(verts[3 * (int64_t)i2], verts[3 * (int64_t)i2 + 1], verts[3 * (int64_t)i2 + 2]);
        const float3 o = make_float3(ro[3 * i], ro[3 * i + 1], ro[3 * i + 2]);
        const float3 d = make_float3(rd[3 * i], rd[3 * i + 1], rd[3 * i + 2]);
        const float3 e1 = sub3(v1, v0), e2 = sub3(v2, v0);
        // u, v of the forward hit (IRayTracer.h:111-145 arithmetic).
        const float3 p = cross3(d, e2);
        const float3 s = sub3(o, v0);
        const float3 q = cross3(s, e1);
        const float inv_det = __frcp_rn(dot3(p, e1));
        const float u = __fmul_rn(inv_det, dot3(p, s));
        const float v = __fmul_rn(inv_det, dot3(q, d));
        const float3 nrm = cross3(e1, e2);
        const float inv_j = __frcp_rn(dot3(d, nrm));  // 1 / det J
        const float3 de2 = cross3(d, e2), de1 = cross3(d, e1);
        float3 lam = make_float3(0.f, 0.f, 0.f);
        lam = fma3(lam, gt[i], nrm);
        lam = fma3(lam, gu[i], de2);
        lam = fma3(lam, -gv[i], de1);
        lam = make_float3(__fmul_rn(lam.x, inv_j), __fmul_rn(lam.y, inv_j), __fmul_rn(lam.z, inv_j));
        const float w0 = __fsub_rn(__fsub_rn(1.0f, u), v);
        g0 = make_float3(__fmul_rn(w0, lam.x), __fmul_rn(w0, lam.y), __fmul_rn(w0, lam.z));
        g1 = make_float3(__fmul_rn(u, lam.x), __fmul_rn(u, lam.y), __fmul_rn(u, lam.z));
        g2 = make_float3(__fmul_rn(v, lam.x), __fmul_rn(v, lam.y), __fmul_rn(v, lam.z));
        if (!(isfinite(g0.x) && isfinite(g0.y) && isfinite(g0.z) && isfinite(g1.x) && isfinite(g1.y) &&
              isfinite(g1.z) && isfinite(g2.x) && isfinite(g2.y) && isfinite(g2.z)))
            i0 = i1 = i2 = -1;  // degenerate geometry (ray parallel to the triangle): no gradient
    }
    warp_add(grad, i0, g0);
    warp_add(grad, i1, g1);
    warp_add(grad, i2, g2);
}

}  // namespace
}  // namespace kdgb

using namespace kdgb;

extern "C" int kdgb_backward(const float *vertices_dev, int32_t n_vertices, const uint32_t *indices_dev,
                             int32_t n_tris, const float *ray_o_dev, const float *ray_d_dev, int32_t n,
                             const int32_t *hit_dev, const float *dL_dt_dev, const float *dL_du_dev,
                             const float *dL_dv_dev, float *dL_dvertex_dev, kdgb_stream_t stream)
{
    if (n_vertices < 0 || n_tris < 0 || n < 0) return fail(KDGB_ERR_INVALID_ARGUMENT, "kdgb_backward: negative count");
    if (n == 0 || n_tris == 0) return KDGB_OK;
    if (!vertices_dev || !indices_dev || !ray_o_dev || !ray_d_dev || !hit_dev || !dL_dt_dev || !dL_du_dev ||
        !dL_dv_dev || !dL_dvertex_dev)
        return fail(KDGB_ERR_INVALID_ARGUMENT, "kdgb_backward: NULL buffer");
    k_backward<<<(unsigned)((n + kAdjBlock - 1) / kAdjBlock), kAdjBlock, 0, (cudaStream_t)stream>>>(
        vertices_dev, n_vertices, indices_dev, n_tris, ray_o_dev, ray_d_dev, n, hit_dev, dL_dt_dev, dL_du_dev, dL_dv_dev,
        dL_dvertex_dev);
    KDGB_LAUNCH_CHECK();
    return KDGB_OK;
}
