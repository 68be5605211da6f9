// Geometry collection and the animated height field.
//
// kdgb_geometry_gather restates AddMeshKernel (Utils/CUDA/GeometryList.cu:
// 197-232, the float4 variant used for CUDAMeshNode): per triangle, gather the
// three vertices through the index buffer and transform them by the model
// matrix, Matrix44f * float4 = four row dot products (Math/CUDA/Matrix.h:
// 41-47), each summed left to right.  The output is the T x 9 triangle buffer
// kdgb_build consumes.
//
// kdgb_geometry_gather_attributes is its normal and colour half (n0/n1/n2
// and c0 of the GeometryList, GeometryList.cu:224-230), which the shading
// loop reads.
//
// kdgb_osc_update_surface restates UpdateSurface of OscCUDAMeshNode
// (Scene/OscCUDAMeshNode.cu:75-94): heights and normals of the oscillating
// grid for one time value.
#include <cuda_runtime.h>

#include "kdgb_internal.cuh"

namespace kdgb {
namespace {

constexpr int kGeoBlock = 128;

struct Mat44 {
    float m[16];  // row major
};

__device__ __forceinline__ float dot4(const float *r, float4 v)
{
    float s = __fmul_rn(r[0], v.x);
    s = __fadd_rn(s, __fmul_rn(r[1], v.y));
    s = __fadd_rn(s, __fmul_rn(r[2], v.z));
    s = __fadd_rn(s, __fmul_rn(r[3], v.w));
    return s;
}

__global__ void k_gather(const float4 *__restrict__ verts, int32_t n_verts, const unsigned *__restrict__ idx,
                         int32_t n_tris, Mat44 M, float *__restrict__ out)
{
    const int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_tris) return;
    float *o = out + 9 * (int64_t)i;
    for (int k = 0; k < 3; ++k) {
        const unsigned vi = idx[3 * (int64_t)i + k];
        if (vi >= (unsigned)n_verts) {
            // An index outside the vertex buffer makes the triangle NaN, so a
            // following kdgb_build reports KDGB_ERR_NONFINITE instead of
            // reading out of bounds here.
            o[3 * k] = o[3 * k + 1] = o[3 * k + 2] = __int_as_float(0x7fc00000);
            continue;
        }
        const float4 v = verts[vi];
        o[3 * k + 0] = dot4(M.m + 0, v);
        o[3 * k + 1] = dot4(M.m + 4, v);
        o[3 * k + 2] = dot4(M.m + 8, v);
    }
}

struct Mat33 {
    float m[9];  // row major
};

// The normal and colour half of AddMeshKernel: per triangle, the three
// vertex normals times the normal matrix (three row dot products, left to
// right, w = 0) and the first vertex's colour.  An index outside the vertex
// buffer gives NaN normals and a zero colour.
__global__ void k_gather_attributes(const float4 *__restrict__ normals, const uchar4 *__restrict__ colors,
                                    int32_t n_verts, const unsigned *__restrict__ idx, int32_t n_tris, Mat33 N,
                                    float4 *__restrict__ n0, float4 *__restrict__ n1, float4 *__restrict__ n2,
                                    uchar4 *__restrict__ c0)
{
    const int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_tris) return;
    float4 *outs[3] = {n0, n1, n2};
    for (int k = 0; k < 3; ++k) {
        const unsigned vi = idx[3 * (int64_t)i + k];
        if (vi >= (unsigned)n_verts) {
            const float nan = __int_as_float(0x7fc00000);
            outs[k][i] = make_float4(nan, nan, nan, 0.0f);
            if (k == 0) c0[i] = make_uchar4(0, 0, 0, 0);
            continue;
        }
        const float4 v = normals[vi];
        float r[3];
        for (int row = 0; row < 3; ++row) {
            float s = __fmul_rn(N.m[3 * row + 0], v.x);
            s = __fadd_rn(s, __fmul_rn(N.m[3 * row + 1], v.y));
            r[row] = __fadd_rn(s, __fmul_rn(N.m[3 * row + 2], v.z));
        }
        outs[k][i] = make_float4(r[0], r[1], r[2], 0.0f);
        if (k == 0) c0[i] = colors[vi];
    }
}

// OscCUDAMeshNode.cu:69-70 amplitude and frequency.
constexpr float kAmplitude = 0.2f;
constexpr float kFrequency = 0.3f;

__global__ void k_osc(float4 *__restrict__ vert, float4 *__restrict__ norm, int32_t d, float height, float time)
{
    const int x = blockDim.x * blockIdx.x + threadIdx.x;
    const int y = blockDim.y * blockIdx.y + threadIdx.y;
    if (x >= d || y >= d) return;
    const int id = y * d + x;
    float4 v = vert[id];
    const float ax = __fadd_rn(__fmul_rn(kFrequency, (float)x), time);
    const float ay = __fadd_rn(__fmul_rn(kFrequency, (float)y), time);
    v.y = __fadd_rn(height, __fmul_rn(kAmplitude, cosf(ax)));
    v.y = __fadd_rn(v.y, __fmul_rn(kAmplitude, sinf(ay)));
    vert[id] = v;
    float4 n;
    n.x = __fmul_rn(__fmul_rn(-kAmplitude, sinf(ax)), kFrequency);
    n.z = __fmul_rn(__fmul_rn(kAmplitude, cosf(ay)), kFrequency);
    n.y = __fsub_rn(__fsub_rn(1.0f, __fmul_rn(n.x, n.x)), __fmul_rn(n.z, n.z));
    n.w = 0.0f;
    norm[id] = n;
}

}  // namespace
}  // namespace kdgb

using namespace kdgb;

extern "C" int kdgb_geometry_gather(const float *vertices_dev, int32_t n_vertices, const uint32_t *indices_dev,
                                    int32_t n_indices, const float model[16], float *tri_v_out_dev,
                                    kdgb_stream_t stream)
{
    if (n_vertices < 0 || n_indices < 0 || n_indices % 3 != 0)
        return fail(KDGB_ERR_INVALID_ARGUMENT, "kdgb_geometry_gather: index count must be a multiple of 3");
    const int32_t n_tris = n_indices / 3;
    if (n_tris == 0) return KDGB_OK;
    if (!vertices_dev || !indices_dev || !tri_v_out_dev)
        return fail(KDGB_ERR_INVALID_ARGUMENT, "kdgb_geometry_gather: NULL buffer");
    Mat44 M;
    for (int k = 0; k < 16; ++k) M.m[k] = model ? model[k] : (k % 5 == 0 ? 1.0f : 0.0f);
    k_gather<<<(n_tris + kGeoBlock - 1) / kGeoBlock, kGeoBlock, 0, (cudaStream_t)stream>>>(
        reinterpret_cast<const float4 *>(vertices_dev), n_vertices, indices_dev, n_tris, M, tri_v_out_dev);
    KDGB_LAUNCH_CHECK();
    return KDGB_OK;
}

extern "C" int kdgb_osc_update_surface(float *vertices_dev, float *normals_dev, int32_t detail, float height,
                                       float time, kdgb_stream_t stream)
{
    if (detail < 1 || detail > 16384) return fail(KDGB_ERR_INVALID_ARGUMENT, "kdgb_osc_update_surface: bad detail");
    if (!vertices_dev || !normals_dev) return fail(KDGB_ERR_INVALID_ARGUMENT, "kdgb_osc_update_surface: NULL buffer");
    // OscCUDAMeshNode.cu:99-106 sizes the grid from `detail` but passes
    // detail + 1 as the bound, so when detail is a multiple of 16 the last
    // row and column of vertices are not updated; kept as is.
    const int d = detail + 1;
    const dim3 block(16, 16, 1);
    const dim3 grid((detail + 15) / 16, (detail + 15) / 16, 1);
    k_osc<<<grid, block, 0, (cudaStream_t)stream>>>(reinterpret_cast<float4 *>(vertices_dev),
                                                    reinterpret_cast<float4 *>(normals_dev), d, height, time);
    KDGB_LAUNCH_CHECK();
    return KDGB_OK;
}

extern "C" int kdgb_geometry_gather_attributes(const float *normals_dev, const uint8_t *colors_dev, int32_t n_vertices,
                                               const uint32_t *indices_dev, int32_t n_indices,
                                               const float normal_matrix[9], float *n0_out_dev, float *n1_out_dev,
                                               float *n2_out_dev, uint8_t *c0_out_dev, kdgb_stream_t stream)
{
    if (n_vertices < 0 || n_indices < 0 || n_indices % 3 != 0)
        return fail(KDGB_ERR_INVALID_ARGUMENT, "kdgb_geometry_gather_attributes: index count must be a multiple of 3");
    const int32_t n_tris = n_indices / 3;
    if (n_tris == 0) return KDGB_OK;
    if (!normals_dev || !colors_dev || !indices_dev || !n0_out_dev || !n1_out_dev || !n2_out_dev || !c0_out_dev)
        return fail(KDGB_ERR_INVALID_ARGUMENT, "kdgb_geometry_gather_attributes: NULL buffer");
    Mat33 N;
    for (int k = 0; k < 9; ++k) N.m[k] = normal_matrix ? normal_matrix[k] : (k % 4 == 0 ? 1.0f : 0.0f);
    k_gather_attributes<<<(n_tris + kGeoBlock - 1) / kGeoBlock, kGeoBlock, 0, (cudaStream_t)stream>>>(
        reinterpret_cast<const float4 *>(normals_dev), reinterpret_cast<const uchar4 *>(colors_dev), n_vertices,
        indices_dev, n_tris, N, reinterpret_cast<float4 *>(n0_out_dev), reinterpret_cast<float4 *>(n1_out_dev),
        reinterpret_cast<float4 *>(n2_out_dev), reinterpret_cast<uchar4 *>(c0_out_dev));
    KDGB_LAUNCH_CHECK();
    return KDGB_OK;
}
