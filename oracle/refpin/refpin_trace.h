// Shared by the tracer pin units (refpin_restart.cu, refpin_shortstack.cu,
// refpin_brute.cu): the scene a pin call traverses, as plain host arrays in
// the reference's layouts (Scene/KDNode.h, Utils/CUDA/GeometryList.h), and
// the Woop rows GeometryList::GetWoopValues would make for it.  TEST
// INFRASTRUCTURE ONLY.
#pragma once
#include <cstdint>
#include <vector>

// The units compile with hidden visibility and section garbage collection, so
// that the reference's host methods the pin never calls (and the OpenEngine
// symbols they name) drop out of the library; the pin entry points are
// exported explicitly.
#define KDGB_PIN_EXPORT __attribute__((visibility("default")))

extern "C" {
typedef struct ref_trace_scene {
    int32_t n_nodes;
    const int8_t *info;          // KDNode.h:65
    const float *split;          // KDNode.h:66
    const int32_t *children;     // KDNode.h:73, int2 per node
    const int32_t *prim_index;   // KDNode.h:68
    const int32_t *bitmap;       // KDNode.h:69
    const float *aabb_min;       // KDNode.h:67, float4 per node
    const float *aabb_max;
    const int32_t *prim_indices; // TriangleMap.h:55
    int32_t n_tris;
    const float *p0, *p1, *p2;   // GeometryList.h:41, float4 per triangle
    const float *n0, *n1, *n2;   // float4 vertex normals
    const uint8_t *c0;           // uchar4 colours
} ref_trace_scene;
}

// The vertex or Woop rows a tracer template reads: the positions, or
// WoopTransformationMatrix(p1, p2, p0) per triangle as CreateWoopValues
// computes them (GeometryList.cu:83-102), run here on the host.
struct KdgbPinTriangles {
    std::vector<float4> a, b, c;
    float4 *v0, *v1, *v2;
    KdgbPinTriangles(const ref_trace_scene *s, int woop) : a(), b(), c()
    {
        const float4 *p0 = (const float4 *)s->p0, *p1 = (const float4 *)s->p1, *p2 = (const float4 *)s->p2;
        if (!woop) {
            v0 = const_cast<float4 *>(p0);
            v1 = const_cast<float4 *>(p1);
            v2 = const_cast<float4 *>(p2);
            return;
        }
        a.resize(s->n_tris); b.resize(s->n_tris); c.resize(s->n_tris);
        for (int i = 0; i < s->n_tris; ++i)
            WoopTransformationMatrix(make_float3(p1[i]), make_float3(p2[i]), make_float3(p0[i]), a[i], b[i], c[i]);
        v0 = a.data(); v1 = b.data(); v2 = c.data();
    }
};

// The light of the tracers' constructors (Raytracer.cu:43-51,
// ShortStack.cu:42-50, BruteTracer.cu:34-42), or the caller's.
#define KDGB_PIN_SET_LIGHT(pos, amb, dif, spe)                                   \
    do {                                                                          \
        float3 v_[4] = {make_float3(pos[0], pos[1], pos[2]), make_float3(amb[0], amb[1], amb[2]), \
                        make_float3(dif[0], dif[1], dif[2]), make_float3(spe[0], spe[1], spe[2])}; \
        cudaMemcpyToSymbol(d_lightPosition, &v_[0], sizeof(float3));             \
        cudaMemcpyToSymbol(d_lightAmbient, &v_[1], sizeof(float3));              \
        cudaMemcpyToSymbol(d_lightDiffuse, &v_[2], sizeof(float3));              \
        cudaMemcpyToSymbol(d_lightSpecular, &v_[3], sizeof(float3));             \
    } while (0)
