// The reference's kd-restart tracer (Utils/CUDA/Raytracer.cu, compiled
// unmodified with the stand-ins of include_cu/) called on the host, ray by
// ray, the way RayTracer::HostTrace does (Raytracer.cu:392-458).  TEST
// INFRASTRUCTURE ONLY: built into oracle/_ref/, never part of the library.
#include <Utils/CUDA/Raytracer.cu>

#include "refpin_trace.h"

using namespace OpenEngine::Utils::CUDA;
using OpenEngine::Scene::KDNode;

namespace {
template <bool woop, bool skip>
uchar4 restart_one(int id, float4 *o, float4 *d, const ref_trace_scene *s, KdgbPinTriangles &v)
{
    return KDRestart<woop, true, skip>(
        id, o, d, (char *)s->info, (float *)s->split, (int2 *)s->children, (int *)s->prim_index,
        (KDNode::bitmap *)s->bitmap, (float4 *)s->aabb_min, (float4 *)s->aabb_max, (int *)s->prim_indices, v.v0, v.v1,
        v.v2, (float4 *)s->n0, (float4 *)s->n1, (float4 *)s->n2, (uchar4 *)s->c0);
}

template <bool woop>
float shadow_one(float3 point, float3 light, const ref_trace_scene *s, KdgbPinTriangles &v)
{
    return ShadowRay<woop, true>(point, light, (char *)s->info, (float *)s->split, (int *)s->prim_index,
                                 (KDNode::bitmap *)s->bitmap, (int2 *)s->children, (int *)s->prim_indices, v.v0,
                                 v.v1, v.v2);
}
}  // namespace

extern "C" {

// Light of the shading loop (d_lightPosition, d_lightAmbient, d_lightDiffuse,
// d_lightSpecular of this unit).
KDGB_PIN_EXPORT void ref_restart_set_light(const float pos[3], const float amb[3], const float dif[3], const float spe[3])
{
    KDGB_PIN_SET_LIGHT(pos, amb, dif, spe);
}

// KDRestart<woop, invDir = true, leaf_skipping> (Raytracer.cu:165-262), the
// template arguments RayTracer::Trace uses, on n rays (origins and
// directions float4).  rgba: n uchar4.  For each ray, first_prim / first_thit
// are the primitive and tHit (t, u, v) its first hit logged
// (Raytracer.cu:226, 230), -1 when it hit nothing.
KDGB_PIN_EXPORT void ref_kdrestart(const ref_trace_scene *s, int woop, int leaf_skipping, const float *o4, const float *d4, int n,
                   uint8_t *rgba, int32_t *first_prim, float *first_thit)
{
    KdgbPinTriangles v(s, woop);
    float4 *o = (float4 *)o4, *d = (float4 *)d4;
    for (int i = 0; i < n; ++i) {
        kdgb_pin_observe_reset();
        uchar4 c;
        if (woop)
            c = leaf_skipping ? restart_one<true, true>(i, o, d, s, v) : restart_one<true, false>(i, o, d, s, v);
        else
            c = leaf_skipping ? restart_one<false, true>(i, o, d, s, v) : restart_one<false, false>(i, o, d, s, v);
        rgba[4 * i] = c.x; rgba[4 * i + 1] = c.y; rgba[4 * i + 2] = c.z; rgba[4 * i + 3] = c.w;
        const KdgbPinObserved &ob = kdgb_pin_observed;
        first_prim[i] = ob.have_first ? ob.first_prim : -1;
        first_thit[3 * i] = ob.first_thit.x;
        first_thit[3 * i + 1] = ob.first_thit.y;
        first_thit[3 * i + 2] = ob.first_thit.z;
    }
}

// ShadowRay<woop, invDir = true> (Raytracer.cu:108-163) from the light to
// each point: lit[i] is its 1 (lit) or 0 (in shadow).
KDGB_PIN_EXPORT void ref_shadow(const ref_trace_scene *s, int woop, const float *points, int n, const float light[3], float *lit)
{
    KdgbPinTriangles v(s, woop);
    const float3 l = make_float3(light[0], light[1], light[2]);
    for (int i = 0; i < n; ++i) {
        const float3 p = make_float3(points[3 * i], points[3 * i + 1], points[3 * i + 2]);
        lit[i] = woop ? shadow_one<true>(p, l, s, v) : shadow_one<false>(p, l, s, v);
    }
}

}  // extern "C"
