// The reference's short-stack tracer (Utils/CUDA/ShortStack.cu, compiled
// unmodified with the stand-ins of include_cu/) called on the host, ray by
// ray, the way ShortStack::HostTrace does (ShortStack.cu:323-355): a local
// stack of SHORT_STACK_SIZE elements per ray.  TEST INFRASTRUCTURE ONLY:
// built into oracle/_ref/, never part of the library.
#include <Utils/CUDA/ShortStack.cu>

#include "refpin_trace.h"

using namespace OpenEngine::Utils::CUDA;
using OpenEngine::Scene::KDNode;

namespace {
template <bool woop, bool skip>
uchar4 shortstack_one(int id, float4 *o, float4 *d, const ref_trace_scene *s, KdgbPinTriangles &v)
{
    ShortStack::Element elms[SHORT_STACK_SIZE];
    return ShortStackTrace<woop, true, skip>(
        id, o, d, elms, (char *)s->info, (float *)s->split, (int2 *)s->children, (int *)s->prim_index,
        (KDNode::bitmap *)s->bitmap, (float4 *)s->aabb_min, (float4 *)s->aabb_max, (int *)s->prim_indices, v.v0, v.v1,
        v.v2, (float4 *)s->n0, (float4 *)s->n1, (float4 *)s->n2, (uchar4 *)s->c0);
}
}  // namespace

extern "C" {

// Light of the shading loop (this unit's d_light* symbols).
KDGB_PIN_EXPORT void ref_shortstack_set_light(const float pos[3], const float amb[3], const float dif[3],
                                              const float spe[3])
{
    KDGB_PIN_SET_LIGHT(pos, amb, dif, spe);
}

// SHORT_STACK_SIZE of the compiled unit (ShortStack.cu:25).
KDGB_PIN_EXPORT int ref_shortstack_depth(void) { return SHORT_STACK_SIZE; }

// ShortStackTrace<woop, invDir = true, leaf_skipping> (ShortStack.cu:96-194),
// the template arguments ShortStack::Trace uses, on n rays (float4 origins
// and directions).  rgba: n uchar4.  last_thit: the tHit (t, u, v) the ray
// logged after its last leaf (ShortStack.cu:169).
KDGB_PIN_EXPORT void ref_shortstack(const ref_trace_scene *s, int woop, int leaf_skipping, const float *o4,
                                    const float *d4, int n, uint8_t *rgba, float *last_thit)
{
    KdgbPinTriangles v(s, woop);
    float4 *o = (float4 *)o4, *d = (float4 *)d4;
    for (int i = 0; i < n; ++i) {
        kdgb_pin_observe_reset();
        uchar4 c;
        if (woop)
            c = leaf_skipping ? shortstack_one<true, true>(i, o, d, s, v) : shortstack_one<true, false>(i, o, d, s, v);
        else
            c = leaf_skipping ? shortstack_one<false, true>(i, o, d, s, v)
                              : shortstack_one<false, false>(i, o, d, s, v);
        rgba[4 * i] = c.x; rgba[4 * i + 1] = c.y; rgba[4 * i + 2] = c.z; rgba[4 * i + 3] = c.w;
        last_thit[3 * i] = kdgb_pin_observed.last_thit.x;
        last_thit[3 * i + 1] = kdgb_pin_observed.last_thit.y;
        last_thit[3 * i + 2] = kdgb_pin_observed.last_thit.z;
    }
}

}  // extern "C"
