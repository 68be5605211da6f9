// The reference's brute-force tracer (Utils/CUDA/BruteTracer.cu, compiled
// unmodified with the stand-ins of include_cu/) called on the host, ray by
// ray, the way BruteTracer::HostTrace does (BruteTracer.cu:174-201).  TEST
// INFRASTRUCTURE ONLY: built into oracle/_ref/, never part of the library.
#include <Utils/CUDA/BruteTracer.cu>

#include "refpin_trace.h"

using namespace OpenEngine::Utils::CUDA;

extern "C" {

// Light of the shading loop (this unit's d_light* symbols).
KDGB_PIN_EXPORT void ref_brute_set_light(const float pos[3], const float amb[3], const float dif[3],
                                         const float spe[3])
{
    KDGB_PIN_SET_LIGHT(pos, amb, dif, spe);
}

// MAX_PRIMS of the compiled unit (BruteTracer.cu:50): Exhaustive tests the
// first min(T, MAX_PRIMS) triangles.
KDGB_PIN_EXPORT int ref_brute_max_prims(void) { return MAX_PRIMS; }

// Exhaustive<woop> (BruteTracer.cu:54-96) on n rays (float4 origins and
// directions) against the scene's triangles.  rgba: n uchar4.
KDGB_PIN_EXPORT void ref_exhaustive(const ref_trace_scene *s, int woop, const float *o4, const float *d4, int n,
                                    uint8_t *rgba)
{
    KdgbPinTriangles v(s, woop);
    float4 *o = (float4 *)o4, *d = (float4 *)d4;
    for (int i = 0; i < n; ++i) {
        const uchar4 c = woop ? Exhaustive<true>(i, o, d, v.v0, v.v1, v.v2, (float4 *)s->n0, (float4 *)s->n1,
                                                 (float4 *)s->n2, (uchar4 *)s->c0, s->n_tris)
                              : Exhaustive<false>(i, o, d, v.v0, v.v1, v.v2, (float4 *)s->n0, (float4 *)s->n1,
                                                  (float4 *)s->n2, (uchar4 *)s->c0, s->n_tris);
        rgba[4 * i] = c.x; rgba[4 * i + 1] = c.y; rgba[4 * i + 2] = c.z; rgba[4 * i + 3] = c.w;
    }
}

}  // extern "C"
