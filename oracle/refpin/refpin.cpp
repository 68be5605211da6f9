// Single-primitive C entry points over the reference's OWN header-only
// intersection code, compiled unmodified from the reference tree (include
// path) with the host stand-ins of include/.  The oracle's restatements are
// checked against these bit for bit (tests/test_refpin.py).  TEST
// INFRASTRUCTURE ONLY: built into oracle/_ref/, never part of the library.
#include <Utils/CUDA/IRayTracer.h>

using OpenEngine::Utils::CUDA::IRayTracer;

static float3 f3(const float *p) { return make_float3(p[0], p[1], p[2]); }

extern "C" {

// IRayTracer::MoellerTrumbore (IRayTracer.h:111-145, host branch) on one
// triangle; tHit starts at (t_max, 0, 0).  Returns 1 on a hit.
int ref_moeller_trumbore(const float tri[9], const float o[3], const float d[3], float t_max, float out[3])
{
    float4 a = make_float4(f3(tri), 1.0f), b = make_float4(f3(tri + 3), 1.0f), c = make_float4(f3(tri + 6), 1.0f);
    int hit = -1;
    float3 th = make_float3(t_max, 0.0f, 0.0f);
    IRayTracer::MoellerTrumbore(&a, &b, &c, 0, f3(o), f3(d), hit, th);
    out[0] = th.x; out[1] = th.y; out[2] = th.z;
    return hit == 0;
}

// IRayTracer::AdjustRayDirection (IRayTracer.h:60-65), in place.
void ref_adjust_dir(float d[3])
{
    float3 v = f3(d);
    IRayTracer::AdjustRayDirection(v);
    d[0] = v.x; d[1] = v.y; d[2] = v.z;
}

// IRayTracer::RayBoxIntersection<true> (IRayTracer.h:147-168).
int ref_ray_box(const float o[3], const float inv[3], const float bmin[3], const float bmax[3])
{
    return IRayTracer::RayBoxIntersection<true>(f3(o), f3(inv), f3(bmin), f3(bmax)) ? 1 : 0;
}

// WoopTransformationMatrix (IntersectionTests.h:438-467) with the argument
// order of CreateWoopValues (GeometryList.cu:96): (p1, p2, p0).
void ref_woop_rows(const float tri[9], float m[12])
{
    float4 m0, m1, m2;
    WoopTransformationMatrix(f3(tri + 3), f3(tri + 6), f3(tri), m0, m1, m2);
    const float4 r[3] = {m0, m1, m2};
    for (int i = 0; i < 3; ++i) {
        m[4 * i] = r[i].x; m[4 * i + 1] = r[i].y; m[4 * i + 2] = r[i].z; m[4 * i + 3] = r[i].w;
    }
}

// IRayTracer::Woop (IRayTracer.h:78-109) on one triangle's rows.
int ref_woop(const float m[12], const float o[3], const float d[3], float t_max, float out[3])
{
    float4 w0 = make_float4(m[0], m[1], m[2], m[3]), w1 = make_float4(m[4], m[5], m[6], m[7]),
           w2 = make_float4(m[8], m[9], m[10], m[11]);
    int hit = -1;
    float3 th = make_float3(t_max, 0.0f, 0.0f);
    IRayTracer::Woop(&w0, &w1, &w2, 0, f3(o), f3(d), hit, th);
    out[0] = th.x; out[1] = th.y; out[2] = th.z;
    return hit == 0;
}

// TriangleAabbIntersectionStep3 (IntersectionTests.h:378-395).
int ref_tri_box_step3(const float tri[9], const float bmin[3], const float bmax[3])
{
    return TriangleAabbIntersectionStep3(f3(tri), f3(tri + 3), f3(tri + 6), f3(bmin), f3(bmax)) ? 1 : 0;
}

}  // extern "C"
