/*
 * kdgb_oracle.c -- CPU restatement of the reference kd-tree build and ray
 * traversal.  TEST INFRASTRUCTURE: the checker for the CUDA library and the
 * timed CPU baseline; never linked into the product.  The intersection
 * primitives, the upper and lower creators, the three tracers with the
 * shading loop and the shadow rays are pinned bit for bit to the reference's
 * own code, compiled unmodified and run on the host (oracle/refpin).  Every
 * function cites the reference lines it restates.
 *
 * Build: gcc -O3 -ffp-contract=off -fopenmp -fPIC -shared (see Makefile).
 * -ffp-contract=off keeps every multiply and add separately rounded, the
 * evaluation order the CUDA kernels use as well.
 */
#include "kdgb_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define OR_ERR_ARG      (-1)
#define OR_ERR_ALLOC    (-2)
#define OR_ERR_LEVELS   (-3)
#define OR_ERR_SPLIT    (-4)
#define OR_ERR_NONFINITE (-5)

const char *or_error_string(int code)
{
    switch (code) {
    case 0: return "ok";
    case OR_ERR_ARG: return "invalid argument";
    case OR_ERR_ALLOC: return "allocation failed";
    case OR_ERR_LEVELS: return "upper build exceeded max_levels (degenerate input)";
    case OR_ERR_SPLIT: return "split produced fewer references than its input";
    case OR_ERR_NONFINITE: return "non-finite vertex coordinate";
    default: return "unknown error";
    }
}

typedef struct { float x, y, z; } v3;
typedef struct { float x, y, z, w; } f4;

static inline float i2f(int32_t i) { float f; memcpy(&f, &i, 4); return f; }
static inline int32_t f2i(float f) { int32_t i; memcpy(&i, &f, 4); return i; }

/* min / max as used by the reference (CUDA fminf/fmaxf on finite data).  Ties
 * between -0 and +0 are resolved by IEEE totalOrder (-0 < +0) so the result
 * does not depend on reduction order; the CUDA kernels use the same order. */
static inline float kmin(float a, float b)
{
    if (a < b) return a;
    if (b < a) return b;
    return signbit(a) ? a : b;
}
static inline float kmax(float a, float b)
{
    if (a > b) return a;
    if (b > a) return b;
    return signbit(a) ? b : a;
}

static inline v3 mk3(float x, float y, float z) { v3 r = {x, y, z}; return r; }
static inline v3 sub3(v3 a, v3 b) { return mk3(a.x - b.x, a.y - b.y, a.z - b.z); }
/* Evaluation order of the un-vendored CUDA-SDK helpers: left to right. */
static inline float dot3(v3 a, v3 b)
{
    float s = a.x * b.x;
    s = s + a.y * b.y;
    s = s + a.z * b.z;
    return s;
}
static inline v3 cross3(v3 a, v3 b)
{
    return mk3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
static inline v3 ld3(const float *p) { return mk3(p[0], p[1], p[2]); }

/* ------------------------------------------------------------------------ */
/* Intersection primitives                                                   */
/* ------------------------------------------------------------------------ */

/* IRayTracer.h:60-65 AdjustRayDirection. */
static inline v3 adjust_dir(v3 d)
{
    const float ooeps = 0x1p-80f; /* exp2f(-80.0) */
    d.x = fabsf(d.x) > ooeps ? d.x : copysignf(ooeps, d.x);
    d.y = fabsf(d.y) > ooeps ? d.y : copysignf(ooeps, d.y);
    d.z = fabsf(d.z) > ooeps ? d.z : copysignf(ooeps, d.z);
    return d;
}

static inline v3 inv3(v3 d) { return mk3(1.0f / d.x, 1.0f / d.y, 1.0f / d.z); }

/* IRayTracer.h:111-145 MoellerTrumbore, host branch (IEEE 1.0f/x).  `tie`
 * selects the reference's `t <= tBest` (last tested wins) or lowest id. */
static inline void mt_test(const float *tri, int prim, v3 o, v3 d, int tie,
                           int *prim_hit, float th[3])
{
    const float *tp = tri + (size_t)prim * 9;
    const v3 v0 = ld3(tp), v1 = ld3(tp + 3), v2 = ld3(tp + 6);
    const v3 e1 = sub3(v1, v0);
    const v3 e2 = sub3(v2, v0);
    const v3 p = cross3(d, e2);
    const v3 t = sub3(o, v0);
    const v3 q = cross3(t, e1);
    const float inv_det = 1.0f / dot3(p, e1);
    const float ht = inv_det * dot3(q, e2);
    if (0.0f <= ht && ht <= th[0]) {
        const float hu = inv_det * dot3(p, t);
        const float hv = inv_det * dot3(q, d);
        if (hu >= 0.0f && hv >= 0.0f && hu + hv <= 1.0f) {
            if (tie == OR_TIE_REF_LAST || *prim_hit == -1 || ht < th[0] || prim < *prim_hit) {
                *prim_hit = prim;
                th[0] = ht; th[1] = hu; th[2] = hv;
            }
        }
    }
}

/* WoopTransformationMatrix (IntersectionTests.h:438-467) of (p1, p2, p0) as
 * CreateWoopValues (GeometryList.cu:81-102) calls it: the inverse of the
 * matrix whose columns are a - c, b - c and (a - c) x (b - c) - c, rows scaled
 * by 1/det, each row's w = row . c. */
static void woop_rows(const float *tri, int prim, f4 m[3])
{
    const float *tp = tri + (size_t)prim * 9;
    const v3 c = ld3(tp), a = ld3(tp + 3), b = ld3(tp + 6);
    const v3 m0 = sub3(a, c), m1 = sub3(b, c), m2 = sub3(cross3(m0, m1), c);
    const float det = (m0.x * (m1.y * m2.z - m1.z * m2.y) + m1.x * (m2.y * m0.z - m2.z * m0.y)) +
                      m2.x * (m0.y * m1.z - m0.z * m1.y);
    const float inv = 1.0f / det;
    const v3 r0 = mk3((m1.y * m2.z - m1.z * m2.y) * inv, (m2.x * m1.z - m2.z * m1.x) * inv,
                      (m1.x * m2.y - m1.y * m2.x) * inv);
    const v3 r1 = mk3((m2.y * m0.z - m2.z * m0.y) * inv, (m0.x * m2.z - m0.z * m2.x) * inv,
                      (m2.x * m0.y - m2.y * m0.x) * inv);
    const v3 r2 = mk3((m0.y * m1.z - m0.z * m1.y) * inv, (m1.x * m0.z - m1.z * m0.x) * inv,
                      (m0.x * m1.y - m0.y * m1.x) * inv);
    const f4 w0 = {r0.x, r0.y, r0.z, dot3(r0, c)}, w1 = {r1.x, r1.y, r1.z, dot3(r1, c)},
             w2 = {r2.x, r2.y, r2.z, dot3(r2, c)};
    m[0] = w0; m[1] = w1; m[2] = w2;
}

/* Woop (IRayTracer.h:78-109): lambda = -(m2.o - m2.w) / (m2.d),
 * u = lambda (m0.d) + m0.o - m0.w, v likewise with m1. */
static inline void woop_test(const float *tri, int prim, v3 o, v3 d, int tie, int *prim_hit, float th[3])
{
    f4 m[3];
    woop_rows(tri, prim, m);
    const v3 n2 = mk3(m[2].x, m[2].y, m[2].z);
    const float lambda = -(dot3(n2, o) - m[2].w) / dot3(n2, d);
    if (0.0f <= lambda && lambda <= th[0]) {
        const v3 n0 = mk3(m[0].x, m[0].y, m[0].z), n1 = mk3(m[1].x, m[1].y, m[1].z);
        const float hu = (lambda * dot3(n0, d) + dot3(n0, o)) - m[0].w;
        const float hv = (lambda * dot3(n1, d) + dot3(n1, o)) - m[1].w;
        if (hu >= -0.0f && hv >= -0.0f && hu + hv <= 1.0f) {
            if (tie == OR_TIE_REF_LAST || *prim_hit == -1 || lambda < th[0] || prim < *prim_hit) {
                *prim_hit = prim;
                th[0] = lambda; th[1] = hu; th[2] = hv;
            }
        }
    }
}

static inline void isect(int woop, const float *tri, int prim, v3 o, v3 d, int tie, int *prim_hit, float th[3])
{
    if (woop) woop_test(tri, prim, o, d, tie, prim_hit, th);
    else mt_test(tri, prim, o, d, tie, prim_hit, th);
}

int or_moeller_trumbore(const float v0[3], const float v1[3], const float v2[3],
                        const float o[3], const float d[3], float t_max, float out[3])
{
    float tri[9];
    memcpy(tri, v0, 12); memcpy(tri + 3, v1, 12); memcpy(tri + 6, v2, 12);
    float th[3] = {t_max, 0.0f, 0.0f};
    int hit = -1;
    mt_test(tri, 0, ld3(o), ld3(d), OR_TIE_REF_LAST, &hit, th);
    out[0] = th[0]; out[1] = th[1]; out[2] = th[2];
    return hit == 0;
}

/* IRayTracer.h:147-168 RayBoxIntersection<true>. */
static inline int ray_box(v3 o, v3 inv, const float *bmin, const float *bmax)
{
    v3 lo = mk3((bmin[0] - o.x) * inv.x, (bmin[1] - o.y) * inv.y, (bmin[2] - o.z) * inv.z);
    v3 hi = mk3((bmax[0] - o.x) * inv.x, (bmax[1] - o.y) * inv.y, (bmax[2] - o.z) * inv.z);
    float n = kmin(lo.x, hi.x);
    n = kmax(n, kmin(lo.y, hi.y));
    n = kmax(n, kmin(lo.z, hi.z));
    float f = kmax(hi.x, lo.x);
    f = kmin(f, kmax(lo.y, hi.y));
    f = kmin(f, kmax(lo.z, hi.z));
    return n <= f;
}

static inline float axis_of(v3 a, int axis)
{
    return axis == OR_X ? a.x : (axis == OR_Y ? a.y : a.z);
}

/* ------------------------------------------------------------------------ */
/* Tracers                                                                   */
/* ------------------------------------------------------------------------ */

static inline void write_miss(int32_t i, int32_t *hit, float *t, float *u, float *v)
{
    hit[i] = -1; t[i] = INFINITY; u[i] = 0.0f; v[i] = 0.0f;
}

/* Leaf test shared by the kd tracers: bitmap order LSB first (Utils.h:198-204,
 * Raytracer.cu:199-215). */
static inline int leaf_test(const or_tree *tr, const float *tri, int node, v3 o, v3 d,
                            int tie, int woop, float th[3])
{
    const int pi = tr->prim_index[node];
    uint32_t bm = (uint32_t)tr->bitmap[node];
    int prim_hit = -1;
    while (bm) {
        const int i = __builtin_ctz(bm);
        const int prim = tr->prim_indices[pi + i];
        isect(woop, tri, prim, o, d, tie, &prim_hit, th);
        bm &= bm - 1u;
    }
    return prim_hit;
}

/* Raytracer.cu:57-106 TraceNode<true> + Raytracer.cu:165-262 KDRestart,
 * stopped at the first leaf that reports a hit (shading left out). */
static void trace_restart_one(const or_tree *tr, const float *tri, const or_trace_params *p,
                              v3 o, v3 din, int32_t *hit, float *ot, float *ou, float *ov, v3 *dused)
{
    const v3 d = adjust_dir(din);
    const v3 inv = inv3(d);
    float th[3] = {0.0f, 0.0f, 0.0f};
    long iters = 0;
    if (dused) *dused = d;
    do {
        float t_next = OR_FINF;
        int node = 0;
        int8_t axis = tr->info[0];
        while ((axis & 3) != OR_LEAF) {
            const float sv = tr->split[node];
            const int l = tr->children[2 * node], r = tr->children[2 * node + 1];
            const float ori = axis_of(o, axis), dir = axis_of(inv, axis);
            const float t_split = (sv - ori) * dir;
            if (th[0] < t_split) {
                node = 0 < dir ? l : r;
                t_next = kmin(t_split, t_next);
            } else {
                node = 0 < dir ? r : l;
            }
            axis = tr->info[node];
        }
        th[0] = t_next * 1.00001f;
        if (!p->leaf_skipping || ray_box(o, inv, tr->aabb_min + 4 * (size_t)node,
                                          tr->aabb_max + 4 * (size_t)node)) {
            const int h = leaf_test(tr, tri, node, o, d, p->tie, p->intersection, th);
            if (h != -1) { *hit = h; *ot = th[0]; *ou = th[1]; *ov = th[2]; return; }
        }
        if (p->max_iterations > 0 && ++iters >= p->max_iterations) break;
    } while (th[0] < OR_FINF);
    *hit = -1; *ot = INFINITY; *ou = 0.0f; *ov = 0.0f;
}

/* ShortStack.h:27-98 ring buffer; ShortStack.cu:58-194 TraceNode and
 * ShortStackTrace, first hit.  The direction is inverted in place before the
 * descent and re-inverted after it, every outer iteration (ShortStack.cu:134,148). */
static void trace_shortstack_one(const or_tree *tr, const float *tri, const or_trace_params *p,
                                 v3 o, v3 din, int32_t *hit, float *ot, float *ou, float *ov, v3 *dused)
{
    enum { MAXN = 64 };
    int sn[MAXN]; float st[MAXN];
    const int N = p->stack_depth;
    int nxt = 0, cnt = 0;
    v3 d = adjust_dir(din);
    float th[3] = {0.0f, 0.0f, 0.0f};
    long iters = 0;
    do {
        int node; float t_next;
        if (cnt == 0) {
            node = 0; t_next = OR_FINF;
        } else {
            nxt = (nxt == 0 ? N : nxt) - 1;
            cnt--;
            node = sn[nxt]; t_next = st[nxt];
        }
        int8_t info = tr->info[node];
        d = inv3(d);
        while ((info & 3) != OR_LEAF) {
            const float sv = tr->split[node];
            const int l = tr->children[2 * node], r = tr->children[2 * node + 1];
            const int axis = info & 3;
            const float ori = axis_of(o, axis), dir = axis_of(d, axis);
            const float t_split = (sv - ori) * dir;
            const int lower = 0 < dir ? l : r;
            const int upper = 0 < dir ? r : l;
            if (th[0] < t_split) {
                node = lower;
                if (t_split < t_next) {
                    sn[nxt] = upper; st[nxt] = t_next;
                    nxt = nxt == N - 1 ? 0 : nxt + 1;
                    cnt = cnt == N ? N : cnt + 1;
                }
                t_next = kmin(t_split, t_next);
            } else {
                node = upper;
            }
            info = tr->info[node];
        }
        d = inv3(d);
        th[0] = t_next * 1.00001f;
        if (!p->leaf_skipping || ray_box(o, inv3(d), tr->aabb_min + 4 * (size_t)node,
                                          tr->aabb_max + 4 * (size_t)node)) {
            const int h = leaf_test(tr, tri, node, o, d, p->tie, p->intersection, th);
            if (h != -1) {
                *hit = h; *ot = th[0]; *ou = th[1]; *ov = th[2];
                if (dused) *dused = d;
                return;
            }
        }
        if (p->max_iterations > 0 && ++iters >= p->max_iterations) break;
    } while (th[0] < OR_FINF);
    *hit = -1; *ot = INFINITY; *ou = 0.0f; *ov = 0.0f;
}

/* BruteTracer.cu:54-96 Exhaustive (first hit, no direction clamp, the
 * 4096-triangle cap of BruteTracer.cu:50 lifted). */
static void trace_brute_one(const float *tri, int32_t T, int tie, int woop, v3 o, v3 d,
                            int32_t *hit, float *ot, float *ou, float *ov)
{
    float th[3] = {OR_FINF, 0.0f, 0.0f};
    int prim_hit = -1;
    for (int prim = 0; prim < T; ++prim) isect(woop, tri, prim, o, d, tie, &prim_hit, th);
    if (th[0] < OR_FINF) { *hit = prim_hit; *ot = th[0]; *ou = th[1]; *ov = th[2]; }
    else { *hit = -1; *ot = INFINITY; *ou = 0.0f; *ov = 0.0f; }
}

static int set_threads(int32_t threads)
{
#ifdef _OPENMP
    return threads > 0 ? threads : omp_get_max_threads();
#else
    (void)threads;
    return 1;
#endif
}

int or_trace(const or_tree *tr, const float *tri, int32_t T, const or_trace_params *p,
             const float *ray_o, const float *ray_d, int32_t n,
             int32_t *hit, float *t, float *u, float *v, int32_t threads)
{
    if (!p || n < 0 || (n > 0 && (!ray_o || !ray_d || !hit || !t || !u || !v))) return OR_ERR_ARG;
    if (p->tracer == OR_TRACER_BRUTE)
        return or_trace_brute(tri, T, p->tie, p->intersection, ray_o, ray_d, n, hit, t, u, v, threads);
    if (!tr || tr->n_nodes <= 0) return OR_ERR_ARG;
    if (p->tracer == OR_TRACER_SHORTSTACK && (p->stack_depth < 1 || p->stack_depth > 64)) return OR_ERR_ARG;
    const int nt = set_threads(threads);
    (void)nt;
#pragma omp parallel for schedule(static, 64) num_threads(nt)
    for (int32_t i = 0; i < n; ++i) {
        const v3 o = ld3(ray_o + 3 * (size_t)i), d = ld3(ray_d + 3 * (size_t)i);
        if (p->tracer == OR_TRACER_SHORTSTACK)
            trace_shortstack_one(tr, tri, p, o, d, hit + i, t + i, u + i, v + i, NULL);
        else
            trace_restart_one(tr, tri, p, o, d, hit + i, t + i, u + i, v + i, NULL);
    }
    return 0;
}

int or_trace_brute(const float *tri, int32_t T, int32_t tie, int32_t intersection,
                   const float *ray_o, const float *ray_d, int32_t n,
                   int32_t *hit, float *t, float *u, float *v, int32_t threads)
{
    if (n < 0 || T < 0) return OR_ERR_ARG;
    const int nt = set_threads(threads);
    (void)nt;
#pragma omp parallel for schedule(static, 64) num_threads(nt)
    for (int32_t i = 0; i < n; ++i) {
        const v3 o = ld3(ray_o + 3 * (size_t)i), d = ld3(ray_d + 3 * (size_t)i);
        trace_brute_one(tri, T, tie, intersection, o, d, hit + i, t + i, u + i, v + i);
    }
    return 0;
}

/* The same Moeller-Trumbore in double precision (an accuracy reference for
 * the fp32 results, not a restatement of reference arithmetic). */
int or_trace_brute_f64(const float *tri, int32_t T,
                       const float *ray_o, const float *ray_d, int32_t n,
                       int32_t *hit, double *t, double *u, double *v, int32_t threads)
{
    if (n < 0 || T < 0) return OR_ERR_ARG;
    const int nt = set_threads(threads);
    (void)nt;
#pragma omp parallel for schedule(static, 64) num_threads(nt)
    for (int32_t i = 0; i < n; ++i) {
        const double ox = ray_o[3 * (size_t)i], oy = ray_o[3 * (size_t)i + 1], oz = ray_o[3 * (size_t)i + 2];
        const double dx = ray_d[3 * (size_t)i], dy = ray_d[3 * (size_t)i + 1], dz = ray_d[3 * (size_t)i + 2];
        double best = (double)OR_FINF, bu = 0.0, bv = 0.0;
        int bh = -1;
        for (int prim = 0; prim < T; ++prim) {
            const float *tp = tri + (size_t)prim * 9;
            const double e1x = (double)tp[3] - tp[0], e1y = (double)tp[4] - tp[1], e1z = (double)tp[5] - tp[2];
            const double e2x = (double)tp[6] - tp[0], e2y = (double)tp[7] - tp[1], e2z = (double)tp[8] - tp[2];
            const double px = dy * e2z - dz * e2y, py = dz * e2x - dx * e2z, pz = dx * e2y - dy * e2x;
            const double sx = ox - tp[0], sy = oy - tp[1], sz = oz - tp[2];
            const double qx = sy * e1z - sz * e1y, qy = sz * e1x - sx * e1z, qz = sx * e1y - sy * e1x;
            const double det = px * e1x + py * e1y + pz * e1z;
            if (det == 0.0) continue;
            const double inv = 1.0 / det;
            const double tt = inv * (qx * e2x + qy * e2y + qz * e2z);
            if (!(0.0 <= tt && tt <= best)) continue;
            const double uu = inv * (px * sx + py * sy + pz * sz);
            const double vv = inv * (qx * dx + qy * dy + qz * dz);
            if (uu >= 0.0 && vv >= 0.0 && uu + vv <= 1.0) {
                if (bh == -1 || tt < best) { bh = prim; best = tt; bu = uu; bv = vv; }
            }
        }
        if (bh != -1 && best < (double)OR_FINF) { hit[i] = bh; t[i] = best; u[i] = bu; v[i] = bv; }
        else { hit[i] = -1; t[i] = INFINITY; u[i] = 0.0; v[i] = 0.0; }
    }
    return 0;
}

/* Raytracer.cu:108-163 ShadowRay<false,true>: a ray from the light toward the
 * point (direction = point - light, not normalised, not clamped); the leaf is
 * skipped once its exit t reaches 0.999; any hit means shadow. */
int or_trace_shadow(const or_tree *tr, const float *tri, int32_t T, int32_t intersection,
                    const float *points, int32_t n, const float light[3],
                    int32_t *occluded, int32_t threads)
{
    (void)T;
    if (!tr || tr->n_nodes <= 0 || n < 0) return OR_ERR_ARG;
    const int nt = set_threads(threads);
    (void)nt;
    const v3 lp = ld3(light);
#pragma omp parallel for schedule(static, 64) num_threads(nt)
    for (int32_t i = 0; i < n; ++i) {
        const v3 pt = ld3(points + 3 * (size_t)i);
        const v3 d = sub3(pt, lp);
        const v3 inv = inv3(d);
        float t_min = 0.0f;
        int occ = 0;
        do {
            float t_next = OR_FINF;
            int node = 0;
            int8_t axis = tr->info[0];
            while ((axis & 3) != OR_LEAF) {
                const float sv = tr->split[node];
                const int l = tr->children[2 * node], r = tr->children[2 * node + 1];
                const float ori = axis_of(lp, axis), dir = axis_of(inv, axis);
                const float t_split = (sv - ori) * dir;
                if (t_min < t_split) {
                    node = 0 < dir ? l : r;
                    t_next = kmin(t_split, t_next);
                } else {
                    node = 0 < dir ? r : l;
                }
                axis = tr->info[node];
            }
            t_min = t_next * 1.00001f;
            if (t_min >= 0.999f) break;
            float th[3] = {t_min, 0.0f, 0.0f};
            if (leaf_test(tr, tri, node, lp, d, OR_TIE_REF_LAST, intersection, th) != -1) { occ = 1; break; }
        } while (t_min < 0.999f);
        occluded[i] = occ;
    }
    return 0;
}

/* ------------------------------------------------------------------------ */
/* Photons                                                                   */
/* ------------------------------------------------------------------------ */

/* Philox4x32-10 (Salmon et al., SC 2011). */
void or_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4])
{
    uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3], k0 = key[0], k1 = key[1];
    for (int r = 0; r < 10; ++r) {
        if (r > 0) { k0 += 0x9E3779B9u; k1 += 0xBB67AE85u; }
        const uint64_t p0 = (uint64_t)0xD2511F53u * c0, p1 = (uint64_t)0xCD9E8D57u * c2;
        const uint32_t lo0 = (uint32_t)p0, hi0 = (uint32_t)(p0 >> 32);
        const uint32_t lo1 = (uint32_t)p1, hi1 = (uint32_t)(p1 >> 32);
        const uint32_t n0 = hi1 ^ c1 ^ k0, n2 = hi0 ^ c3 ^ k1;
        c0 = n0; c1 = lo1; c2 = n2; c3 = lo0;
    }
    out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

static inline float u24(uint32_t x) { return (float)(x >> 8) * 0x1p-24f; }

/* sin / cos of 2*pi*u: quadrant reduction on u, Taylor polynomials on
 * [-pi/4, pi/4]; the same operation order as the CUDA sampler. */
static inline void sincos_2pi(float u, float *s, float *c)
{
    const float u4 = u * 4.0f;
    const float k = floorf(u4 + 0.5f);
    const float x = (u4 - k) * 1.57079632679489662f;
    const float x2 = x * x;
    float ps = 1.0f - x2 * 0.0238095238095238095f;
    ps = 1.0f - (x2 * 0.05f) * ps;
    ps = 1.0f - (x2 * 0.166666666666666667f) * ps;
    const float sx = x * ps;
    float pc = 1.0f - x2 * 0.0178571428571428571f;
    pc = 1.0f - (x2 * 0.0333333333333333333f) * pc;
    pc = 1.0f - (x2 * 0.0833333333333333333f) * pc;
    const float cx = 1.0f - (x2 * 0.5f) * pc;
    const int q = ((int)k) & 3;
    *s = q == 0 ? sx : (q == 1 ? cx : (q == 2 ? -sx : -cx));
    *c = q == 0 ? cx : (q == 1 ? -sx : (q == 2 ? -cx : sx));
}

static inline v3 sample_sphere(float u0, float u1)
{
    const float z = 1.0f - 2.0f * u0;
    const float r = sqrtf(fmaxf(0.0f, 1.0f - z * z));
    float s, c;
    sincos_2pi(u1, &s, &c);
    return mk3(r * c, r * s, z);
}

/* Cosine-weighted direction around n; basis of Duff et al., JCGT 2017. */
static inline v3 sample_cosine(v3 n, float u0, float u1)
{
    const float r = sqrtf(u0);
    float s, c;
    sincos_2pi(u1, &s, &c);
    const float x = r * c, y = r * s;
    const float z = sqrtf(fmaxf(0.0f, 1.0f - u0));
    const float sign = copysignf(1.0f, n.z);
    const float a = -1.0f / (sign + n.z);
    const float b = (n.x * n.y) * a;
    const v3 t = mk3(1.0f + ((sign * n.x) * n.x) * a, sign * b, -(sign * n.x));
    const v3 bt = mk3(b, sign + (n.y * n.y) * a, -n.y);
    return mk3((t.x * x + bt.x * y) + n.x * z, (t.y * x + bt.y * y) + n.y * z, (t.z * x + bt.z * y) + n.z * z);
}

int or_trace_photons(const or_tree *tr, const float *tri, int32_t T, const or_trace_params *p,
                     const or_photon_params *ph, int32_t n, int32_t *seg_hit, float *seg_t, int32_t threads)
{
    (void)T;
    if (!tr || !p || !ph || n < 0 || ph->bounces < 0) return OR_ERR_ARG;
    if (p->tracer != OR_TRACER_RESTART && p->tracer != OR_TRACER_SHORTSTACK) return OR_ERR_ARG;
    const int nt = set_threads(threads);
    (void)nt;
    const int S = ph->bounces + 1;
    const uint32_t key[2] = {(uint32_t)(ph->seed & 0xffffffffu), (uint32_t)(ph->seed >> 32)};
    const v3 light = ld3(ph->light);
#pragma omp parallel for schedule(static, 64) num_threads(nt)
    for (int32_t i = 0; i < n; ++i) {
        const int64_t base = (int64_t)i * S;
        uint32_t ctr[4] = {(uint32_t)i, 0u, 0u, 0u}, r[4];
        or_philox4x32_10(ctr, key, r);
        v3 o = light;
        v3 d = sample_sphere(u24(r[0]), u24(r[1]));
        int k = 0;
        while (k < S) {
            int32_t h;
            float t, u, v;
            if (p->tracer == OR_TRACER_SHORTSTACK) trace_shortstack_one(tr, tri, p, o, d, &h, &t, &u, &v, NULL);
            else trace_restart_one(tr, tri, p, o, d, &h, &t, &u, &v, NULL);
            seg_hit[base + k] = h;
            seg_t[base + k] = h >= 0 ? t : INFINITY;
            ++k;
            if (h < 0 || k == S) break;
            ctr[2] = (uint32_t)k;
            or_philox4x32_10(ctr, key, r);
            if (!(u24(r[2]) < ph->survival)) break;
            const float *tp = tri + 9 * (size_t)h;
            const v3 v0 = ld3(tp);
            const v3 cr = cross3(sub3(ld3(tp + 3), v0), sub3(ld3(tp + 6), v0));
            const float inv = 1.0f / sqrtf(dot3(cr, cr));
            v3 nrm = mk3(cr.x * inv, cr.y * inv, cr.z * inv);
            if (dot3(nrm, d) > 0.0f) nrm = mk3(-nrm.x, -nrm.y, -nrm.z);
            const v3 pt = mk3(o.x + t * d.x, o.y + t * d.y, o.z + t * d.z);
            o = mk3(pt.x + 1e-4f * nrm.x, pt.y + 1e-4f * nrm.y, pt.z + 1e-4f * nrm.z);
            d = sample_cosine(nrm, u24(r[0]), u24(r[1]));
        }
        for (; k < S; ++k) { seg_hit[base + k] = -2; seg_t[base + k] = INFINITY; }
    }
    return 0;
}

/* ------------------------------------------------------------------------ */
/* Shading (Raytracer.cu:165-262, ShortStack.cu:100-190, BruteTracer.cu:54-96, */
/* ColorKernels.h:15-85)                                                     */
/* ------------------------------------------------------------------------ */

/* x^y for x in [0, 1], y >= 0 (the specular term): 2^(y log2 x), log2 from
 * the series ln m = 2 atanh((m-1)/(m+1)) = 2 s (1 + s^2/3 + s^4/5 + ...) on
 * m in [sqrt(1/2), sqrt(2)), 2^f from the Taylor series of e^(f ln 2) on
 * f in [-1/2, 1/2]; within 2e-5 relative (the fp32 product y log2 x
 * dominates at large y).  The reference calls __powf on the
 * device and powf on the host; this own restatement with every operation
 * separately rounded is what the CUDA kernel computes as well. */
float or_kpow(float x, float y)
{
    if (y == 0.0f) return 1.0f;
    if (!(x > 0.0f)) return 0.0f;
    if (x >= 1.0f) return 1.0f;
    int e = 0;
    if (x < 0x1p-126f) { x = x * 0x1p24f; e = -24; }
    const int32_t b = f2i(x);
    e += ((b >> 23) & 0xff) - 127;
    float m = i2f((b & 0x007fffff) | 0x3f800000);
    if (m > 1.41421356f) { m = m * 0.5f; e += 1; }
    const float s = (m - 1.0f) / (m + 1.0f);
    const float s2 = s * s;
    float poly = 0.0909090909f;
    poly = 0.111111111f + s2 * poly;
    poly = 0.142857143f + s2 * poly;
    poly = 0.2f + s2 * poly;
    poly = 0.333333333f + s2 * poly;
    poly = 1.0f + s2 * poly;
    const float ln_m = (2.0f * s) * poly;
    const float z = y * ((float)e + ln_m * 1.44269504f);
    if (z < -150.0f) return 0.0f;
    const float n = floorf(z + 0.5f);
    const float g = (z - n) * 0.693147181f;
    float q = 2.48015873e-5f;
    q = 1.98412698e-4f + g * q;
    q = 1.38888889e-3f + g * q;
    q = 8.33333333e-3f + g * q;
    q = 4.16666667e-2f + g * q;
    q = 0.166666667f + g * q;
    q = 0.5f + g * q;
    q = 1.0f + g * q;
    q = 1.0f + g * q;
    const int ni = (int)n, n1 = ni / 2, n2 = ni - n1;
    return (q * i2f((n1 + 127) << 23)) * i2f((n2 + 127) << 23);
}

/* normalize of the CUDA-SDK helpers with IEEE 1/sqrt (their host branch). */
static inline v3 nrm3(v3 v)
{
    const float inv = 1.0f / sqrtf(dot3(v, v));
    return mk3(v.x * inv, v.y * inv, v.z * inv);
}
static inline float sat(float x) { return x > 0.0f ? (x < 1.0f ? x : 1.0f) : 0.0f; }
static inline float clamp01(float x) { return fmaxf(0.0f, fminf(x, 1.0f)); }
static inline uint8_t to_u8(float x)
{
    const float y = truncf(x * 255.0f);
    return (uint8_t)(y > 0.0f ? (y < 255.0f ? y : 255.0f) : 0.0f);
}

/* PhongLighting (ColorKernels.h:15-41) with shadow = 1. */
static inline f4 phong(f4 c, v3 n, v3 pt, v3 origin, const or_light *L)
{
    const v3 lpos = ld3(L->position);
    const v3 ld = nrm3(sub3(lpos, pt));
    const float diffuse = sat(dot3(ld, n) * 1.0f);
    const float k = 2.0f * dot3(n, ld);
    const v3 refl = nrm3(mk3(k * n.x - ld.x, k * n.y - ld.y, k * n.z - ld.z));
    const float stemp = sat(dot3(nrm3(sub3(origin, pt)), refl));
    const float spec_prop = 1.0f - c.w;
    const float specular = spec_prop * or_kpow(stemp, 128.0f * spec_prop);
    const float *A = L->ambient, *D = L->diffuse, *S = L->specular;
    const float lx = c.x * (A[0] + D[0] * diffuse) + ((S[0] * specular) * 10.0f) * 1.0f;
    const float ly = c.y * (A[1] + D[1] * diffuse) + ((S[1] * specular) * 10.0f) * 1.0f;
    const float lz = c.z * (A[2] + D[2] * diffuse) + ((S[2] * specular) * 10.0f) * 1.0f;
    const float alpha = c.w < specular ? specular : c.w;
    f4 r = {clamp01(lx), clamp01(ly), clamp01(lz), alpha};
    return r;
}

/* Lighting (ColorKernels.h:43-78): colour of the hit, reflected direction,
 * next origin 1e-5 along it. */
static inline f4 lighting(float t, float u, float v, v3 *o, v3 *d, const float *n0, const float *n1,
                          const float *n2, const uint8_t *c0, int prim, const or_light *L)
{
    const v3 pt = mk3(o->x + t * d->x, o->y + t * d->y, o->z + t * d->z);
    const float w = (1.0f - u) - v;
    const float *a = n0 + 4 * (size_t)prim, *b = n1 + 4 * (size_t)prim, *c = n2 + 4 * (size_t)prim;
    const v3 n = nrm3(mk3((w * a[0] + u * b[0]) + v * c[0], (w * a[1] + u * b[1]) + v * c[1],
                          (w * a[2] + u * b[2]) + v * c[2]));
    const uint8_t *cc = c0 + 4 * (size_t)prim;
    f4 col = {cc[0] / 255.0f, cc[1] / 255.0f, cc[2] / 255.0f, cc[3] / 255.0f};
    const float k = 2.0f * dot3(n, mk3(-d->x, -d->y, -d->z));
    const v3 nd = nrm3(mk3(k * n.x + d->x, k * n.y + d->y, k * n.z + d->z));
    col = phong(col, n, pt, *o, L);
    *o = mk3(pt.x + 0.00001f * nd.x, pt.y + 0.00001f * nd.y, pt.z + 0.00001f * nd.z);
    *d = nd;
    return col;
}

/* BlendColor (ColorKernels.h:80-85). */
static inline f4 blend(f4 orig, f4 nc)
{
    const float k = (1.0f - orig.w) * nc.w;
    f4 r = {orig.x + k * nc.x, orig.y + k * nc.y, orig.z + k * nc.z, orig.w + k * 1.0f};
    return r;
}

void or_light_default(or_light *L)
{
    /* Raytracer.cu:43-51: light at (0,4,0), colour (1, 0.92, 0.8) scaled
     * 0.3 / 0.7 / 0.3 for ambient / diffuse / specular. */
    const float col[3] = {1.0f, 0.92f, 0.8f};
    L->position[0] = 0.0f; L->position[1] = 4.0f; L->position[2] = 0.0f;
    for (int k = 0; k < 3; ++k) {
        L->ambient[k] = col[k] * 0.3f;
        L->diffuse[k] = col[k] * 0.7f;
        L->specular[k] = col[k] * 0.3f;
    }
}

int or_trace_shaded(const or_tree *tr, const float *tri, int32_t T, const or_trace_params *p,
                    const float *n0, const float *n1, const float *n2, const uint8_t *c0, const or_light *L,
                    int32_t max_bounces, const float *ray_o, const float *ray_d, int32_t n, uint8_t *rgba,
                    int32_t threads)
{
    if (!p || !L || !n0 || !n1 || !n2 || !c0 || n < 0 || max_bounces < 1 ||
        (n > 0 && (!ray_o || !ray_d || !rgba)))
        return OR_ERR_ARG;
    if (p->tracer != OR_TRACER_BRUTE && (!tr || tr->n_nodes <= 0)) return OR_ERR_ARG;
    const int nt = set_threads(threads);
    (void)nt;
#pragma omp parallel for schedule(static, 64) num_threads(nt)
    for (int32_t i = 0; i < n; ++i) {
        v3 o = ld3(ray_o + 3 * (size_t)i), d = ld3(ray_d + 3 * (size_t)i);
        if (p->tracer != OR_TRACER_BRUTE) d = adjust_dir(d);
        f4 col = {0.0f, 0.0f, 0.0f, 0.0f};
        for (int b = 0; b < max_bounces; ++b) {
            int32_t h;
            float t, u, v;
            v3 dh = d;
            if (p->tracer == OR_TRACER_BRUTE) trace_brute_one(tri, T, p->tie, p->intersection, o, d, &h, &t, &u, &v);
            else if (p->tracer == OR_TRACER_SHORTSTACK) trace_shortstack_one(tr, tri, p, o, d, &h, &t, &u, &v, &dh);
            else trace_restart_one(tr, tri, p, o, d, &h, &t, &u, &v, &dh);
            if (h < 0) break;
            d = dh;
            col = blend(col, lighting(t, u, v, &o, &d, n0, n1, n2, c0, h, L));
            if (p->tracer != OR_TRACER_BRUTE) d = adjust_dir(d);
            if (!(col.w < 0.97f)) break;
        }
        uint8_t *px = rgba + 4 * (size_t)i;
        px[0] = to_u8(col.x); px[1] = to_u8(col.y); px[2] = to_u8(col.z); px[3] = to_u8(col.w);
    }
    return 0;
}

/* ------------------------------------------------------------------------ */
/* Build                                                                     */
/* ------------------------------------------------------------------------ */

void or_build_params_default(or_build_params *p)
{
    p->lower = OR_LOWER_BITMAP;
    p->split_empty_space = 1;
    p->propagate_aabbs = 1;
    p->empty_space_threshold = 0.35f;
    p->traversal_cost = 24.0f;
    p->intersection_cost = 1.0f;
    p->min_leaf = 0;
    p->esc_zmax_as_x = 1;
    p->max_levels = 64;
    p->leaf_size = 32;
    p->mode = 0;
    p->upper_levels = 8;
    p->sah_bins = 32;
    p->split_method = OR_SPLIT_BOX;
}

void or_trace_params_default(or_trace_params *p)
{
    p->tracer = OR_TRACER_RESTART;
    p->leaf_skipping = 1;
    p->tie = OR_TIE_LOWEST_ID;
    p->stack_depth = 4;
    p->max_iterations = 0;
    p->intersection = OR_ISECT_MOELLER;
}

void or_geometry_from_tris(const float *tri, int32_t T, float *p0, float *p1, float *p2)
{
    for (int32_t i = 0; i < T; ++i)
        for (int k = 0; k < 3; ++k) {
            float *dst = k == 0 ? p0 : (k == 1 ? p1 : p2);
            dst[4 * (size_t)i + 0] = tri[9 * (size_t)i + 3 * k + 0];
            dst[4 * (size_t)i + 1] = tri[9 * (size_t)i + 3 * k + 1];
            dst[4 * (size_t)i + 2] = tri[9 * (size_t)i + 3 * k + 2];
            dst[4 * (size_t)i + 3] = 1.0f;
        }
}

/* Growable node store (TriangleNode SoA).  New nodes are zero-filled; the
 * reference leaves fields it never writes (leaf splitPos/children, the boxes
 * of empty-space chain nodes, ...) uninitialised, which this restatement
 * defines as zero. */
typedef struct nodes {
    int32_t n, cap;
    int8_t *info; float *split; f4 *bmin; f4 *bmax;
    int32_t *pidx; int32_t *amt; int32_t *ch; float *area; int32_t *parent;
} nodes;

static void *grow(void *p, size_t old_elems, size_t new_elems, size_t esz)
{
    void *q = realloc(p, new_elems * esz);
    if (!q) return NULL;
    memset((char *)q + old_elems * esz, 0, (new_elems - old_elems) * esz);
    return q;
}

static int nodes_resize(nodes *s, int32_t n)
{
    if (n > s->cap) {
        int32_t nc = s->cap ? s->cap : 64;
        while (nc < n) nc *= 2;
#define G(f, T_, k) do { void *q = grow(s->f, (size_t)s->cap * (k), (size_t)nc * (k), sizeof(T_)); if (!q) return OR_ERR_ALLOC; s->f = q; } while (0)
        G(info, int8_t, 1); G(split, float, 1); G(bmin, f4, 1); G(bmax, f4, 1);
        G(pidx, int32_t, 1); G(amt, int32_t, 1); G(ch, int32_t, 2); G(area, float, 1); G(parent, int32_t, 1);
#undef G
        s->cap = nc;
    }
    s->n = n;
    return 0;
}

static void nodes_free(nodes *s)
{
    free(s->info); free(s->split); free(s->bmin); free(s->bmax); free(s->pidx);
    free(s->amt); free(s->ch); free(s->area); free(s->parent);
    memset(s, 0, sizeof(*s));
}

static inline float f4c(f4 a, int axis) { return axis == OR_X ? a.x : (axis == OR_Y ? a.y : a.z); }

typedef struct ivec { int32_t *a; size_t n, cap; } ivec;
static int ivec_push(ivec *v, int32_t x)
{
    if (v->n == v->cap) {
        size_t nc = v->cap ? v->cap * 2 : 256;
        int32_t *q = realloc(v->a, nc * sizeof(int32_t));
        if (!q) return OR_ERR_ALLOC;
        v->a = q; v->cap = nc;
    }
    v->a[v->n++] = x;
    return 0;
}

/* Exclusive scan of in[0..n) into out[0..n]; out[n] = total. */
static void excl_scan(const int32_t *in, int64_t n, int32_t *out)
{
    int32_t s = 0;
    for (int64_t i = 0; i < n; ++i) { out[i] = s; s += in[i]; }
    out[n] = s;
}

/* Half surface area of a box with edge lengths e0, e1, e2. */
static inline float half_area(float e0, float e1, float e2) { return (e0 * e1 + e1 * e2) + e2 * e0; }

/* Binned SAH over the references [s, s + a) inside tight box (mn, mx): B
 * equal bins per axis with extent > 0; a reference counts in the bin of its
 * box min (left histogram) and of its box max (right histogram); the plane at
 * bin boundary k has NL = sum of left counts below k and NR = sum of right
 * counts from k up, cost AL*NL + AR*NR with half box areas.  The first
 * strict minimum over (axis X, Y, Z; k = 1..B-1) wins; planes that leave a
 * side empty or put every reference on both sides are skipped.  Returns 0
 * when no plane qualifies (the median split is kept). */
static int sah_binned_split(const f4 *cmin, const f4 *cmax, int32_t s, int32_t a, f4 mn, f4 mx, int B,
                            int *axis_out, float *split_out)
{
    int32_t lo[3][256], hi[3][256];
    const float mnv[3] = {mn.x, mn.y, mn.z}, mxv[3] = {mx.x, mx.y, mx.z};
    float ext[3], scale[3];
    int valid[3];
    for (int ax = 0; ax < 3; ++ax) {
        ext[ax] = mxv[ax] - mnv[ax];
        valid[ax] = ext[ax] > 0.0f;
        scale[ax] = valid[ax] ? (float)B / ext[ax] : 0.0f;
        for (int b = 0; b < B; ++b) lo[ax][b] = hi[ax][b] = 0;
    }
    for (int32_t r = s; r < s + a; ++r) {
        const float lv[3] = {cmin[r].x, cmin[r].y, cmin[r].z}, hv[3] = {cmax[r].x, cmax[r].y, cmax[r].z};
        for (int ax = 0; ax < 3; ++ax) {
            if (!valid[ax]) continue;
            int bl = (int)((lv[ax] - mnv[ax]) * scale[ax]);
            int bh = (int)((hv[ax] - mnv[ax]) * scale[ax]);
            bl = bl < 0 ? 0 : (bl > B - 1 ? B - 1 : bl);
            bh = bh < 0 ? 0 : (bh > B - 1 ? B - 1 : bh);
            lo[ax][bl]++;
            hi[ax][bh]++;
        }
    }
    float best = INFINITY, best_sp = 0.0f;
    int best_ax = -1;
    for (int ax = 0; ax < 3; ++ax) {
        if (!valid[ax]) continue;
        const float w = ext[ax] / (float)B;
        int32_t total_hi = 0;
        for (int b = 0; b < B; ++b) total_hi += hi[ax][b];
        int32_t nl = 0, hi_below = 0;
        for (int k = 1; k < B; ++k) {
            nl += lo[ax][k - 1];
            hi_below += hi[ax][k - 1];
            const int32_t nr = total_hi - hi_below;
            const float pk = mnv[ax] + (float)k * w;
            float le[3] = {ext[0], ext[1], ext[2]}, re[3] = {ext[0], ext[1], ext[2]};
            le[ax] = pk - mnv[ax];
            re[ax] = mxv[ax] - pk;
            const float al = half_area(le[0], le[1], le[2]), ar = half_area(re[0], re[1], re[2]);
            const float cost = al * (float)nl + ar * (float)nr;
            if (nl > 0 && nr > 0 && !(nl == a && nr == a) && cost < best) {
                best = cost;
                best_ax = ax;
                best_sp = pk;
            }
        }
    }
    if (best_ax < 0) return 0;
    *axis_out = best_ax + 1;
    *split_out = best_sp;
    return 1;
}

/*
 * Upper ("large node") phase: TriangleMapUpperCreator.cu:110-183 (Create),
 * :185-205 (ProcessNodes), :241-318 (ReduceAabb), :320-368 (CreateEmptySplits),
 * :467-759 (CreateChildren, BOX method); kernels TriangleUpper.h:10-52,
 * ReduceSegments.h:230-371,466-484, EmptySpaceSplitting.h:10-184,299-368,
 * TriangleUpperChildren.h:10-62,144-395.  The 256-reference segments of the
 * reference only schedule its reduction; the tight box of a node is the
 * exact min/max over its references, which is what is computed here.
 */
/* One separating axis of Akenine-Moeller's triangle/box test (step 3: a
 * triangle edge crossed with a box axis), in the two coordinates (s, t)
 * perpendicular to the box axis: edge a->b, third vertex c, box half sizes
 * hs, ht, all relative to the box centre.  The slack r = (... + 1e-5) *
 * 1.0001 is IntersectionTests.h:20-21 (GAMMA, EPSILON); the expressions
 * follow a0XTests/a1XTests/a2XTests (IntersectionTests.h:23-149). */
static inline int sat_edge(float as, float at, float bs, float bt, float cs, float ct, float hs, float ht)
{
    const float p0 = at * bs - as * bt;
    const float p1 = (bs - as) * ct - (bt - at) * cs;
    float r = ht * fabsf(bs - as) + hs * fabsf(bt - at) + 0.00001f;
    r *= 1.0001f;
    return !((p0 > r && p1 > r) || (p0 < -r && p1 < -r));
}

/* TriangleAabbIntersectionStep3 (IntersectionTests.h:378-395): the nine
 * edge-axis tests against the box [lo, hi]. */
static int tri_box_step3(v3 v0, v3 v1, v3 v2, v3 lo, v3 hi)
{
    const v3 h = mk3((hi.x - lo.x) * 0.5f, (hi.y - lo.y) * 0.5f, (hi.z - lo.z) * 0.5f);
    const v3 c = mk3(lo.x + h.x, lo.y + h.y, lo.z + h.z);
    v0 = sub3(v0, c); v1 = sub3(v1, c); v2 = sub3(v2, c);
    int ok = 1;
    /* box axis x: coordinates (y, z) */
    ok &= sat_edge(v0.y, v0.z, v1.y, v1.z, v2.y, v2.z, h.y, h.z);
    ok &= sat_edge(v1.y, v1.z, v2.y, v2.z, v0.y, v0.z, h.y, h.z);
    ok &= sat_edge(v2.y, v2.z, v0.y, v0.z, v1.y, v1.z, h.y, h.z);
    /* box axis y: coordinates (z, x) */
    ok &= sat_edge(v0.z, v0.x, v1.z, v1.x, v2.z, v2.x, h.z, h.x);
    ok &= sat_edge(v1.z, v1.x, v2.z, v2.x, v0.z, v0.x, h.z, h.x);
    ok &= sat_edge(v2.z, v2.x, v0.z, v0.x, v1.z, v1.x, h.z, h.x);
    /* box axis z: coordinates (x, y) */
    ok &= sat_edge(v0.x, v0.y, v1.x, v1.y, v2.x, v2.y, h.x, h.y);
    ok &= sat_edge(v1.x, v1.y, v2.x, v2.y, v0.x, v0.y, h.x, h.y);
    ok &= sat_edge(v2.x, v2.y, v0.x, v0.y, v1.x, v1.y, h.x, h.y);
    return ok;
}

/* SetDivideSide<false> (TriangleUpperChildren.h:64-142): a reference whose
 * box straddles the plane is tested against the two halves of the node box
 * with the triangle itself, and may go to one side only (or to none, when
 * the triangle misses the node box although its clipped box does not). */
static inline void divide_sides(const float *tri, int32_t prim, f4 bmin, f4 bmax, int axis, float sp,
                                int32_t *left, int32_t *right)
{
    const float *tp = tri + 9 * (size_t)prim;
    const v3 v0 = ld3(tp), v1 = ld3(tp + 3), v2 = ld3(tp + 6);
    const v3 lo = mk3(bmin.x, bmin.y, bmin.z), hi = mk3(bmax.x, bmax.y, bmax.z);
    const v3 lhi = mk3(axis == OR_X ? sp : hi.x, axis == OR_Y ? sp : hi.y, axis == OR_Z ? sp : hi.z);
    const v3 rlo = mk3(axis == OR_X ? sp : lo.x, axis == OR_Y ? sp : lo.y, axis == OR_Z ? sp : lo.z);
    *left = tri_box_step3(v0, v1, v2, lo, lhi);
    *right = tri_box_step3(v0, v1, v2, rlo, hi);
}

static int build_upper(const float *tri, int32_t T, const or_build_params *p, nodes *nd,
                       f4 **fmin_out, f4 **fmax_out, int32_t *nfinal_out, ivec *leaf_ids,
                       int32_t *levels_out)
{
    const int LS = p->leaf_size;
    int rc = 0;
    f4 *cmin = NULL, *cmax = NULL, *nmin = NULL, *nmax = NULL, *fmin = NULL, *fmax = NULL;
    f4 *pmin = NULL, *pmax = NULL;
    int32_t *side = NULL, *saddr = NULL, *lside = NULL, *laddr = NULL, *owner = NULL;
    int32_t *csize = NULL, *lnode = NULL, *lnaddr = NULL, *req = NULL, *eaddr = NULL;
    int8_t *planes = NULL;
    int32_t nfinal = 0, ncap_final = 0;

    /* Root node (TriangleMapUpperCreator.cu:128-136). */
    if ((rc = nodes_resize(nd, 1))) goto out;
    nd->pidx[0] = 0; nd->amt[0] = T; nd->parent[0] = 0;
    memset(&nd->bmin[0], 0, sizeof(f4)); memset(&nd->bmax[0], 0, sizeof(f4));

    /* CalcPrimitiveAabb (TriangleUpper.h:10-28). */
    int64_t N = T;
    cmin = malloc(sizeof(f4) * (size_t)(N > 0 ? N : 1));
    cmax = malloc(sizeof(f4) * (size_t)(N > 0 ? N : 1));
    if (!cmin || !cmax) { rc = OR_ERR_ALLOC; goto out; }
    for (int32_t i = 0; i < T; ++i) {
        const float *tp = tri + 9 * (size_t)i;
        for (int k = 0; k < 9; ++k) if (!isfinite(tp[k])) { rc = OR_ERR_NONFINITE; goto out; }
        float mnx = tp[0], mny = tp[1], mnz = tp[2], mxx = tp[0], mxy = tp[1], mxz = tp[2];
        mnx = kmin(mnx, tp[3]); mny = kmin(mny, tp[4]); mnz = kmin(mnz, tp[5]);
        mxx = kmax(mxx, tp[3]); mxy = kmax(mxy, tp[4]); mxz = kmax(mxz, tp[5]);
        f4 a = {kmin(mnx, tp[6]), kmin(mny, tp[7]), kmin(mnz, tp[8]), i2f(i)};
        f4 b = {kmax(mxx, tp[6]), kmax(mxy, tp[7]), kmax(mxz, tp[8]), 0.0f};
        cmin[i] = a; cmax[i] = b;
    }

    int32_t active = 0, R = 1, level = 0;
    while (R > 0) {
        if (level >= p->max_levels) { rc = OR_ERR_LEVELS; goto out; }
        ++level;

        /* ReduceAabb (TriangleMapUpperCreator.cu:241-318). */
        free(pmin); free(pmax);
        pmin = malloc(sizeof(f4) * (size_t)R); pmax = malloc(sizeof(f4) * (size_t)R);
        if (!pmin || !pmax) { rc = OR_ERR_ALLOC; goto out; }
        for (int32_t k = 0; k < R; ++k) { pmin[k] = nd->bmin[active + k]; pmax[k] = nd->bmax[active + k]; }
#pragma omp parallel for schedule(dynamic, 16)
        for (int32_t k = 0; k < R; ++k) {
            const int32_t s = nd->pidx[active + k], a = nd->amt[active + k];
            float x0 = OR_FINF, y0 = OR_FINF, z0 = OR_FINF, x1 = -OR_FINF, y1 = -OR_FINF, z1 = -OR_FINF;
            for (int32_t r = s; r < s + a; ++r) {
                x0 = kmin(x0, cmin[r].x); y0 = kmin(y0, cmin[r].y); z0 = kmin(z0, cmin[r].z);
                x1 = kmax(x1, cmax[r].x); y1 = kmax(y1, cmax[r].y); z1 = kmax(z1, cmax[r].z);
            }
            f4 a0 = {x0, y0, z0, 0.0f}, a1 = {x1, y1, z1, 0.0f};
            nd->bmin[active + k] = a0; nd->bmax[active + k] = a1;
        }

        /* CreateEmptySplits, not at the root (TriangleMapUpperCreator.cu:302-303,
         * EmptySpaceSplitting.h:10-184); in tuned mode on every level, before
         * the median or the binned SAH split of the remaining box. */
        const int sah_level = p->mode == 1 && level > p->upper_levels;
        if (p->split_empty_space && active != 0) {
            free(planes); free(req); free(eaddr);
            planes = calloc((size_t)R, 1); req = calloc((size_t)R, sizeof(int32_t));
            eaddr = calloc((size_t)R + 1, sizeof(int32_t));
            if (!planes || !req || !eaddr) { rc = OR_ERR_ALLOC; goto out; }
            const float thr = p->empty_space_threshold;
            int any = 0;
            for (int32_t k = 0; k < R; ++k) {
                const f4 a = pmin[k], b = pmax[k];
                const f4 rmn = nd->bmin[active + k], rmx = nd->bmax[active + k];
                int pl = 0, nr = 0;
                if (rmn.x - a.x > thr * (b.x - a.x)) { pl |= 1; nr += 2; }
                if (rmn.y - a.y > thr * (b.y - a.y)) { pl |= 2; nr += 2; }
                if (rmn.z - a.z > thr * (b.z - a.z)) { pl |= 4; nr += 2; }
                if (b.x - rmx.x > thr * (b.x - a.x)) { pl |= 8; nr += 2; }
                if (b.y - rmx.y > thr * (b.y - a.y)) { pl |= 16; nr += 2; }
                if (b.z - rmx.z > thr * (b.z - a.z)) { pl |= 32; nr += 2; }
                planes[k] = (int8_t)pl; req[k] = nr;
                if (pl) any = 1;
            }
            if (any) {
                excl_scan(req, R, eaddr);
                const int32_t empty_nodes = eaddr[R];
                const int32_t base = nd->n;
                if ((rc = nodes_resize(nd, nd->n + empty_nodes))) goto out;
                for (int32_t k = 0; k < R; ++k) {
                    int pl = planes[k];
                    if (pl == 0) continue;
                    const int32_t leaf = active + k;
                    int32_t par = nd->parent[leaf];
                    const int32_t start = base + eaddr[k];
                    if (nd->ch[2 * par] == leaf) nd->ch[2 * par] = start;
                    else nd->ch[2 * par + 1] = start;
                    const f4 mn = nd->bmin[leaf], mx = nd->bmax[leaf];
                    par = start;
                    static const int8_t lo_axis[3] = {OR_X, OR_Y, OR_Z};
                    for (int b = 0; b < 3; ++b) {
                        if (pl & (1 << b)) {
                            pl -= (1 << b);
                            nd->info[par] = lo_axis[b];
                            nd->split[par] = f4c(mn, lo_axis[b]);
                            const int32_t l = par + 1, r = pl ? l + 1 : leaf;
                            nd->ch[2 * par] = l; nd->ch[2 * par + 1] = r;
                            nd->info[l] = OR_LEAF; nd->amt[l] = 0;
                            par = r;
                        }
                    }
                    for (int b = 3; b < 5; ++b) {
                        if (pl & (1 << b)) {
                            pl -= (1 << b);
                            nd->info[par] = lo_axis[b - 3];
                            nd->split[par] = f4c(mx, lo_axis[b - 3]);
                            const int32_t r = par + 1, l = pl ? r + 1 : leaf;
                            nd->ch[2 * par] = l; nd->ch[2 * par + 1] = r;
                            nd->info[r] = OR_LEAF; nd->amt[r] = 0;
                            par = l;
                        }
                    }
                    if (pl & 32) {
                        /* EmptySpaceSplitting.h:172-181 cuts the max-z face on x at
                         * maxPlane.x; esc_zmax_as_x = 0 uses z and maxPlane.z. */
                        nd->info[par] = p->esc_zmax_as_x ? OR_X : OR_Z;
                        nd->split[par] = p->esc_zmax_as_x ? mx.x : mx.z;
                        const int32_t r = par + 1, l = leaf;
                        nd->ch[2 * par] = l; nd->ch[2 * par + 1] = r;
                        nd->info[r] = OR_LEAF; nd->amt[r] = 0;
                    }
                }
            }
        }

        /* CalcUpperNodeSplitInfo (ReduceSegments.h:466-484). */
        for (int32_t k = 0; k < R; ++k) {
            const f4 mn = nd->bmin[active + k], mx = nd->bmax[active + k];
            const float sx = mx.x - mn.x, sy = mx.y - mn.y, sz = mx.z - mn.z;
            const float mdx = sx * 0.5f + mn.x, mdy = sy * 0.5f + mn.y, mdz = sz * 0.5f + mn.z;
            const int y_above_x = sx < sy;
            const float mxs = y_above_x ? sy : sx;
            const float sp = y_above_x ? mdy : mdx;
            const int8_t ax = y_above_x ? OR_Y : OR_X;
            const int z_higher = mxs < sz;
            nd->split[active + k] = z_higher ? mdz : sp;
            nd->info[active + k] = z_higher ? OR_Z : ax;
        }
        /* Tuned mode below the median levels: binned SAH split (no reference
         * counterpart; the reference splits every upper level at the median). */
        if (sah_level) {
#pragma omp parallel for schedule(dynamic, 8)
            for (int32_t k = 0; k < R; ++k) {
                int axis;
                float sp;
                if (sah_binned_split(cmin, cmax, nd->pidx[active + k], nd->amt[active + k], nd->bmin[active + k],
                                     nd->bmax[active + k], p->sah_bins, &axis, &sp)) {
                    nd->info[active + k] = (int8_t)axis;
                    nd->split[active + k] = sp;
                }
            }
        }

        /* CreateChildren (TriangleMapUpperCreator.cu:467-759). */
        const int32_t child_start = nd->n;
        if ((rc = nodes_resize(nd, nd->n + 2 * R))) goto out;
        free(side); free(saddr); free(owner); free(csize);
        side = malloc(sizeof(int32_t) * (size_t)(2 * N + 1));
        saddr = malloc(sizeof(int32_t) * (size_t)(2 * N + 2));
        owner = malloc(sizeof(int32_t) * (size_t)(N > 0 ? N : 1));
        csize = malloc(sizeof(int32_t) * (size_t)(2 * R));
        if (!side || !saddr || !owner || !csize) { rc = OR_ERR_ALLOC; goto out; }
        for (int32_t k = 0; k < R; ++k) {
            const int32_t s = nd->pidx[active + k], a = nd->amt[active + k];
            for (int32_t r = s; r < s + a; ++r) owner[r] = k;
        }
        /* SetSplitSide (TriangleUpperChildren.h:10-62), or SetDivideSide<false>
         * (TriangleUpperChildren.h:64-142) with the DIVIDE split method. */
        const int divide = p->split_method == OR_SPLIT_DIVIDE;
#pragma omp parallel for schedule(static)
        for (int64_t r = 0; r < N; ++r) {
            const int32_t node = active + owner[r];
            const int axis = nd->info[node];
            const float sp = nd->split[node];
            side[r] = f4c(cmin[r], axis) <= sp;
            side[N + r] = sp < f4c(cmax[r], axis);
            if (divide && side[r] && side[N + r])
                divide_sides(tri, f2i(cmin[r].w), nd->bmin[node], nd->bmax[node], axis, sp, &side[r], &side[N + r]);
        }
        side[2 * N] = 0;
        excl_scan(side, 2 * N, saddr);
        int64_t new_tris = saddr[2 * N];
        /* Box sides keep every reference; DIVIDE may drop references whose
         * triangle misses the node box. */
        if (!divide && new_tris < N) { rc = OR_ERR_SPLIT; goto out; }

        /* CalcNodeChildSize (TriangleUpperChildren.h:144-162). */
        int created_leafs = 0;
        for (int32_t k = 0; k < R; ++k) {
            const int32_t s = nd->pidx[active + k], a = nd->amt[active + k];
            csize[2 * k] = saddr[s + a] - saddr[s];
            csize[2 * k + 1] = saddr[s + a + N] - saddr[s + N];
            if (csize[2 * k] < LS || csize[2 * k + 1] < LS) created_leafs = 1;
        }

        int32_t children_created;
        if (created_leafs) {
            free(lside); free(laddr);
            lside = malloc(sizeof(int32_t) * (size_t)(2 * N + 1));
            laddr = malloc(sizeof(int32_t) * (size_t)(2 * N + 2));
            if (!lside || !laddr) { rc = OR_ERR_ALLOC; goto out; }
            /* SetPrimitiveLeafSide (TriangleUpperChildren.h:164-186). */
            for (int64_t r = 0; r < N; ++r) {
                const int32_t k = owner[r];
                lside[r] = (csize[2 * k] < LS) * side[r];
                lside[N + r] = (csize[2 * k + 1] < LS) * side[N + r];
            }
            excl_scan(lside, 2 * N, laddr);
            const int32_t leaf_tris = laddr[2 * N];
            new_tris -= leaf_tris;
            const int32_t upper = nfinal;
            if (nfinal + leaf_tris > ncap_final) {
                int32_t nc = ncap_final ? ncap_final : 1024;
                while (nc < nfinal + leaf_tris) nc *= 2;
                f4 *a = realloc(fmin, sizeof(f4) * (size_t)nc), *b;
                if (!a) { rc = OR_ERR_ALLOC; goto out; }
                fmin = a;
                b = realloc(fmax, sizeof(f4) * (size_t)nc);
                if (!b) { rc = OR_ERR_ALLOC; goto out; }
                fmax = b;
                ncap_final = nc;
            }
            nfinal += leaf_tris;
            free(nmin); free(nmax);
            nmin = malloc(sizeof(f4) * (size_t)(new_tris > 0 ? new_tris : 1));
            nmax = malloc(sizeof(f4) * (size_t)(new_tris > 0 ? new_tris : 1));
            if (!nmin || !nmax) { rc = OR_ERR_ALLOC; goto out; }
            /* SplitTriangles, leaf variant (TriangleUpperChildren.h:329-383). */
#pragma omp parallel for schedule(static)
            for (int64_t r = 0; r < N; ++r) {
                const int32_t node = active + owner[r];
                const int axis = nd->info[node];
                const float sp = nd->split[node];
                const f4 a = cmin[r], b = cmax[r];
                if (side[r] == 1) {
                    f4 hi = {axis == OR_X ? kmin(sp, b.x) : b.x, axis == OR_Y ? kmin(sp, b.y) : b.y,
                             axis == OR_Z ? kmin(sp, b.z) : b.z, b.w};
                    if (lside[r]) { fmin[upper + laddr[r]] = a; fmax[upper + laddr[r]] = hi; }
                    else { nmin[saddr[r] - laddr[r]] = a; nmax[saddr[r] - laddr[r]] = hi; }
                }
                const int64_t rr = r + N;
                if (side[rr] == 1) {
                    f4 lo = {axis == OR_X ? kmax(sp, a.x) : a.x, axis == OR_Y ? kmax(sp, a.y) : a.y,
                             axis == OR_Z ? kmax(sp, a.z) : a.z, a.w};
                    if (lside[rr]) { fmin[upper + laddr[rr]] = lo; fmax[upper + laddr[rr]] = b; }
                    else { nmin[saddr[rr] - laddr[rr]] = lo; nmax[saddr[rr] - laddr[rr]] = b; }
                }
            }
            /* MarkNodeLeafs + scan (TriangleUpperChildren.h:190-201,
             * TriangleMapUpperCreator.cu:658-668). */
            free(lnode); free(lnaddr);
            lnode = malloc(sizeof(int32_t) * (size_t)(2 * R));
            lnaddr = malloc(sizeof(int32_t) * (size_t)(2 * R + 1));
            if (!lnode || !lnaddr) { rc = OR_ERR_ALLOC; goto out; }
            for (int32_t k = 0; k < R; ++k) {
                lnode[k] = csize[2 * k] < LS;
                lnode[R + k] = csize[2 * k + 1] < LS;
            }
            excl_scan(lnode, 2 * R, lnaddr);
            const int32_t leaf_nodes = lnaddr[2 * R];
            /* CreateUpperChildren, leaf variant (TriangleUpperChildren.h:236-281). */
            for (int32_t k = 0; k < R; ++k) {
                const int32_t par = active + k;
                const int32_t pi = nd->pidx[par];
                int leaf = csize[2 * k] < LS;
                int32_t la = lnaddr[k];
                const int32_t lid = (leaf ? la : k - la + leaf_nodes) + child_start;
                nd->pidx[lid] = leaf ? laddr[pi] + upper : saddr[pi] - laddr[pi];
                nd->amt[lid] = csize[2 * k];
                nd->parent[lid] = par;
                const int32_t kk = k + R;
                leaf = csize[2 * k + 1] < LS;
                la = lnaddr[kk];
                const int32_t rid = (leaf ? la : kk - la + leaf_nodes) + child_start;
                nd->pidx[rid] = leaf ? laddr[pi + N] + upper : saddr[pi + N] - laddr[pi + N];
                nd->amt[rid] = csize[2 * k + 1];
                nd->parent[rid] = par;
                nd->ch[2 * par] = lid; nd->ch[2 * par + 1] = rid;
            }
            children_created = 2 * R - leaf_nodes;
            /* MarkLeafNodes (TriangleUpperChildren.h:385-395). */
            for (int32_t i = 0; i < leaf_nodes; ++i)
                if ((rc = ivec_push(leaf_ids, child_start + i))) goto out;
        } else {
            free(nmin); free(nmax);
            nmin = malloc(sizeof(f4) * (size_t)(new_tris > 0 ? new_tris : 1));
            nmax = malloc(sizeof(f4) * (size_t)(new_tris > 0 ? new_tris : 1));
            if (!nmin || !nmax) { rc = OR_ERR_ALLOC; goto out; }
            /* CreateUpperChildren (TriangleUpperChildren.h:203-234). */
            for (int32_t k = 0; k < R; ++k) {
                const int32_t par = active + k;
                const int32_t lid = child_start + k, rid = lid + R;
                const int32_t pi = nd->pidx[par];
                nd->pidx[lid] = saddr[pi];
                nd->pidx[rid] = saddr[pi + N];
                nd->amt[lid] = csize[2 * k];
                nd->amt[rid] = csize[2 * k + 1];
                nd->ch[2 * par] = lid; nd->ch[2 * par + 1] = rid;
                nd->parent[lid] = par; nd->parent[rid] = par;
            }
            /* SplitTriangles (TriangleUpperChildren.h:283-327). */
#pragma omp parallel for schedule(static)
            for (int64_t r = 0; r < N; ++r) {
                const int32_t node = active + owner[r];
                const int axis = nd->info[node];
                const float sp = nd->split[node];
                const f4 a = cmin[r], b = cmax[r];
                if (side[r] == 1) {
                    f4 hi = {axis == OR_X ? kmin(sp, b.x) : b.x, axis == OR_Y ? kmin(sp, b.y) : b.y,
                             axis == OR_Z ? kmin(sp, b.z) : b.z, b.w};
                    nmin[saddr[r]] = a; nmax[saddr[r]] = hi;
                }
                if (side[r + N] == 1) {
                    f4 lo = {axis == OR_X ? kmax(sp, a.x) : a.x, axis == OR_Y ? kmax(sp, a.y) : a.y,
                             axis == OR_Z ? kmax(sp, a.z) : a.z, a.w};
                    nmin[saddr[r + N]] = lo; nmax[saddr[r + N]] = b;
                }
            }
            children_created = 2 * R;
        }

        /* PropagateAabbToChildren<false> (EmptySpaceSplitting.h:299-331). */
        if (p->split_empty_space) {
            for (int32_t k = 0; k < R; ++k) {
                const int32_t par = active + k;
                const int axis = nd->info[par] & 3;
                const float sp = nd->split[par];
                const int32_t l = nd->ch[2 * par], r = nd->ch[2 * par + 1];
                const f4 mn = nd->bmin[par], mx = nd->bmax[par];
                f4 rmn = {axis == OR_X ? sp : mn.x, axis == OR_Y ? sp : mn.y, axis == OR_Z ? sp : mn.z, 0.0f};
                f4 lmx = {axis == OR_X ? sp : mx.x, axis == OR_Y ? sp : mx.y, axis == OR_Z ? sp : mx.z, 0.0f};
                nd->bmin[l] = mn; nd->bmin[r] = rmn;
                nd->bmax[l] = lmx; nd->bmax[r] = mx;
            }
        }

        f4 *t0 = cmin, *t1 = cmax;
        cmin = nmin; cmax = nmax; nmin = t0; nmax = t1;
        N = new_tris;
        active = nd->n - children_created;
        R = children_created;
    }

    /* PropagateParentAabb<true> when empty-space splitting is off
     * (TriangleMapUpperCreator.cu:171-182, EmptySpaceSplitting.h:333-368). */
    if (!p->split_empty_space && p->propagate_aabbs) {
        for (size_t i = 0; i < leaf_ids->n; ++i) {
            const int32_t c = leaf_ids->a[i];
            const int32_t par = nd->parent[c];
            const f4 mn = nd->bmin[par], mx = nd->bmax[par];
            const int axis = nd->info[par] & 3;
            const float sp = nd->split[par];
            if (nd->ch[2 * par] == c) {
                f4 a = {mn.x, mn.y, mn.z, 0.0f};
                f4 b = {axis == OR_X ? sp : mx.x, axis == OR_Y ? sp : mx.y, axis == OR_Z ? sp : mx.z, 0.0f};
                nd->bmin[c] = a; nd->bmax[c] = b;
            } else {
                f4 a = {axis == OR_X ? sp : mn.x, axis == OR_Y ? sp : mn.y, axis == OR_Z ? sp : mn.z, 0.0f};
                f4 b = {mx.x, mx.y, mx.z, 0.0f};
                nd->bmin[c] = a; nd->bmax[c] = b;
            }
        }
    }

    *fmin_out = fmin; *fmax_out = fmax; fmin = fmax = NULL;
    *nfinal_out = nfinal;
    *levels_out = level;
out:
    free(cmin); free(cmax); free(nmin); free(nmax); free(fmin); free(fmax);
    free(pmin); free(pmax); free(side); free(saddr); free(lside); free(laddr);
    free(owner); free(csize); free(lnode); free(lnaddr); free(req); free(eaddr); free(planes);
    return rc;
}

/* Triangle area 0.5*|e1 x e2| (LowerTriangleMap.h:24-38). */
static inline float tri_area(const float *tri, int32_t prim)
{
    const float *tp = tri + 9 * (size_t)prim;
    const v3 v0 = ld3(tp), v1 = ld3(tp + 3), v2 = ld3(tp + 6);
    const v3 c = cross3(sub3(v1, v0), sub3(v2, v0));
    return 0.5f * sqrtf(dot3(c, c));
}

/* CalcAreaForSets (LowerTriangleMap.h:412-461). */
static inline void calc_area_for_sets(const int32_t sets_in[4], int axis, int32_t set_index,
                                      uint32_t area_idx, const float *areas,
                                      float *opt, float *la, float *ra, uint32_t *ls, uint32_t *rs,
                                      int *opt_axis, int32_t *split_index)
{
    uint32_t s[4] = {(uint32_t)sets_in[0] & area_idx, (uint32_t)sets_in[1] & area_idx,
                     (uint32_t)sets_in[2] & area_idx, (uint32_t)sets_in[3] & area_idx};
    float a[4] = {0.0f, 0.0f, 0.0f, 0.0f};
    uint32_t bits = area_idx;
    while (bits) {
        const int i = __builtin_ctz(bits);
        const uint32_t m = 1u << i;
        a[0] = a[0] + ((s[0] & m) ? areas[i] : 0.0f);
        a[1] = a[1] + ((s[1] & m) ? areas[i] : 0.0f);
        a[2] = a[2] + ((s[2] & m) ? areas[i] : 0.0f);
        a[3] = a[3] + ((s[3] & m) ? areas[i] : 0.0f);
        bits &= bits - 1u;
    }
    const float low = (float)__builtin_popcount(s[0]) * a[0] + (float)__builtin_popcount(s[1]) * a[1];
    const float high = (float)__builtin_popcount(s[2]) * a[2] + (float)__builtin_popcount(s[3]) * a[3];
    if (low < *opt) {
        *ls = s[0]; *rs = s[1]; *la = a[0]; *ra = a[1];
        *opt = low; *opt_axis = axis; *split_index = set_index;
    }
    if (high < *opt) {
        *ls = s[2]; *rs = s[3]; *la = a[2]; *ra = a[3];
        *opt = high; *opt_axis = axis; *split_index = (int32_t)((uint32_t)set_index | 0x80000000u);
    }
}

/* CalcRelationForSets (LowerTriangleMap.h:260-295): the node's sets of one
 * plane pair, weighted by small^2 + large^2 of the two set sizes; the first
 * strictly smaller weight wins. */
static inline void relation_for_sets(const int32_t sets_in[4], uint32_t node_set, int axis, int32_t set_index,
                                     int *weight, uint32_t *ls, uint32_t *rs, int *opt_axis, int32_t *split_index)
{
    const uint32_t s[4] = {(uint32_t)sets_in[0] & node_set, (uint32_t)sets_in[1] & node_set,
                           (uint32_t)sets_in[2] & node_set, (uint32_t)sets_in[3] & node_set};
    for (int h = 0; h < 2; ++h) {
        const int a = __builtin_popcount(s[2 * h]), b = __builtin_popcount(s[2 * h + 1]);
        const int small = a < b ? a : b, large = a < b ? b : a;
        const int w = small * small + large * large;
        if (w < *weight) {
            *weight = w;
            *ls = s[2 * h]; *rs = s[2 * h + 1];
            *opt_axis = axis;
            *split_index = h ? (int32_t)((uint32_t)set_index | 0x80000000u) : set_index;
        }
    }
}

/*
 * Lower phase with bitmap sets, two creators:
 *  - SAH: TriangleMapSAHCreator.cu:67-260 with kernels LowerTriangleMap.h:24-155
 *    (areas, preprocessing, splitting planes) and :412-636 (CalcSAH,
 *    CreateLowerSAHChildren, PropagateAabbToChildren).  With
 *    intersection_cost = 1 and min_leaf = 0 the split rule is the
 *    reference's `optimalArea < (bitcount - traversalCost) * nodeArea`.
 *  - BALANCED ("SSAH"): TriangleMapBalancedCreator.cu:60-248 with
 *    PreprocessLeafNodes (LowerTriangleMap.h:40-53), the same splitting
 *    planes, CalcSplit (:299-369) and CreateChildren (:371-410).  Node areas
 *    stay zero (the creator never writes them); TrimChildBitmaps never runs
 *    (removeFalsePrimitives is fixed to false, TriangleMapBalancedCreator.cu:35).
 */
static int build_lower(const float *tri, const or_build_params *p, nodes *nd,
                       const f4 *fmin, const f4 *fmax, int32_t NF,
                       const int32_t *prim_indices, const ivec *leaf_ids, int32_t *levels_out)
{
    int rc = 0;
    const int balanced = p->lower == OR_LOWER_BALANCED;
    float *areas = malloc(sizeof(float) * (size_t)(NF > 0 ? NF : 1));
    int32_t *sts = malloc(sizeof(int32_t) * 12 * (size_t)(NF > 0 ? NF : 1));
    int32_t *act = NULL, *ssplit = NULL, *saddr = NULL, *csets = NULL;
    float *careas = NULL;
    if (!areas || !sts) { rc = OR_ERR_ALLOC; goto out; }

    const int32_t R0 = (int32_t)leaf_ids->n;
    if (balanced) {
        /* PreprocessLeafNodes (LowerTriangleMap.h:40-53): every reference. */
        for (int32_t k = 0; k < R0; ++k) {
            const int32_t leaf = leaf_ids->a[k];
            nd->amt[leaf] = (int32_t)((1u << nd->amt[leaf]) - 1u);
        }
    } else {
        for (int32_t i = 0; i < NF; ++i) areas[i] = tri_area(tri, prim_indices[i]);
        /* PreprocesLowerNodes (LowerTriangleMap.h:56-81). */
        for (int32_t k = 0; k < R0; ++k) {
            const int32_t leaf = leaf_ids->a[k];
            const int32_t pi = nd->pidx[leaf], amt = nd->amt[leaf];
            float area = 0.0f;
            uint32_t bmp = 0;
            for (int32_t i = 0; i < amt; ++i) {
                const float a = areas[pi + i];
                bmp += a > 0.0f ? (1u << i) : 0u;
                area += a;
            }
            nd->area[leaf] = area;
            nd->amt[leaf] = (int32_t)bmp;
        }
    }
    /* CreateSplittingPlanes (LowerTriangleMap.h:84-155): sets per prim slot,
     * per axis {lowLeft, lowRight, highLeft, highRight}. */
#pragma omp parallel for schedule(dynamic, 16)
    for (int32_t k = 0; k < R0; ++k) {
        const int32_t leaf = leaf_ids->a[k];
        const int32_t pi = nd->pidx[leaf];
        const uint32_t bmp = (uint32_t)nd->amt[leaf];
        uint32_t tris = bmp;
        while (tris) {
            const int id = __builtin_ctz(tris);
            const f4 lo = fmin[pi + id], hi = fmax[pi + id];
            uint32_t sx[4] = {0, 0, 0, 0}, sy[4] = {0, 0, 0, 0}, sz[4] = {0, 0, 0, 0};
            uint32_t b = bmp;
            while (b) {
                const int i = __builtin_ctz(b);
                const uint32_t m = 1u << i;
                const f4 mn = fmin[pi + i], mx = fmax[pi + i];
                sx[0] |= mn.x <= lo.x ? m : 0; sx[1] |= lo.x < mx.x ? m : 0;
                sx[2] |= mn.x <= hi.x ? m : 0; sx[3] |= hi.x < mx.x ? m : 0;
                sy[0] |= mn.y <= lo.y ? m : 0; sy[1] |= lo.y < mx.y ? m : 0;
                sy[2] |= mn.y <= hi.y ? m : 0; sy[3] |= hi.y < mx.y ? m : 0;
                sz[0] |= mn.z <= lo.z ? m : 0; sz[1] |= lo.z < mx.z ? m : 0;
                sz[2] |= mn.z <= hi.z ? m : 0; sz[3] |= hi.z < mx.z ? m : 0;
                b &= b - 1u;
            }
            for (int c = 0; c < 4; ++c) {
                sts[4 * (size_t)(pi + id) + c] = (int32_t)sx[c];
                sts[4 * ((size_t)NF + pi + id) + c] = (int32_t)sy[c];
                sts[4 * (2 * (size_t)NF + pi + id) + c] = (int32_t)sz[c];
            }
            tris &= tris - 1u;
        }
    }

    int32_t R = R0, active = nd->n, lv = 0;
    int use_idx = 1;
    while (R > 0) {
        ++lv;
        free(act); free(ssplit); free(saddr); free(csets); free(careas);
        act = malloc(sizeof(int32_t) * (size_t)R);
        ssplit = malloc(sizeof(int32_t) * (size_t)R);
        saddr = malloc(sizeof(int32_t) * (size_t)R + sizeof(int32_t));
        csets = malloc(sizeof(int32_t) * 2 * (size_t)R);
        careas = malloc(sizeof(float) * 2 * (size_t)R);
        if (!act || !ssplit || !saddr || !csets || !careas) { rc = OR_ERR_ALLOC; goto out; }
        for (int32_t k = 0; k < R; ++k) act[k] = use_idx ? leaf_ids->a[k] : active + k;

        const float ct = p->traversal_cost, ci = p->intersection_cost;
        if (balanced) {
            /* CalcSplit (LowerTriangleMap.h:299-369). */
#pragma omp parallel for schedule(dynamic, 16)
            for (int32_t k = 0; k < R; ++k) {
                const int32_t par = act[k];
                const int32_t pi = nd->pidx[par];
                const uint32_t bmp = (uint32_t)nd->amt[par];
                int weight = 32 * 32, axis = 0;
                uint32_t ls = 0, rs = 0;
                int32_t split_index = 0;
                uint32_t tris = bmp;
                while (tris) {
                    const int i = __builtin_ctz(tris);
                    relation_for_sets(sts + 4 * (size_t)(pi + i), bmp, OR_X, pi + i, &weight, &ls, &rs, &axis,
                                      &split_index);
                    relation_for_sets(sts + 4 * ((size_t)NF + pi + i), bmp, OR_Y, pi + i, &weight, &ls, &rs, &axis,
                                      &split_index);
                    relation_for_sets(sts + 4 * (2 * (size_t)NF + pi + i), bmp, OR_Z, pi + i, &weight, &ls, &rs,
                                      &axis, &split_index);
                    tris &= tris - 1u;
                }
                /* A split needs a plane (the reference's sets are
                 * uninitialised otherwise; with traversal_cost >= 0 no
                 * split is possible without one). */
                const float cnt = (float)__builtin_popcount(bmp);
                const float ssah = (ct + (float)weight) / cnt;
                const int split = weight < 32 * 32 && ssah < cnt;
                if (split) {
                    careas[2 * k] = 0.0f; careas[2 * k + 1] = 0.0f;
                    csets[2 * k] = (int32_t)ls; csets[2 * k + 1] = (int32_t)rs;
                    f4 sp4;
                    if ((uint32_t)split_index & 0x80000000u) sp4 = fmax[(uint32_t)split_index ^ 0x80000000u];
                    else sp4 = fmin[split_index];
                    nd->split[par] = f4c(sp4, axis);
                }
                nd->info[par] = split ? (int8_t)axis : OR_LEAF;
                ssplit[k] = split;
            }
        } else {
        /* CalcSAH (LowerTriangleMap.h:463-555). */
#pragma omp parallel for schedule(dynamic, 16)
        for (int32_t k = 0; k < R; ++k) {
            const int32_t par = act[k];
            const int32_t pi = nd->pidx[par];
            const uint32_t bmp = (uint32_t)nd->amt[par];
            float area[32];
            uint32_t b = bmp;
            while (b) { const int i = __builtin_ctz(b); area[i] = areas[pi + i]; b &= b - 1u; }
            float opt = OR_FINF, la = 0.0f, ra = 0.0f;
            uint32_t ls = 0, rs = 0;
            int axis = 0;
            int32_t split_index = 0;
            uint32_t tris = bmp;
            while (tris) {
                const int i = __builtin_ctz(tris);
                calc_area_for_sets(sts + 4 * (size_t)(pi + i), OR_X, pi + i, bmp, area,
                                   &opt, &la, &ra, &ls, &rs, &axis, &split_index);
                calc_area_for_sets(sts + 4 * ((size_t)NF + pi + i), OR_Y, pi + i, bmp, area,
                                   &opt, &la, &ra, &ls, &rs, &axis, &split_index);
                calc_area_for_sets(sts + 4 * (2 * (size_t)NF + pi + i), OR_Z, pi + i, bmp, area,
                                   &opt, &la, &ra, &ls, &rs, &axis, &split_index);
                tris &= tris - 1u;
            }
            const float node_area = nd->area[par];
            const int cnt = __builtin_popcount(bmp);
            int split = (ci * opt) < ((ci * (float)cnt) - ct) * node_area;
            if (cnt <= p->min_leaf) split = 0;
            if (split) {
                careas[2 * k] = la; careas[2 * k + 1] = ra;
                csets[2 * k] = (int32_t)ls; csets[2 * k + 1] = (int32_t)rs;
                f4 sp4;
                if ((uint32_t)split_index & 0x80000000u) sp4 = fmax[(uint32_t)split_index ^ 0x80000000u];
                else sp4 = fmin[split_index];
                nd->split[par] = f4c(sp4, axis);
            }
            nd->info[par] = split ? (int8_t)axis : OR_LEAF;
            ssplit[k] = split;
        }
        }
        excl_scan(ssplit, R, saddr);
        const int32_t splits = saddr[R];
        const int32_t child_base = nd->n;
        if ((rc = nodes_resize(nd, nd->n + 2 * splits))) goto out;
        /* CreateLowerSAHChildren (LowerTriangleMap.h:557-600); CreateChildren
         * (:371-410) is the same without areas. */
        for (int32_t k = 0; k < R; ++k) {
            if (!ssplit[k]) continue;
            const int32_t par = act[k];
            const int32_t l = child_base + saddr[k], r = l + splits;
            nd->area[l] = careas[2 * k]; nd->pidx[l] = nd->pidx[par]; nd->amt[l] = csets[2 * k];
            nd->area[r] = careas[2 * k + 1]; nd->pidx[r] = nd->pidx[par]; nd->amt[r] = csets[2 * k + 1];
            nd->ch[2 * par] = l; nd->ch[2 * par + 1] = r;
        }
        const int32_t created = 2 * splits;
        /* PropagateAabbToChildren (LowerTriangleMap.h:602-636). */
        if (p->propagate_aabbs && created > 0) {
            for (int32_t k = 0; k < R; ++k) {
                const int32_t par = act[k];
                const int axis = nd->info[par] & 3;
                if (axis == OR_LEAF) continue;
                const float sp = nd->split[par];
                const int32_t l = nd->ch[2 * par], r = nd->ch[2 * par + 1];
                const f4 mn = nd->bmin[par], mx = nd->bmax[par];
                f4 rmn = {axis == OR_X ? sp : mn.x, axis == OR_Y ? sp : mn.y, axis == OR_Z ? sp : mn.z, 0.0f};
                f4 lmx = {axis == OR_X ? sp : mx.x, axis == OR_Y ? sp : mx.y, axis == OR_Z ? sp : mx.z, 0.0f};
                nd->bmin[l] = mn; nd->bmin[r] = rmn;
                nd->bmax[l] = lmx; nd->bmax[r] = mx;
            }
        }
        use_idx = 0;
        active = nd->n - created;
        R = created;
    }
    *levels_out = lv;
out:
    free(areas); free(sts); free(act); free(ssplit); free(saddr); free(csets); free(careas);
    return rc;
}

int or_build(const float *tri, int32_t T, const or_build_params *p, or_tree *out)
{
    if (!out || !p || T < 0 || (T > 0 && !tri)) return OR_ERR_ARG;
    if (p->leaf_size < 1 || p->leaf_size > 32) return OR_ERR_ARG;
    if (p->mode == 1 && (p->sah_bins < 2 || p->sah_bins > 32 || p->upper_levels < 0)) return OR_ERR_ARG;
    if (p->lower < OR_LOWER_BITMAP || p->lower > OR_LOWER_BALANCED) return OR_ERR_ARG;
    if (p->split_method != OR_SPLIT_BOX && p->split_method != OR_SPLIT_DIVIDE) return OR_ERR_ARG;
    /* A negative cost lets the balanced rule split a node into itself and
     * an empty child forever. */
    if (p->lower == OR_LOWER_BALANCED && !(p->traversal_cost >= 0.0f)) return OR_ERR_ARG;
    memset(out, 0, sizeof(*out));
    nodes nd;
    memset(&nd, 0, sizeof(nd));
    ivec leaf_ids = {0};
    f4 *fmin = NULL, *fmax = NULL;
    int32_t NF = 0, up_levels = 0, lo_levels = 0;
    int rc = build_upper(tri, T, p, &nd, &fmin, &fmax, &NF, &leaf_ids, &up_levels);
    if (rc) goto fail;

    /* ExtractIndexFromAabb (TriangleUpper.h:43-52). */
    int32_t *prim_indices = malloc(sizeof(int32_t) * (size_t)(NF > 0 ? NF : 1));
    if (!prim_indices) { rc = OR_ERR_ALLOC; goto fail; }
    for (int32_t i = 0; i < NF; ++i) prim_indices[i] = f2i(fmin[i].w);

    if (p->lower == OR_LOWER_SAH || p->lower == OR_LOWER_BALANCED) {
        rc = build_lower(tri, p, &nd, fmin, fmax, NF, prim_indices, &leaf_ids, &lo_levels);
        if (rc) { free(prim_indices); goto fail; }
    } else {
        /* TriangleMapBitmapCreator.cu:32-49 PreprocessLeafNodes. */
        for (size_t k = 0; k < leaf_ids.n; ++k) {
            const int32_t leaf = leaf_ids.a[k];
            nd.info[leaf] = OR_LEAF;
            nd.amt[leaf] = (int32_t)((1u << nd.amt[leaf]) - 1u);
        }
    }

    out->n_nodes = nd.n;
    out->n_refs = NF;
    out->n_upper_leaves = (int32_t)leaf_ids.n;
    out->upper_levels = up_levels;
    out->lower_levels = lo_levels;
    out->info = nd.info; out->split = nd.split;
    out->aabb_min = (float *)nd.bmin; out->aabb_max = (float *)nd.bmax;
    out->prim_index = nd.pidx; out->bitmap = nd.amt; out->children = nd.ch;
    out->area = nd.area; out->parent = nd.parent;
    out->prim_indices = prim_indices;
    out->leaf_ids = leaf_ids.a ? leaf_ids.a : calloc(1, sizeof(int32_t));
    out->prim_min = (float *)(fmin ? fmin : calloc(1, sizeof(f4)));
    out->prim_max = (float *)(fmax ? fmax : calloc(1, sizeof(f4)));
    return 0;
fail:
    nodes_free(&nd);
    free(leaf_ids.a); free(fmin); free(fmax);
    return rc;
}

void or_tree_free(or_tree *t)
{
    if (!t) return;
    free(t->info); free(t->split); free(t->aabb_min); free(t->aabb_max); free(t->prim_index);
    free(t->bitmap); free(t->children); free(t->area); free(t->parent); free(t->prim_indices);
    free(t->leaf_ids); free(t->prim_min); free(t->prim_max);
    memset(t, 0, sizeof(*t));
}

/* ------------------------------------------------------------------------ */
/* Single-primitive entry points for the pin test against the reference's    */
/* own header-only code (oracle/refpin, tests/test_refpin.py).               */
/* ------------------------------------------------------------------------ */

void or_pin_adjust_dir(float d[3])
{
    const v3 a = adjust_dir(ld3(d));
    d[0] = a.x; d[1] = a.y; d[2] = a.z;
}

int or_pin_ray_box(const float o[3], const float inv[3], const float bmin[3], const float bmax[3])
{
    return ray_box(ld3(o), ld3(inv), bmin, bmax);
}

void or_pin_woop_rows(const float tri[9], float m[12])
{
    f4 r[3];
    woop_rows(tri, 0, r);
    for (int i = 0; i < 3; ++i) {
        m[4 * i] = r[i].x; m[4 * i + 1] = r[i].y; m[4 * i + 2] = r[i].z; m[4 * i + 3] = r[i].w;
    }
}

int or_pin_woop(const float tri[9], const float o[3], const float d[3], float t_max, float out[3])
{
    float th[3] = {t_max, 0.0f, 0.0f};
    int hit = -1;
    woop_test(tri, 0, ld3(o), ld3(d), OR_TIE_REF_LAST, &hit, th);
    out[0] = th[0]; out[1] = th[1]; out[2] = th[2];
    return hit == 0;
}

int or_pin_tri_box(const float tri[9], const float bmin[3], const float bmax[3])
{
    return tri_box_step3(ld3(tri), ld3(tri + 3), ld3(tri + 6), ld3(bmin), ld3(bmax));
}
