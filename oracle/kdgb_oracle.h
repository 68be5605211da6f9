/*
 * kdgb_oracle.h -- CPU restatement of the reference kd-tree build and ray
 * traversal (OpenEngineDK/extensions-PhotonMapping, Utils/CUDA).
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker for the CUDA path
 * and the timed CPU baseline in bench.py.  Nothing in the product library
 * links, loads or calls it; the product fails loudly when its CUDA
 * extension is missing instead of falling back here.
 *
 * Parity status: the reference's build and tracers cannot be compiled here
 * as a whole (they need OpenEngine core, extensions-CUDA, CUDPP and cutil,
 * none of which are present) and it ships no tests, golden vectors or
 * fixtures.  Its own code is compiled unmodified in pieces instead
 * (oracle/refpin, host stand-ins for CUDA) and run on the host, and this
 * restatement is pinned to it bit for bit:
 *   - the intersection primitives (or_pin_*, tests/test_refpin.py);
 *   - the upper creator's kernels (TriangleUpper*.h, EmptySpaceSplitting.h)
 *     and the lower creators' (LowerTriangleMap.h), replayed one thread at a
 *     time: whole trees (tests/test_refpin_upper.py, test_refpin.py);
 *   - the tracer sources (Raytracer.cu, ShortStack.cu, BruteTracer.cu, built
 *     with nvcc): shaded pixels, first hits and shadow rays
 *     (tests/test_refpin_trace.py).
 * The restatement follows the reference source line by line
 * (citations on each function) with one documented evaluation order for the
 * un-vendored float3 helpers:
 *   dot(a,b)   = (a.x*b.x + a.y*b.y) + a.z*b.z
 *   cross(a,b) = (a.y*b.z - a.z*b.y, a.z*b.x - a.x*b.z, a.x*b.y - a.y*b.x)
 * every multiply and add rounded separately (no FMA contraction), IEEE
 * division (the reference's host path, IRayTracer.h:127-128) and IEEE sqrt.
 *
 * All arrays are plain host memory.  Functions return 0 on success and a
 * negative number on error (see or_error_string).
 */
#ifndef KDGB_ORACLE_H
#define KDGB_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Utils/CUDA/Utils.h:18 -- the integer 0x7f800000 converted to float. */
#define OR_FINF 2139095040.0f

enum { OR_LEAF = 0, OR_X = 1, OR_Y = 2, OR_Z = 3 };
enum { OR_LOWER_BITMAP = 0, OR_LOWER_SAH = 1, OR_LOWER_BALANCED = 2 };
/* TriangleMap::SplitMethod (TriangleMap.h:34); SPLIT is not implemented by
 * the reference (TriangleMapUpperCreator.cu:551-552). */
enum { OR_SPLIT_BOX = 0, OR_SPLIT_DIVIDE = 1 };
enum { OR_TIE_LOWEST_ID = 0, OR_TIE_REF_LAST = 1 };
enum { OR_TRACER_RESTART = 0, OR_TRACER_SHORTSTACK = 1, OR_TRACER_BRUTE = 2 };

typedef struct or_build_params {
    int32_t lower;                 /* OR_LOWER_BITMAP (reference default), OR_LOWER_SAH or OR_LOWER_BALANCED */
    int32_t split_empty_space;     /* TriangleMapUpperCreator.cu:31 default true */
    int32_t propagate_aabbs;       /* TriangleMap.cu:47 default true */
    float   empty_space_threshold; /* TriangleMapUpperCreator.cu:28 default 0.35 */
    float   traversal_cost;        /* TriangleMap.cu:48 default 24 */
    float   intersection_cost;     /* 1.0 reproduces the reference SAH rule exactly */
    int32_t min_leaf;              /* SAH never splits nodes with <= min_leaf prims (0 = reference) */
    int32_t esc_zmax_as_x;         /* 1 = reproduce EmptySpaceSplitting.h:172-181 (max-z face cut on x) */
    int32_t max_levels;            /* guard against non-terminating upper loops */
    int32_t leaf_size;             /* upper leaf threshold: children with < leaf_size refs become leaves (32) */
    int32_t mode;                  /* 0 reference, 1 tuned (binned SAH below upper_levels) */
    int32_t upper_levels;          /* tuned: median / empty-space levels before the binned SAH */
    int32_t sah_bins;              /* tuned: bins per axis */
    int32_t split_method;          /* OR_SPLIT_BOX (TriangleMapUpperCreator.cu:32 default) or OR_SPLIT_DIVIDE */
} or_build_params;

typedef struct or_tree {
    int32_t n_nodes;
    int32_t n_refs;          /* length of prim_indices */
    int32_t n_upper_leaves;  /* length of leaf_ids */
    int32_t upper_levels;    /* upper loop iterations */
    int32_t lower_levels;    /* SAH loop iterations */
    int8_t  *info;           /* KDNode.h:65   0 LEAF, 1 X, 2 Y, 3 Z */
    float   *split;          /* KDNode.h:66 */
    float   *aabb_min;       /* KDNode.h:67   float4 per node, w = 0 */
    float   *aabb_max;
    int32_t *prim_index;     /* KDNode.h:68 */
    int32_t *bitmap;         /* KDNode.h:69   amount during the upper build, bitmap after */
    int32_t *children;       /* KDNode.h:73   int2 per node */
    float   *area;           /* TriangleNode.h:20 */
    int32_t *parent;         /* TriangleNode.h:21 */
    int32_t *prim_indices;   /* TriangleMap.h:55 */
    int32_t *leaf_ids;       /* TriangleMap.h:57 */
    float   *prim_min;       /* final clipped reference boxes (float4, w = tri id bits) */
    float   *prim_max;
} or_tree;

typedef struct or_trace_params {
    int32_t tracer;          /* OR_TRACER_* */
    int32_t leaf_skipping;   /* IRayTracer.cu:33 default true */
    int32_t tie;             /* OR_TIE_* */
    int32_t stack_depth;     /* ShortStack.cu:25 default 4 */
    int32_t max_iterations;  /* restart / pop guard per ray; 0 = unlimited */
    int32_t intersection;    /* OR_ISECT_*: IRayTracer.cu:33 default Moeller-Trumbore */
} or_trace_params;

enum { OR_ISECT_MOELLER = 0, OR_ISECT_WOOP = 1 };

void or_build_params_default(or_build_params *p);
void or_trace_params_default(or_trace_params *p);
const char *or_error_string(int code);

/* Builds the reference tree over T triangles (tri: T*9 floats, v0 v1 v2). */
int or_build(const float *tri, int32_t T, const or_build_params *p, or_tree *out);
void or_tree_free(or_tree *t);

/* Triangle SoA as GeometryList.h:41 (p0,p1,p2 float4 with w = 1). */
void or_geometry_from_tris(const float *tri, int32_t T, float *p0, float *p1, float *p2);

/*
 * First-hit trace of n rays.  Tree arrays are or_tree fields (may come from
 * any builder).  ray_o / ray_d: n*3 floats.  Outputs hit id (-1 miss), t, u, v.
 * `threads` = OpenMP threads (<= 0: all).
 */
int or_trace(const or_tree *tree, const float *tri, int32_t T,
             const or_trace_params *p,
             const float *ray_o, const float *ray_d, int32_t n,
             int32_t *hit, float *t, float *u, float *v, int32_t threads);

/* Brute force over all T triangles (BruteTracer.cu:54-96, cap lifted). */
int or_trace_brute(const float *tri, int32_t T, int32_t tie, int32_t intersection,
                   const float *ray_o, const float *ray_d, int32_t n,
                   int32_t *hit, float *t, float *u, float *v, int32_t threads);

/* FP64 brute force: same Moeller-Trumbore in double, lowest-id ties. */
int or_trace_brute_f64(const float *tri, int32_t T,
                       const float *ray_o, const float *ray_d, int32_t n,
                       int32_t *hit, double *t, double *u, double *v, int32_t threads);

/* Shadow rays (Raytracer.cu:108-163): occluded[i] = 1 when point i is in shadow. */
int or_trace_shadow(const or_tree *tree, const float *tri, int32_t T, int32_t intersection,
                    const float *points, int32_t n, const float light[3],
                    int32_t *occluded, int32_t threads);

/* Photon tracing: CPU restatement of kdgb_trace_photons (Philox4x32-10
 * emission + cosine-weighted diffuse bounces + Russian roulette).  The
 * reference has no photon pass; this is the checker of the CUDA version. */
typedef struct or_photon_params {
    float    light[3];
    uint64_t seed;
    int32_t  bounces;
    float    survival;
} or_photon_params;

int or_trace_photons(const or_tree *tree, const float *tri, int32_t T, const or_trace_params *p,
                     const or_photon_params *ph, int32_t n, int32_t *seg_hit, float *seg_t, int32_t threads);

/* Light of the shading loop (ColorKernels.h:10-13 constants). */
typedef struct or_light {
    float position[3], ambient[3], diffuse[3], specular[3];
} or_light;

/* The reference's defaults (Raytracer.cu:43-51). */
void or_light_default(or_light *L);

/* Shaded trace (Raytracer.cu:165-262 KDRestart, ShortStack.cu:100-190,
 * BruteTracer.cu:54-96 Exhaustive with ColorKernels.h:15-85): per ray, hit,
 * Phong-shade, reflect and continue until the ray escapes, the accumulated
 * alpha reaches 0.97 or max_bounces hits were shaded.  n0/n1/n2: T float4
 * vertex normals per triangle; c0: T uchar4 colours; rgba: n uchar4. */
int or_trace_shaded(const or_tree *tr, const float *tri, int32_t T, const or_trace_params *p,
                    const float *n0, const float *n1, const float *n2, const uint8_t *c0, const or_light *L,
                    int32_t max_bounces, const float *ray_o, const float *ray_d, int32_t n, uint8_t *rgba,
                    int32_t threads);

/* The x^y of the specular term (exported for tests). */
float or_kpow(float x, float y);

/* Philox4x32-10 block (exported for tests). */
void or_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);

/* Single primitives for the pin test against the reference's own header-only
 * code: AdjustRayDirection, RayBoxIntersection<true>, WoopTransformationMatrix
 * of (p1, p2, p0), Woop (REF_LAST acceptance) and
 * TriangleAabbIntersectionStep3, restated as the traversal and the build use
 * them. */
void or_pin_adjust_dir(float d[3]);
int or_pin_ray_box(const float o[3], const float inv[3], const float bmin[3], const float bmax[3]);
void or_pin_woop_rows(const float tri[9], float m[12]);
int or_pin_woop(const float tri[9], const float o[3], const float d[3], float t_max, float out[3]);
int or_pin_tri_box(const float tri[9], const float bmin[3], const float bmax[3]);

/* Moeller-Trumbore restated (IRayTracer.h:111-145); exported for unit tests. */
int or_moeller_trumbore(const float v0[3], const float v1[3], const float v2[3],
                        const float o[3], const float d[3], float t_max,
                        float out_tuv[3]);

#ifdef __cplusplus
}
#endif
#endif
