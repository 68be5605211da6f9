/*
 * kdgb.h -- C ABI of the GB300 kd-tree builder and ray tracer.
 *
 * Drop-in for the tree-build and trace path of OpenEngineDK/
 * extensions-PhotonMapping.  The reference exposes that path as C++ classes
 * (TriangleMap, KDNode/TriangleNode, IRayTracer and its three tracers); each
 * entry point below names the reference interface it replaces.  The C++
 * plugin shims in kdgb_plugin.hpp keep the reference class names on top of
 * this ABI.
 *
 * Conventions
 *  - Every function returns an int status (KDGB_OK = 0) and never throws.
 *    kdgb_status_string() names a status, kdgb_last_error() gives the detail
 *    of the last failure on the calling thread.
 *  - Pointers named *_dev are device pointers; everything is stream ordered
 *    on the cudaStream_t passed in (0 = legacy default stream).  Calls that
 *    must size their output (kdgb_build) synchronise that stream.
 *  - A kdgb_tree handle may be traced from several streams at once; building
 *    or destroying it must not overlap other use of the same handle.
 *  - Triangles are T*9 floats (v0.xyz v1.xyz v2.xyz); rays are n*3 float
 *    origins and n*3 float directions; hit outputs are SoA.
 *  - Arithmetic: fp32, each multiply/add rounded separately (no FMA
 *    contraction), IEEE division and square root, so results match the CPU
 *    restatement of the reference bit for bit.
 */
#ifndef KDGB_H
#define KDGB_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct CUstream_st *kdgb_stream_t; /* same type as cudaStream_t */

#if defined(__GNUC__)
#define KDGB_API __attribute__((visibility("default")))
#else
#define KDGB_API
#endif

#define KDGB_ABI_VERSION 6

/* Utils/CUDA/Utils.h:18: the reference's "infinity" is the integer
 * 0x7f800000 converted to float. */
#define KDGB_FINF 2139095040.0f

typedef enum kdgb_status {
    KDGB_OK = 0,
    KDGB_ERR_INVALID_ARGUMENT = 1,
    KDGB_ERR_CUDA = 2,
    KDGB_ERR_OUT_OF_MEMORY = 3,
    KDGB_ERR_CAPACITY = 4,      /* a fixed-size pool or queue is full */
    KDGB_ERR_DEGENERATE = 5,    /* upper build did not terminate within max_levels */
    KDGB_ERR_NONFINITE = 6,     /* NaN or Inf vertex coordinate */
    KDGB_ERR_TIMEOUT = 7,       /* a bounded device-side wait gave up */
    KDGB_ERR_UNSUPPORTED = 8,
    KDGB_ERR_NO_DEVICE = 9
} kdgb_status;

/* KDNode.h:59-62 */
enum { KDGB_LEAF = 0, KDGB_X = 1, KDGB_Y = 2, KDGB_Z = 3 };

/* TriangleMap.h:33 LowerAlgorithm: BITMAP converts the upper leaves to
 * bitmap leaves (TriangleMapBitmapCreator), SAH splits them by the surface
 * area heuristic (TriangleMapSAHCreator), BALANCED by the reference's
 * "SSAH" set-size rule (TriangleMapBalancedCreator: split when
 * (traversal_cost + small^2 + large^2) / n < n; traversal_cost must be
 * >= 0).  The values differ from the reference enum's order. */
enum { KDGB_LOWER_BITMAP = 0, KDGB_LOWER_SAH = 1, KDGB_LOWER_BALANCED = 2 };

/* TriangleMap.h:34 SplitMethod of the upper phase: BOX sides from the
 * clipped reference boxes (SetSplitSide), DIVIDE also tests a straddling
 * triangle against the two halves of the node box (SetDivideSide, may drop
 * references whose triangle misses the node).  The reference's SPLIT is not
 * implemented there either and is rejected (KDGB_ERR_UNSUPPORTED). */
enum { KDGB_SPLIT_BOX = 0, KDGB_SPLIT_DIVIDE = 1, KDGB_SPLIT_SPLIT = 2 };

/* Build modes.  REFERENCE reproduces TriangleMap::Create bit for bit.
 * TUNED splits the top `upper_levels` levels at the reference's spatial
 * median and the remaining upper levels by a binned SAH (sah_bins bins per
 * axis, down to nodes of < leaf_size references), with the reference's
 * empty-space cuts on every level but the root; the lower phase is chosen
 * by `lower` as before. */
enum { KDGB_BUILD_REFERENCE = 0, KDGB_BUILD_TUNED = 1 };

/* Tracers: Raytracer (kd-restart), ShortStack, BruteTracer. */
enum { KDGB_TRACER_RESTART = 0, KDGB_TRACER_SHORTSTACK = 1, KDGB_TRACER_BRUTE = 2 };

/* Ray-triangle test (IRayTracer::SetIntersectionAlgorithm): Moeller-Trumbore
 * (IRayTracer.h:111-145) or Woop's unit-triangle transform (IRayTracer.h:
 * 78-109 with the per-triangle values of GeometryList.cu:81-102 /
 * IntersectionTests.h:438-467), computed for a tree on its first Woop trace
 * after each build. */
enum { KDGB_ISECT_MOELLER = 0, KDGB_ISECT_WOOP = 1 };

/* How a trace is spread over the GPU (no reference counterpart).  GRID:
 * one thread per ray, blocks in ray order.  QUEUE: a persistent launch
 * (as many blocks as fit on the device at once) whose warps take 32-ray
 * chunks from a device-side work queue; for a batch traced with
 * rays_per_mesh (ray_mesh_dev NULL) the queue hands out the rays of the
 * meshes with the most triangles first.  Results are identical.  The queue
 * state lives in the tree handle: QUEUE traces of one handle must not
 * overlap on the GPU (other streams). */
enum { KDGB_SCHEDULE_GRID = 0, KDGB_SCHEDULE_QUEUE = 1 };

/* Exact-tie rule between triangles hit at the same t.  LOWEST_ID is the
 * default; REF_LAST keeps the reference's `t <= tBest` (IRayTracer.h:133),
 * where the last triangle tested wins. */
enum { KDGB_TIE_LOWEST_ID = 0, KDGB_TIE_REF_LAST = 1 };

typedef struct kdgb_build_params {
    int32_t mode;                  /* KDGB_BUILD_* */
    int32_t lower;                 /* KDGB_LOWER_*, TriangleMap.cu:46 default BITMAP */
    int32_t split_empty_space;     /* TriangleMapUpperCreator.cu:31 default 1 */
    int32_t propagate_aabbs;       /* TriangleMap.cu:47 default 1 */
    float   empty_space_threshold; /* TriangleMapUpperCreator.cu:28 default 0.35 */
    float   traversal_cost;        /* TriangleMap.cu:48 default 24 */
    float   intersection_cost;     /* 1 = reference SAH rule */
    int32_t min_leaf;              /* SAH never splits nodes with <= min_leaf triangles (0 = reference) */
    int32_t esc_zmax_as_x;         /* 1 = EmptySpaceSplitting.h:172-181 behaviour (max-z face cut on x) */
    int32_t max_levels;            /* upper-phase level guard, default 64 */
    int32_t leaf_size;             /* KDNode.h:21 KDNODE_MAX_LOWER_SIZE, default 32, <= 32 */
    int32_t upper_levels;          /* TUNED: median/empty-space levels before SAH, default 8 */
    int32_t sah_bins;              /* TUNED: SAH bins per axis, 2..32, default 32 */
    int32_t split_method;          /* KDGB_SPLIT_*, TriangleMapUpperCreator.cu:32 default BOX */
} kdgb_build_params;

typedef struct kdgb_trace_params {
    int32_t tracer;          /* KDGB_TRACER_* */
    int32_t leaf_skipping;   /* IRayTracer.cu:33 default 1 */
    int32_t tie;             /* KDGB_TIE_* */
    int32_t stack_depth;     /* ShortStack.cu:25 SHORT_STACK_SIZE, 1..8, default 4 */
    int32_t max_iterations;  /* per-ray restart/pop guard, 0 = unlimited */
    int32_t block_size;      /* threads per block, 0 = library choice */
    int32_t tile_width;      /* >0: rays are a row-major image of this width; threads walk
                                4x8 pixel packets (IRayTracer.h:67-76) */
    int32_t intersection;    /* KDGB_ISECT_*, default MOELLER (IRayTracer.cu:33) */
    int32_t schedule;        /* KDGB_SCHEDULE_*, default GRID; QUEUE is not used by the fused
                                primary + shadow trace, photons or shading */
} kdgb_trace_params;

/* SoA device arrays of a tree, mirroring the KDNode / TriangleNode getters
 * (Scene/KDNode.h:85-94, Scene/TriangleNode.h:30-31) and
 * TriangleMap::GetPrimitiveIndices (TriangleMap.h:79).  For
 * kdgb_tree_upload the same struct carries HOST pointers. */
typedef struct kdgb_tree_view {
    int32_t n_nodes;
    int32_t n_refs;          /* length of prim_indices */
    int32_t n_upper_leaves;  /* length of leaf_ids */
    int32_t n_tris;
    int8_t  *info;           /* n_nodes */
    float   *split;          /* n_nodes */
    float   *aabb_min;       /* n_nodes * 4 (float4, w = 0) */
    float   *aabb_max;       /* n_nodes * 4 */
    int32_t *prim_index;     /* n_nodes */
    int32_t *bitmap;         /* n_nodes (KDNode::amount / bitmap) */
    int32_t *children;       /* n_nodes * 2 (int2) */
    float   *area;           /* n_nodes */
    int32_t *parent;         /* n_nodes */
    int32_t *prim_indices;   /* n_refs */
    int32_t *leaf_ids;       /* n_upper_leaves */
    float   *p0, *p1, *p2;   /* n_tris * 4 each, GeometryList SoA (GeometryList.h:41) */
} kdgb_tree_view;

typedef struct kdgb_tree kdgb_tree;

typedef struct kdgb_build_stats {
    int32_t upper_levels;
    int32_t lower_levels;
    int32_t n_nodes;
    int32_t n_refs;
    int32_t n_leaves;
    int32_t max_depth;
    float   build_ms;         /* device time of the last build (CUDA events) */
} kdgb_build_stats;

KDGB_API int         kdgb_abi_version(void);
KDGB_API const char *kdgb_status_string(int status);
KDGB_API const char *kdgb_last_error(void);
/* Number of kernel launches this library has issued since it was loaded
 * (instrumentation; no counterpart in the reference). */
KDGB_API int64_t     kdgb_launch_count(void);
KDGB_API void        kdgb_build_params_default(kdgb_build_params *p);
KDGB_API void        kdgb_trace_params_default(kdgb_trace_params *p);

/* Replaces TriangleMap::Create (Utils/CUDA/TriangleMap.cu:51-62): builds the
 * tree over n_tris device triangles.  The handle owns copies of the geometry
 * and all tree arrays.  Synchronises `stream` once per tree level. */
KDGB_API int kdgb_build(const float *tri_v_dev, int32_t n_tris, const kdgb_build_params *params,
               kdgb_tree **out, kdgb_stream_t stream);

/* Rebuilds an existing handle in place (same as TriangleMap::Create called
 * again each frame, PhotonRenderingView.cpp:45-60), reusing its memory. */
KDGB_API int kdgb_rebuild(kdgb_tree *tree, const float *tri_v_dev, int32_t n_tris,
                 const kdgb_build_params *params, kdgb_stream_t stream);

/* Creates a handle from tree arrays held in HOST memory (e.g. a tree built
 * on the CPU) plus host triangles; used to trace an externally built tree. */
KDGB_API int kdgb_tree_upload(const kdgb_tree_view *host_arrays, const float *tri_v_host, int32_t n_tris,
                     kdgb_tree **out, kdgb_stream_t stream);

/* Frees the handle.  The frees are ordered on the legacy default stream,
 * which a non-blocking stream does not wait for: work still queued on such
 * a stream must be finished first, or use kdgb_tree_release. */
KDGB_API int kdgb_tree_destroy(kdgb_tree *tree);

/* kdgb_tree_destroy ordered on `stream`: the device memory is freed after
 * the work already queued on `stream` (pass the stream the tree was last
 * used on), then that stream is synchronised.  The reference's TriangleMap
 * has no destructor (TriangleMap.cu:27-49); its device blocks live until
 * exit. */
KDGB_API int kdgb_tree_release(kdgb_tree *tree, kdgb_stream_t stream);

/* Replaces the KDNode / TriangleNode getters: device SoA pointers, valid
 * until the next kdgb_rebuild or kdgb_tree_destroy of this handle. */
KDGB_API int kdgb_tree_view_get(const kdgb_tree *tree, kdgb_tree_view *view);

/* Copies the SoA arrays into caller-owned HOST buffers (the fields of
 * `host_dst` that are non-NULL; sizes from kdgb_tree_view_get) and waits for
 * the copy.  Replaces the cudaMemcpy-per-field inspection of
 * KDNode::ToString / TriangleMap::PrintNode (KDNode.cu:64-119,
 * TriangleMap.cu:118-162). */
KDGB_API int kdgb_tree_download(const kdgb_tree *tree, kdgb_tree_view *host_dst);

KDGB_API int kdgb_tree_stats(const kdgb_tree *tree, kdgb_build_stats *stats);

/* Replaces IRayTracer::Trace (IRayTracer.h:47) of RayTracer (Raytracer.cu:295),
 * ShortStack (ShortStack.cu:231) and BruteTracer (BruteTracer.cu:123): first
 * hit of n rays; the uchar4 canvas output becomes hit id (-1 = miss), t, u, v.
 * Misses write t = +inf, u = v = 0. */
KDGB_API int kdgb_trace(const kdgb_tree *tree, const kdgb_trace_params *params,
               const float *ray_o_dev, const float *ray_d_dev, int32_t n,
               int32_t *hit_dev, float *t_dev, float *u_dev, float *v_dev,
               kdgb_stream_t stream);

/* Replaces RayTracer's ShadowRay (Raytracer.cu:108-163): occluded[i] = 1 when
 * the segment from `light` (3 host floats) toward point i is blocked. */
KDGB_API int kdgb_trace_shadow(const kdgb_tree *tree, const kdgb_trace_params *params,
                      const float *points_dev, int32_t n, const float light[3],
                      int32_t *occluded_dev, kdgb_stream_t stream);

/* Primary rays followed by one shadow ray per hit toward `light`, fused in
 * one launch; the shadow origin is p = o + t*d (separately rounded).
 * occluded is 0 for misses. */
KDGB_API int kdgb_trace_primary_shadow(const kdgb_tree *tree, const kdgb_trace_params *params,
                              const float *ray_o_dev, const float *ray_d_dev, int32_t n,
                              const float light[3],
                              int32_t *hit_dev, float *t_dev, float *u_dev, float *v_dev,
                              int32_t *occluded_dev, kdgb_stream_t stream);

/* Measurement aid (no reference counterpart): the same launch as
 * kdgb_trace_primary_shadow with the short-stack tracer, compiled with
 * counters, writing the same outputs.  counts (8 host uint64) receive the
 * primary rays' node records read, leaves reached, leaf boxes read and
 * triangle records tested, then the same four for the shadow rays (which read
 * no leaf boxes).  The timed trace kernels are compiled without the
 * counters.  Synchronises `stream`; allocates 64 bytes of device memory per
 * call. */
KDGB_API int kdgb_trace_count_steps(const kdgb_tree *tree, const kdgb_trace_params *params,
                           const float *ray_o_dev, const float *ray_d_dev, int32_t n,
                           const float light[3],
                           int32_t *hit_dev, float *t_dev, float *u_dev, float *v_dev,
                           int32_t *occluded_dev, uint64_t counts[8], kdgb_stream_t stream);

typedef struct kdgb_photon_params {
    float    light[3];   /* point light position (photon origin) */
    uint64_t seed;       /* Philox4x32-10 key */
    int32_t  bounces;    /* diffuse bounces after the first hit (3) */
    float    survival;   /* Russian-roulette survival probability (0.7) */
} kdgb_photon_params;

/* Defaults: light (0.5, 3, 0.5) (the frame's point light), seed 3,
 * 3 bounces, survival 0.7. */
KDGB_API void kdgb_photon_params_default(kdgb_photon_params *p);

/* Photon tracing (no reference counterpart; the reference's PhotonMapping
 * name never got a photon pass): n photons leave `light` in uniform
 * directions and bounce diffusely (cosine-weighted around the hit normal)
 * with Russian roulette, all random numbers from a counter-based
 * Philox4x32-10 stream (key = seed, counter = (photon, bounce)).  Each
 * segment is traced with the kd tracer in `params` (restart or short-stack).
 * Outputs n*(bounces+1) segments: hit id (-1 miss, -2 photon already ended)
 * and t (+inf when no hit). */
KDGB_API int kdgb_trace_photons(const kdgb_tree *tree, const kdgb_trace_params *params,
                                const kdgb_photon_params *photons, int32_t n_photons,
                                int32_t *seg_hit_dev, float *seg_t_dev, kdgb_stream_t stream);

/* Light of the shading loop (the __constant__ d_light* of
 * ColorKernels.h:10-13). */
typedef struct kdgb_light {
    float position[3];
    float ambient[3];
    float diffuse[3];
    float specular[3];
} kdgb_light;

/* The tracers' constructor defaults (Raytracer.cu:43-51). */
KDGB_API void kdgb_light_default(kdgb_light *light);

/* Replaces the pixel output of RayTracer / ShortStack / BruteTracer ::Trace
 * (Raytracer.cu:165-262, ShortStack.cu:100-190, BruteTracer.cu:54-96 with
 * Lighting / PhongLighting / BlendColor, ColorKernels.h:15-85), writing an
 * RGBA8 buffer instead of the OpenGL canvas.  Per ray: find the first hit,
 * shade it (interpolated vertex normal, triangle colour, Phong light),
 * blend it front to back, reflect the ray about the normal and continue from
 * the hit point until the ray escapes, the blended alpha reaches 0.97 or
 * max_bounces hits were shaded (0 = 64; the reference has no bound).
 * n0/n1/n2: n_tris float4 vertex normals per triangle and c0: n_tris uchar4
 * colours, the GeometryList layout (kdgb_geometry_gather_attributes fills
 * them); light NULL = kdgb_light_default.  The vector helpers are evaluated
 * left to right with IEEE 1/sqrt in normalize and the specular power is
 * this library's series restatement of pow, so the pixels are
 * deterministic and match the CPU restatement bit for bit. */
KDGB_API int kdgb_trace_shaded(const kdgb_tree *tree, const kdgb_trace_params *params, const float *n0_dev,
                               const float *n1_dev, const float *n2_dev, const uint8_t *c0_dev,
                               const kdgb_light *light, int32_t max_bounces, const float *ray_o_dev,
                               const float *ray_d_dev, int32_t n, uint8_t *rgba_dev, kdgb_stream_t stream);

/* BruteTracer::Trace's pixels without a tree (BruteTracer.cu:54-96 with the
 * shading of ColorKernels.h:15-85): as kdgb_trace_shaded with
 * KDGB_TRACER_BRUTE over n_tris device triangles (params: tie and
 * intersection are used). */
KDGB_API int kdgb_trace_brute_shaded(const float *tri_v_dev, int32_t n_tris, const kdgb_trace_params *params,
                                     const float *n0_dev, const float *n1_dev, const float *n2_dev,
                                     const uint8_t *c0_dev, const kdgb_light *light, int32_t max_bounces,
                                     const float *ray_o_dev, const float *ray_d_dev, int32_t n, uint8_t *rgba_dev,
                                     kdgb_stream_t stream);

/* kdgb_trace_brute with trace parameters (tie and intersection used), for
 * BruteTracer with SetIntersectionAlgorithm(WOOP) (BruteTracer.cu:139). */
KDGB_API int kdgb_trace_brute_ex(const float *tri_v_dev, int32_t n_tris, const kdgb_trace_params *params,
                                 const float *ray_o_dev, const float *ray_d_dev, int32_t n, int32_t *hit_dev,
                                 float *t_dev, float *u_dev, float *v_dev, kdgb_stream_t stream);

/* Batched build (no reference counterpart; the reference builds one scene
 * per TriangleMap): n_meshes independent meshes stored back to back in
 * tri_v_dev (mesh m = triangles [mesh_offsets[m], mesh_offsets[m+1]),
 * mesh_offsets: n_meshes+1 HOST ints) are built as one forest in a single
 * level loop: every level processes the active nodes of all meshes at once.
 * The root of mesh m is node m; each mesh's tree is the tree kdgb_build
 * makes for that mesh alone (same splits, leaves and reference order, node
 * ids interleaved).  Trace it with kdgb_trace_batch. */
KDGB_API int kdgb_build_batch(const float *tri_v_dev, const int32_t *mesh_offsets, int32_t n_meshes,
                              const kdgb_build_params *params, kdgb_tree **out, kdgb_stream_t stream);

/* Rebuilds a tree handle as a batch (same meaning as kdgb_build_batch),
 * reusing its device buffers. */
KDGB_API int kdgb_rebuild_batch(kdgb_tree *tree, const float *tri_v_dev, const int32_t *mesh_offsets,
                                int32_t n_meshes, const kdgb_build_params *params, kdgb_stream_t stream);

/* Traces rays of a batch: ray i belongs to mesh ray_mesh_dev[i], or to mesh
 * i / rays_per_mesh when ray_mesh_dev is NULL.  Hit ids are relative to the
 * mesh's first triangle. */
KDGB_API int kdgb_trace_batch(const kdgb_tree *tree, const kdgb_trace_params *params,
                              const float *ray_o_dev, const float *ray_d_dev, const int32_t *ray_mesh_dev,
                              int32_t rays_per_mesh, int32_t n, int32_t *hit_dev, float *t_dev, float *u_dev,
                              float *v_dev, kdgb_stream_t stream);

/* Graph rebuilds (no reference counterpart: TriangleMap::Create waits on the
 * device at every level of its host loop, TriangleMapUpperCreator.cu:
 * 110-759).  A kdgb_graph records one complete rebuild of `tree` -- and,
 * with n_rays > 0, a trace of its rays -- into a CUDA graph.  Launching it
 * rebuilds with no host synchronisation and no device allocation: the level
 * loops are conditional WHILE graph nodes driven by device-side counters.
 *  - The tree must have completed a kdgb_build / kdgb_rebuild (or batch
 *    build) first; the graph's fixed buffers are that build's sizes times
 *    `headroom` (1 to 64; 1.25 leaves 25% for geometry that changes
 *    between launches).
 *  - tri_v_dev (n_tris triangles; n_meshes > 1: a batch with HOST
 *    mesh_offsets as in kdgb_build_batch), the rays and the outputs are
 *    recorded by address: refill them in place between launches.  The trace
 *    is kdgb_trace (one mesh) or kdgb_trace_batch (ray_mesh_dev /
 *    rays_per_mesh) with `trace`; kd tracers only.
 *  - A rebuild that would outgrow a buffer stops and leaves the tree invalid
 *    (its traces report misses); kdgb_graph_status then returns
 *    KDGB_ERR_CAPACITY.  Rebuild with kdgb_rebuild / kdgb_rebuild_batch and
 *    create the graph again.
 *  - kdgb_graph_status synchronises the stream, returns the last launch's
 *    build status and refreshes the tree's host-side counts
 *    (kdgb_tree_stats, kdgb_tree_view_get are stale until then).
 *  - A host-driven rebuild that reallocates any of the tree's buffers
 *    invalidates the graph: kdgb_graph_launch then returns
 *    KDGB_ERR_INVALID_ARGUMENT.  Destroy graphs before their tree.
 *  - The graph is captured in the context of `stream`: with a stream of an
 *    SM partition (kdgb_sm_partition_stream) its kernels run on that
 *    partition's SMs, on whatever stream the graph is launched. */
typedef struct kdgb_graph kdgb_graph;

KDGB_API int kdgb_graph_create(kdgb_tree *tree, const float *tri_v_dev, int32_t n_tris,
                               const int32_t *mesh_offsets, int32_t n_meshes, const kdgb_build_params *params,
                               float headroom, const kdgb_trace_params *trace, const float *ray_o_dev,
                               const float *ray_d_dev, const int32_t *ray_mesh_dev, int32_t rays_per_mesh,
                               int32_t n_rays, int32_t *hit_dev, float *t_dev, float *u_dev, float *v_dev,
                               kdgb_graph **out, kdgb_stream_t stream);
KDGB_API int kdgb_graph_launch(kdgb_graph *graph, kdgb_stream_t stream);
KDGB_API int kdgb_graph_status(kdgb_graph *graph, kdgb_stream_t stream);
KDGB_API int kdgb_graph_destroy(kdgb_graph *graph);

/* SM partitions (no reference counterpart): the current device's SMs split
 * into two green contexts, the first with at least `sms` SMs (rounded up to
 * the device's granularity) and the second with the rest, for pipelined
 * frames: the rebuilds of the frames in flight on one partition and their
 * traces on the other, instead of taking the whole device from each other
 * kernel by kernel.  kdgb_sm_partition_stream makes a non-blocking stream
 * (priority as cudaStreamCreateWithPriority) whose kernels run on partition
 * `which` (0 or 1) only; memory, events and copies work with it as with any
 * stream of the device.  A graph created with such a stream keeps to its
 * partition (kdgb_graph_create).  The partition owns its streams:
 * kdgb_sm_partition_destroy synchronises and destroys them, after the
 * graphs captured on them are destroyed.  KDGB_ERR_UNSUPPORTED when the
 * driver has no green contexts. */
typedef struct kdgb_sm_partition kdgb_sm_partition;

KDGB_API int kdgb_sm_partition_create(int32_t sms, kdgb_sm_partition **out);
KDGB_API int kdgb_sm_partition_sms(const kdgb_sm_partition *part, int32_t which, int32_t *sms);
KDGB_API int kdgb_sm_partition_stream(kdgb_sm_partition *part, int32_t which, int32_t priority,
                                      kdgb_stream_t *out);
KDGB_API int kdgb_sm_partition_destroy(kdgb_sm_partition *part);

/* Autotuner (no reference counterpart).  Picks leaf_size (16/24/32),
 * sah_bins (8/16/32, tuned mode only), stack_depth (2/4/8, short-stack
 * only), block_size (64/128/256) and the schedule (grid or queue) for a
 * workload by coordinate descent from `build` / `trace`, scoring each
 * candidate by builds_per_trace * rebuild_ms + trace_ms (median of `reps`
 * timed runs on `stream`; 1 = rebuild every frame, 0 = a static scene).
 * rebuild_ms is a graph rebuild (kdgb_graph_launch), as a per-frame rebuild
 * runs; a host-driven rebuild before it only sizes the graph.  The workload is
 * one mesh (n_meshes = 1, mesh_offsets NULL) or a batch (HOST mesh_offsets
 * as in kdgb_build_batch, rays by ray_mesh_dev or rays_per_mesh); n_rays
 * may be 0 to tune the build alone.  Candidates that fail (a tree that does
 * not terminate within 4 levels more than the starting one, or no memory)
 * are skipped.  Synchronises the stream; allocates a temporary tree. */
typedef struct kdgb_autotune_result {
    kdgb_build_params build; /* chosen build parameters */
    kdgb_trace_params trace; /* chosen trace parameters */
    float build_ms;          /* rebuild time of the choice */
    float trace_ms;          /* trace time of the choice */
    float baseline;          /* objective of the starting parameters */
    float objective;         /* objective of the choice (<= baseline) */
    int32_t trials;          /* candidates measured */
} kdgb_autotune_result;

KDGB_API int kdgb_autotune(const float *tri_v_dev, int32_t n_tris, const int32_t *mesh_offsets, int32_t n_meshes,
                           const float *ray_o_dev, const float *ray_d_dev, const int32_t *ray_mesh_dev,
                           int32_t rays_per_mesh, int32_t n_rays, const kdgb_build_params *build,
                           const kdgb_trace_params *trace, float builds_per_trace, int32_t reps,
                           kdgb_autotune_result *out, kdgb_stream_t stream);

/* Adjoint of first-hit t, u, v with respect to vertex positions (no
 * reference counterpart).  vertices: n_vertices*3 floats; indices:
 * n_tris*3 vertex ids (the index buffer of CUDAMeshNode, CUDAMeshNode.h:36);
 * hit: the triangle ids a forward trace recorded for the n rays (reused, not
 * re-traced; -1 = no contribution); dL_dt/du/dv: upstream gradients per ray.
 * ADDS dL/dvertex (n_vertices*3) into dL_dvertex_dev with warp-aggregated
 * float atomics (summation order, hence the last bits, are not
 * deterministic). */
KDGB_API int kdgb_backward(const float *vertices_dev, int32_t n_vertices, const uint32_t *indices_dev,
                           int32_t n_tris, const float *ray_o_dev, const float *ray_d_dev, int32_t n,
                           const int32_t *hit_dev, const float *dL_dt_dev, const float *dL_du_dev,
                           const float *dL_dv_dev, float *dL_dvertex_dev, kdgb_stream_t stream);

/* Replaces GeometryList::AddMesh(CUDAMeshNode*) (GeometryList.cu:318-341,
 * kernel AddMeshKernel :197-232): gathers n_indices/3 triangles of an
 * indexed mesh (vertices: n_vertices float4) and applies the row-major
 * model matrix `model` (16 host floats, NULL = identity) to each vertex,
 * writing the T x 9 triangle buffer kdgb_build takes.  An index outside the
 * vertex buffer yields a NaN triangle (kdgb_build then reports
 * KDGB_ERR_NONFINITE). */
KDGB_API int kdgb_geometry_gather(const float *vertices_dev, int32_t n_vertices, const uint32_t *indices_dev,
                                  int32_t n_indices, const float model[16], float *tri_v_out_dev,
                                  kdgb_stream_t stream);

/* The normal and colour half of GeometryList::AddMesh (GeometryList.cu:
 * 224-230): per triangle of the index buffer, the three vertex normals
 * (n_vertices float4) times the row-major 3x3 normal matrix (NULL =
 * identity; w = 0) into n0/n1/n2, and the first vertex's colour (n_vertices
 * uchar4) into c0: the inputs of kdgb_trace_shaded. */
KDGB_API int kdgb_geometry_gather_attributes(const float *normals_dev, const uint8_t *colors_dev, int32_t n_vertices,
                                             const uint32_t *indices_dev, int32_t n_indices,
                                             const float normal_matrix[9], float *n0_out_dev, float *n1_out_dev,
                                             float *n2_out_dev, uint8_t *c0_out_dev, kdgb_stream_t stream);

/* Replaces OscCUDAMeshNode::Handle (OscCUDAMeshNode.cu:96-107, kernel
 * UpdateSurface :75-94): moves the (detail+1)^2 float4 vertices and normals
 * of the oscillating height field to time `time` (the reference passes its
 * accumulated microseconds / 700000). */
KDGB_API int kdgb_osc_update_surface(float *vertices_dev, float *normals_dev, int32_t detail, float height,
                                     float time, kdgb_stream_t stream);

/* Replaces BruteTracer::Trace without a tree (BruteTracer.cu:54-96), with
 * the 4096-triangle cap of BruteTracer.cu:50 lifted. */
KDGB_API int kdgb_trace_brute(const float *tri_v_dev, int32_t n_tris, int32_t tie,
                     const float *ray_o_dev, const float *ray_d_dev, int32_t n,
                     int32_t *hit_dev, float *t_dev, float *u_dev, float *v_dev,
                     kdgb_stream_t stream);

/* Check of the bounded device-side waits (no counterpart in the reference,
 * which ignores CUDPP's return codes, TriangleMapUpperCreator.cu:58-76).
 * Runs one block of the look-back scan on a tile whose predecessor never
 * publishes its status, with the wait limited to spin_limit polls (>= 1;
 * the library's own scans allow 2^22).  The wait gives up, records its
 * status in *recorded_status (KDGB_ERR_TIMEOUT) and finishes the tile with
 * the missing prefix counted as *assumed_prefix (0); the device stays
 * usable.  Allocates a few KB, synchronises `stream`. */
KDGB_API int kdgb_check_scan_giveup(int32_t spin_limit, int32_t *recorded_status, int32_t *assumed_prefix,
                                    kdgb_stream_t stream);

/* Largest triangle count kdgb_trace_brute_noalloc accepts. */
#define KDGB_NOALLOC_MAX_TRIS 65536

/* No counterpart in the reference.  The same first-hit brute-force trace as
 * kdgb_trace_brute, for callers that cannot allocate device memory while
 * they run: a frame loop that must not stall on cudaMalloc's implicit device
 * synchronisation, or a host application whose own allocator has already
 * reserved the device's memory.  It calls no cudaMalloc, cudaFree or other
 * allocating routine; its scratch is a fixed device array of
 * KDGB_NOALLOC_MAX_TRIS packed triangles (3 MiB) inside the library, held by
 * every GPU that loads the library until the process exits.
 *  - n_tris > KDGB_NOALLOC_MAX_TRIS is rejected with KDGB_ERR_CAPACITY.
 *  - The first call on a device looks up the array's device address
 *    (cudaGetSymbolAddress) with that device current and caches it with the
 *    id of the device's context; make that first call before any stream
 *    capture (such a call is refused with KDGB_ERR_UNSUPPORTED).  After
 *    cudaDeviceReset the context id changes and the next call looks the
 *    address up again, so it too must come before any capture.
 *  - All calls share the one array and each call overwrites the part it
 *    uses; calls whose work overlaps on the GPU (other streams, other host
 *    threads) race on it and must be serialised by the caller. */
KDGB_API int kdgb_trace_brute_noalloc(const float *tri_v_dev, int32_t n_tris, int32_t tie,
                                      const float *ray_o_dev, const float *ray_d_dev, int32_t n,
                                      int32_t *hit_dev, float *t_dev, float *u_dev, float *v_dev,
                                      kdgb_stream_t stream);

#ifdef __cplusplus
}
#endif
#endif
