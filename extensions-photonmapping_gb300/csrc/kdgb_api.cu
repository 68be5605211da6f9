// C ABI of the kd-tree builder and tracers (include/kdgb.h).
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <mutex>
#include <new>
#include <string>
#include <vector>

#include "kdgb_internal.cuh"

namespace kdgb {

int trace_launch(const Tree &t, const kdgb_trace_params &p, const float *o, const float *d, int64_t n,
                 int32_t *hit, float *tt, float *uu, float *vv, int32_t *occ, const float *light, cudaStream_t s,
                 const int32_t *ray_mesh = nullptr, int32_t rays_per_mesh = 0, unsigned long long *counts = nullptr);
int shadow_launch(const Tree &t, const kdgb_trace_params &p, const float *pts, int64_t n, const float *light,
                  int32_t *occ, cudaStream_t s);
int brute_launch(const float4 *p0, const float4 *p1, const float4 *p2, const float4 *woop, int32_t T, int tie,
                 const float *o, const float *d, int64_t n, int32_t *hit, float *tt, float *uu, float *vv,
                 cudaStream_t s);
int photon_launch(const Tree &t, const kdgb_trace_params &p, const kdgb_photon_params &ph, int64_t n,
                  int32_t *seg_hit, float *seg_t, cudaStream_t s);
int shade_launch(const Tree &t, const kdgb_trace_params &p, const float *n0, const float *n1, const float *n2,
                 const uint8_t *c0, const kdgb_light &light, int max_bounces, const float *o, const float *d, int64_t n,
                 uint8_t *rgba, cudaStream_t s);

namespace {
thread_local std::string g_last_error;
std::once_flag g_pool_once;

// Stream-ordered allocations come from the device's default pool; keeping
// freed blocks cached makes per-level scratch allocations cheap.
void setup_pool()
{
    std::call_once(g_pool_once, [] {
        int dev = 0;
        if (cudaGetDevice(&dev) != cudaSuccess) return;
        cudaMemPool_t pool;
        if (cudaDeviceGetDefaultMemPool(&pool, dev) != cudaSuccess) return;
        uint64_t thr = UINT64_MAX;
        cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
    });
}
}  // namespace

static std::atomic<int64_t> g_launches{0};

void note_launch(int n) { g_launches.fetch_add(n, std::memory_order_relaxed); }

void set_error(const std::string &msg) { g_last_error = msg; }

int fail(int status, const std::string &msg)
{
    g_last_error = msg;
    return status;
}

int cuda_fail(cudaError_t e, const char *what)
{
    g_last_error = std::string(what) + ": " + cudaGetErrorString(e);
    cudaGetLastError();  // clear a non-sticky error
    return e == cudaErrorMemoryAllocation ? KDGB_ERR_OUT_OF_MEMORY : KDGB_ERR_CUDA;
}

template <class T>
int ensure(DevArray<T> &a, int64_t n, cudaStream_t s, int64_t keep, bool zero)
{
    if (n <= a.cap && a.p) return KDGB_OK;
    const int64_t cap = n > 0 ? n : 1;
    T *p = nullptr;
    KDGB_CUDA(cudaMallocAsync(&p, sizeof(T) * (size_t)cap, s));
    if (zero) {
        cudaError_t e = cudaMemsetAsync(p, 0, sizeof(T) * (size_t)cap, s);
        if (e != cudaSuccess) { cudaFreeAsync(p, s); return cuda_fail(e, "cudaMemsetAsync"); }
    }
    if (a.p && keep > 0) {
        cudaError_t e = cudaMemcpyAsync(p, a.p, sizeof(T) * (size_t)keep, cudaMemcpyDeviceToDevice, s);
        if (e != cudaSuccess) { cudaFreeAsync(p, s); return cuda_fail(e, "cudaMemcpyAsync"); }
    }
    if (a.p) cudaFreeAsync(a.p, s);
    a.p = p;
    a.cap = cap;
    return KDGB_OK;
}

template <class T>
void release(DevArray<T> &a, cudaStream_t s)
{
    if (a.p) cudaFreeAsync(a.p, s);
    a.p = nullptr;
    a.cap = 0;
}

template int ensure<int8_t>(DevArray<int8_t> &, int64_t, cudaStream_t, int64_t, bool);
template int ensure<float>(DevArray<float> &, int64_t, cudaStream_t, int64_t, bool);
template int ensure<float4>(DevArray<float4> &, int64_t, cudaStream_t, int64_t, bool);
template int ensure<int32_t>(DevArray<int32_t> &, int64_t, cudaStream_t, int64_t, bool);
template int ensure<int2>(DevArray<int2> &, int64_t, cudaStream_t, int64_t, bool);
template int ensure<int4>(DevArray<int4> &, int64_t, cudaStream_t, int64_t, bool);
template int ensure<unsigned>(DevArray<unsigned> &, int64_t, cudaStream_t, int64_t, bool);
template int ensure<float2>(DevArray<float2> &, int64_t, cudaStream_t, int64_t, bool);
template int ensure<BuildState>(DevArray<BuildState> &, int64_t, cudaStream_t, int64_t, bool);

static void release_all(Tree &t, cudaStream_t s)
{
    release(t.p0, s); release(t.p1, s); release(t.p2, s); release(t.prec, s);
    release(t.info, s); release(t.split, s); release(t.bmin, s); release(t.bmax, s);
    release(t.pidx, s); release(t.bitmap, s); release(t.parent, s); release(t.children, s);
    release(t.area, s); release(t.prim_indices, s); release(t.leaf_ids, s);
    release(t.tnode, s); release(t.tbox, s); release(t.ttri, s); release(t.mesh_off, s); release(t.woop, s);
    release(t.mesh_order, s); release(t.qctr, s);
    t.woop_valid = false;
    Workspace &w = t.ws;
    for (int b = 0; b < 2; ++b) {
        release(w.rmin[b], s);
        release(w.rmax[b], s);
    }
    release(w.fmin, s); release(w.fmax, s); release(w.keys, s);
    for (int b = 0; b < 2; ++b) { release(w.planes[b], s); release(w.ess[b], s); }
    release(w.cnt, s); release(w.lbase, s); release(w.chunksum, s);
    release(w.tilesum, s); release(w.tileoff, s); release(w.stats, s); release(w.scan, s); release(w.misc0, s); release(w.misc1, s);
    release(w.big, s); release(w.bighist, s); release(w.areas, s); release(w.sts, s); release(w.ssplit, s); release(w.lcnt[0], s); release(w.lcnt[1], s);
    release(w.roff, s); release(w.careas, s); release(w.csets, s); release(w.ranges, s); release(w.state, s);
    release(w.lowlist[0], s); release(w.lowlist[1], s);
    t.plan = BuildPlan();
    if (w.host) {
        cudaStreamSynchronize(s);
        cudaFreeHost(w.host);
        w.host = nullptr;
    }
}

static int check_device()
{
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess || n == 0) {
        cudaGetLastError();
        return fail(KDGB_ERR_NO_DEVICE, "no CUDA device available");
    }
    setup_pool();
    return KDGB_OK;
}

static int validate_build_params(const kdgb_build_params &p)
{
    if (p.mode != KDGB_BUILD_REFERENCE && p.mode != KDGB_BUILD_TUNED)
        return fail(KDGB_ERR_INVALID_ARGUMENT, "unknown build mode");
    if (p.lower != KDGB_LOWER_BITMAP && p.lower != KDGB_LOWER_SAH && p.lower != KDGB_LOWER_BALANCED)
        return fail(KDGB_ERR_INVALID_ARGUMENT, "unknown lower algorithm");
    if (p.split_method == KDGB_SPLIT_SPLIT)
        return fail(KDGB_ERR_UNSUPPORTED, "split method SPLIT is not implemented (as in the reference)");
    if (p.split_method != KDGB_SPLIT_BOX && p.split_method != KDGB_SPLIT_DIVIDE)
        return fail(KDGB_ERR_INVALID_ARGUMENT, "unknown split method");
    if (p.leaf_size < 1 || p.leaf_size > 32) return fail(KDGB_ERR_INVALID_ARGUMENT, "leaf_size must be in 1..32");
    if (p.max_levels < 1 || p.max_levels > 4096) return fail(KDGB_ERR_INVALID_ARGUMENT, "max_levels out of range");
    if (!std::isfinite(p.empty_space_threshold) || !std::isfinite(p.traversal_cost) ||
        !std::isfinite(p.intersection_cost))
        return fail(KDGB_ERR_INVALID_ARGUMENT, "non-finite cost parameter");
    // A negative cost lets the balanced rule split a node into itself and an
    // empty child forever.
    if (p.lower == KDGB_LOWER_BALANCED && p.traversal_cost < 0.0f)
        return fail(KDGB_ERR_INVALID_ARGUMENT, "balanced lower creator needs traversal_cost >= 0");
    if (p.mode == KDGB_BUILD_TUNED && (p.upper_levels < 0 || p.sah_bins < 2 || p.sah_bins > 32))
        return fail(KDGB_ERR_INVALID_ARGUMENT, "tuned build: upper_levels >= 0, sah_bins in 2..32");
    return KDGB_OK;
}

static int validate_offsets(const int32_t *mesh_offsets, int32_t n_meshes, const char *who)
{
    if (n_meshes < 1 || !mesh_offsets) return fail(KDGB_ERR_INVALID_ARGUMENT, std::string(who) + ": no meshes");
    if (mesh_offsets[0] != 0) return fail(KDGB_ERR_INVALID_ARGUMENT, std::string(who) + ": mesh_offsets[0] must be 0");
    for (int32_t m = 0; m < n_meshes; ++m)
        if (mesh_offsets[m + 1] < mesh_offsets[m])
            return fail(KDGB_ERR_INVALID_ARGUMENT, std::string(who) + ": mesh_offsets must be non-decreasing");
    return KDGB_OK;
}

static int validate_trace_params(const kdgb_trace_params &p, int64_t n)
{
    if (p.tracer < KDGB_TRACER_RESTART || p.tracer > KDGB_TRACER_BRUTE)
        return fail(KDGB_ERR_INVALID_ARGUMENT, "unknown tracer");
    if (p.tie != KDGB_TIE_LOWEST_ID && p.tie != KDGB_TIE_REF_LAST) return fail(KDGB_ERR_INVALID_ARGUMENT, "unknown tie rule");
    if (p.stack_depth < 1 || p.stack_depth > 8) return fail(KDGB_ERR_INVALID_ARGUMENT, "stack_depth must be in 1..8");
    if (p.block_size < 0 || p.block_size > 1024 || (p.block_size % 32) != 0)
        return fail(KDGB_ERR_INVALID_ARGUMENT, "block_size must be 0 or a multiple of 32 up to 1024");
    if (p.max_iterations < 0) return fail(KDGB_ERR_INVALID_ARGUMENT, "max_iterations must be >= 0");
    if (p.tile_width < 0) return fail(KDGB_ERR_INVALID_ARGUMENT, "tile_width must be >= 0");
    if (p.intersection != KDGB_ISECT_MOELLER && p.intersection != KDGB_ISECT_WOOP)
        return fail(KDGB_ERR_INVALID_ARGUMENT, "unknown intersection algorithm");
    if (p.schedule != KDGB_SCHEDULE_GRID && p.schedule != KDGB_SCHEDULE_QUEUE)
        return fail(KDGB_ERR_INVALID_ARGUMENT, "unknown schedule");
    if (p.tile_width > 0 && (p.tile_width % 4 != 0 || n % ((int64_t)p.tile_width * 8) != 0))
        return fail(KDGB_ERR_INVALID_ARGUMENT, "tile_width needs width % 4 == 0 and height % 8 == 0");
    return KDGB_OK;
}

// The batch's meshes ordered by triangle count, largest first (ties by
// mesh index), for queue-scheduled traces.
static int set_mesh_order(Tree &t, const int32_t *mesh_off_host, int32_t n_meshes, cudaStream_t s)
{
    std::vector<int32_t> order(n_meshes);
    for (int32_t m = 0; m < n_meshes; ++m) order[m] = m;
    std::stable_sort(order.begin(), order.end(), [&](int32_t x, int32_t y) {
        return mesh_off_host[x + 1] - mesh_off_host[x] > mesh_off_host[y + 1] - mesh_off_host[y];
    });
    KDGB_CHECK(ensure(t.mesh_order, n_meshes, s));
    KDGB_CUDA(cudaMemcpyAsync(t.mesh_order.p, order.data(), sizeof(int32_t) * n_meshes, cudaMemcpyHostToDevice, s));
    KDGB_CUDA(cudaStreamSynchronize(s));  // the host vector goes out of scope
    return KDGB_OK;
}

static int do_build(Tree &t, const float *tri_v_dev, int32_t n_tris, const kdgb_build_params &p, cudaStream_t s,
                    const int32_t *mesh_off_host = nullptr, int32_t n_meshes = 1)
{
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    KDGB_CUDA(cudaEventCreate(&e0));
    KDGB_CUDA(cudaEventCreate(&e1));
    cudaEventRecord(e0, s);
    int rc = KDGB_OK;
    t.n_meshes = n_meshes > 1 ? n_meshes : 1;
    if (n_meshes > 1) {
        rc = ensure(t.mesh_off, (int64_t)n_meshes + 1, s);
        if (rc == KDGB_OK) {
            const cudaError_t e = cudaMemcpyAsync(t.mesh_off.p, mesh_off_host, sizeof(int32_t) * (n_meshes + 1),
                                                  cudaMemcpyHostToDevice, s);
            if (e != cudaSuccess) rc = cuda_fail(e, "mesh offsets");
        }
        if (rc == KDGB_OK) rc = set_mesh_order(t, mesh_off_host, n_meshes, s);
    }
    if (rc == KDGB_OK) rc = build_tree(t, tri_v_dev, n_tris, p, s, n_meshes > 1 ? t.mesh_off.p : nullptr, t.n_meshes);
    cudaEventRecord(e1, s);
    if (rc == KDGB_OK) {
        cudaError_t e = cudaEventSynchronize(e1);
        if (e != cudaSuccess) rc = cuda_fail(e, "build");
        float ms = 0.0f;
        cudaEventElapsedTime(&ms, e0, e1);
        t.stats.build_ms = ms;
        t.stats.n_nodes = t.n_nodes;
        t.stats.n_refs = t.n_refs;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return rc;
}

}  // namespace kdgb

using namespace kdgb;

struct kdgb_graph {
    kdgb_tree *tree = nullptr;
    cudaStream_t cs = nullptr, body = nullptr;
    Fork fork;  // the side branch of the captured build
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    uint64_t signature = 0;
    GraphKernels kernels;
    int64_t trace_kernels = 0;
    int64_t per_launch = 0;  // kernels one launch runs at the plan's level counts
};

extern "C" {

int kdgb_abi_version(void) { return KDGB_ABI_VERSION; }

const char *kdgb_status_string(int status)
{
    switch (status) {
    case KDGB_OK: return "ok";
    case KDGB_ERR_INVALID_ARGUMENT: return "invalid argument";
    case KDGB_ERR_CUDA: return "CUDA error";
    case KDGB_ERR_OUT_OF_MEMORY: return "out of device memory";
    case KDGB_ERR_CAPACITY: return "capacity exceeded";
    case KDGB_ERR_DEGENERATE: return "degenerate input";
    case KDGB_ERR_NONFINITE: return "non-finite input";
    case KDGB_ERR_TIMEOUT: return "device wait timed out";
    case KDGB_ERR_UNSUPPORTED: return "unsupported";
    case KDGB_ERR_NO_DEVICE: return "no CUDA device";
    default: return "unknown status";
    }
}

const char *kdgb_last_error(void) { return g_last_error.c_str(); }

int64_t kdgb_launch_count(void) { return g_launches.load(std::memory_order_relaxed); }

void kdgb_build_params_default(kdgb_build_params *p)
{
    if (!p) return;
    p->mode = KDGB_BUILD_REFERENCE;
    p->lower = KDGB_LOWER_BITMAP;
    p->split_empty_space = 1;
    p->propagate_aabbs = 1;
    p->empty_space_threshold = 0.35f;
    p->traversal_cost = 24.0f;
    p->intersection_cost = 1.0f;
    p->min_leaf = 0;
    p->esc_zmax_as_x = 1;
    p->max_levels = 64;
    p->leaf_size = 32;
    p->upper_levels = 8;
    p->sah_bins = 32;
    p->split_method = KDGB_SPLIT_BOX;
}

void kdgb_trace_params_default(kdgb_trace_params *p)
{
    if (!p) return;
    p->tracer = KDGB_TRACER_RESTART;
    p->leaf_skipping = 1;
    p->tie = KDGB_TIE_LOWEST_ID;
    p->stack_depth = 4;
    p->max_iterations = 0;
    p->block_size = 0;
    p->tile_width = 0;
    p->schedule = KDGB_SCHEDULE_GRID;
    p->intersection = KDGB_ISECT_MOELLER;
}

int kdgb_build(const float *tri_v_dev, int32_t n_tris, const kdgb_build_params *params, kdgb_tree **out,
               kdgb_stream_t stream)
{
    if (!out) return fail(KDGB_ERR_INVALID_ARGUMENT, "out is NULL");
    *out = nullptr;
    if (n_tris < 0 || (n_tris > 0 && !tri_v_dev)) return fail(KDGB_ERR_INVALID_ARGUMENT, "bad triangle buffer");
    KDGB_CHECK(check_device());
    kdgb_build_params p;
    if (params) p = *params; else kdgb_build_params_default(&p);
    KDGB_CHECK(validate_build_params(p));
    kdgb_tree *h = new (std::nothrow) kdgb_tree();
    if (!h) return fail(KDGB_ERR_OUT_OF_MEMORY, "host allocation");
    cudaStream_t s = (cudaStream_t)stream;
    const int rc = do_build(h->t, tri_v_dev, n_tris, p, s);
    if (rc != KDGB_OK) {
        release_all(h->t, s);
        cudaStreamSynchronize(s);
        delete h;
        return rc;
    }
    *out = h;
    return KDGB_OK;
}

int kdgb_rebuild(kdgb_tree *tree, const float *tri_v_dev, int32_t n_tris, const kdgb_build_params *params,
                 kdgb_stream_t stream)
{
    if (!tree) return fail(KDGB_ERR_INVALID_ARGUMENT, "tree is NULL");
    if (n_tris < 0 || (n_tris > 0 && !tri_v_dev)) return fail(KDGB_ERR_INVALID_ARGUMENT, "bad triangle buffer");
    KDGB_CHECK(check_device());
    kdgb_build_params p;
    if (params) p = *params; else kdgb_build_params_default(&p);
    KDGB_CHECK(validate_build_params(p));
    return do_build(tree->t, tri_v_dev, n_tris, p, (cudaStream_t)stream);
}

int kdgb_tree_upload(const kdgb_tree_view *a, const float *tri_v_host, int32_t n_tris, kdgb_tree **out,
                     kdgb_stream_t stream)
{
    if (!out || !a) return fail(KDGB_ERR_INVALID_ARGUMENT, "NULL argument");
    *out = nullptr;
    const int32_t n = a->n_nodes, r = a->n_refs, nl = a->n_upper_leaves;
    if (n < 1 || r < 0 || nl < 0 || n_tris < 0 || (n_tris > 0 && !tri_v_host) || !a->info || !a->split ||
        !a->aabb_min || !a->aabb_max || !a->prim_index || !a->bitmap || !a->children ||
        (r > 0 && !a->prim_indices))
        return fail(KDGB_ERR_INVALID_ARGUMENT, "incomplete tree arrays");
    // Validate everything the tracers dereference so a malformed tree is an
    // error here rather than an out-of-bounds access on the device.
    for (int32_t i = 0; i < n; ++i) {
        const int axis = a->info[i];
        if (axis < 0 || axis > 3) return fail(KDGB_ERR_INVALID_ARGUMENT, "info out of range");
        if (axis == KDGB_LEAF) {
            const uint32_t bmp = (uint32_t)a->bitmap[i];
            if (bmp) {
                const int hi = 31 - __builtin_clz(bmp);
                if (a->prim_index[i] < 0 || (int64_t)a->prim_index[i] + hi >= r)
                    return fail(KDGB_ERR_INVALID_ARGUMENT, "leaf references out of range");
            }
        } else {
            const int32_t c0 = a->children[2 * i], c1 = a->children[2 * i + 1];
            if (c0 < 0 || c0 >= n || c1 < 0 || c1 >= n) return fail(KDGB_ERR_INVALID_ARGUMENT, "child out of range");
        }
    }
    for (int32_t i = 0; i < r; ++i)
        if (a->prim_indices[i] < 0 || a->prim_indices[i] >= n_tris)
            return fail(KDGB_ERR_INVALID_ARGUMENT, "primitive index out of range");
    KDGB_CHECK(check_device());
    cudaStream_t s = (cudaStream_t)stream;
    kdgb_tree *h = new (std::nothrow) kdgb_tree();
    if (!h) return fail(KDGB_ERR_OUT_OF_MEMORY, "host allocation");
    Tree &t = h->t;
    int rc = KDGB_OK;
    float *dtri = nullptr;
    std::vector<float> zeros;
    do {
        if ((rc = ensure(t.info, n, s)) || (rc = ensure(t.split, n, s)) || (rc = ensure(t.bmin, n, s)) ||
            (rc = ensure(t.bmax, n, s)) || (rc = ensure(t.pidx, n, s)) || (rc = ensure(t.bitmap, n, s)) ||
            (rc = ensure(t.children, n, s)) || (rc = ensure(t.area, n, s, 0, true)) ||
            (rc = ensure(t.parent, n, s, 0, true)) || (rc = ensure(t.prim_indices, r, s)) ||
            (rc = ensure(t.leaf_ids, nl, s)))
            break;
        cudaError_t e = cudaSuccess;
        auto up = [&](void *dst, const void *src, size_t bytes) {
            if (e == cudaSuccess && bytes && src) e = cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, s);
        };
        up(t.info.p, a->info, (size_t)n);
        up(t.split.p, a->split, 4 * (size_t)n);
        up(t.bmin.p, a->aabb_min, 16 * (size_t)n);
        up(t.bmax.p, a->aabb_max, 16 * (size_t)n);
        up(t.pidx.p, a->prim_index, 4 * (size_t)n);
        up(t.bitmap.p, a->bitmap, 4 * (size_t)n);
        up(t.children.p, a->children, 8 * (size_t)n);
        up(t.area.p, a->area, 4 * (size_t)n);
        up(t.parent.p, a->parent, 4 * (size_t)n);
        up(t.prim_indices.p, a->prim_indices, 4 * (size_t)r);
        up(t.leaf_ids.p, a->leaf_ids, 4 * (size_t)nl);
        if (e != cudaSuccess) { rc = cuda_fail(e, "tree upload"); break; }
        if (n_tris > 0) {
            if ((e = cudaMallocAsync(&dtri, sizeof(float) * 9 * (size_t)n_tris, s)) != cudaSuccess ||
                (e = cudaMemcpyAsync(dtri, tri_v_host, sizeof(float) * 9 * (size_t)n_tris, cudaMemcpyHostToDevice, s)) !=
                    cudaSuccess) {
                rc = cuda_fail(e, "triangle upload");
                break;
            }
        }
        if ((rc = load_geometry(t, dtri, n_tris, s))) break;
        t.n_nodes = n;
        t.n_refs = r;
        t.n_upper_leaves = nl;
        if ((rc = pack_for_traversal(t, s))) break;
        if ((e = cudaStreamSynchronize(s)) != cudaSuccess) { rc = cuda_fail(e, "tree upload"); break; }
    } while (0);
    if (dtri) cudaFreeAsync(dtri, s);
    if (rc != KDGB_OK) {
        release_all(t, s);
        cudaStreamSynchronize(s);
        delete h;
        return rc;
    }
    t.stats.n_nodes = n;
    t.stats.n_refs = r;
    *out = h;
    return KDGB_OK;
}

int kdgb_tree_destroy(kdgb_tree *tree)
{
    if (!tree) return KDGB_OK;
    release_all(tree->t, 0);
    cudaError_t e = cudaStreamSynchronize(0);
    delete tree;
    if (e != cudaSuccess) return cuda_fail(e, "kdgb_tree_destroy");
    return KDGB_OK;
}

int kdgb_tree_release(kdgb_tree *tree, kdgb_stream_t stream)
{
    if (!tree) return KDGB_OK;
    cudaStream_t s = (cudaStream_t)stream;
    release_all(tree->t, s);
    cudaError_t e = cudaStreamSynchronize(s);
    delete tree;
    if (e != cudaSuccess) return cuda_fail(e, "kdgb_tree_release");
    return KDGB_OK;
}

int kdgb_check_scan_giveup(int32_t spin_limit, int32_t *recorded_status, int32_t *assumed_prefix,
                           kdgb_stream_t stream)
{
    if (!recorded_status || !assumed_prefix) return fail(KDGB_ERR_INVALID_ARGUMENT, "NULL argument");
    int32_t r[2] = {0, 0};
    KDGB_CHECK(scan_giveup_check(spin_limit, r, (cudaStream_t)stream));
    *recorded_status = r[0];
    *assumed_prefix = r[1];
    return KDGB_OK;
}

int kdgb_tree_view_get(const kdgb_tree *tree, kdgb_tree_view *v)
{
    if (!tree || !v) return fail(KDGB_ERR_INVALID_ARGUMENT, "NULL argument");
    const Tree &t = tree->t;
    v->n_nodes = t.n_nodes;
    v->n_refs = t.n_refs;
    v->n_upper_leaves = t.n_upper_leaves;
    v->n_tris = t.n_tris;
    v->info = t.info.p;
    v->split = t.split.p;
    v->aabb_min = reinterpret_cast<float *>(t.bmin.p);
    v->aabb_max = reinterpret_cast<float *>(t.bmax.p);
    v->prim_index = t.pidx.p;
    v->bitmap = t.bitmap.p;
    v->children = reinterpret_cast<int32_t *>(t.children.p);
    v->area = t.area.p;
    v->parent = t.parent.p;
    v->prim_indices = t.prim_indices.p;
    v->leaf_ids = t.leaf_ids.p;
    v->p0 = reinterpret_cast<float *>(t.p0.p);
    v->p1 = reinterpret_cast<float *>(t.p1.p);
    v->p2 = reinterpret_cast<float *>(t.p2.p);
    return KDGB_OK;
}

int kdgb_tree_download(const kdgb_tree *tree, kdgb_tree_view *d)
{
    if (!tree || !d) return fail(KDGB_ERR_INVALID_ARGUMENT, "NULL argument");
    const Tree &t = tree->t;
    const size_t n = (size_t)t.n_nodes, r = (size_t)t.n_refs, nl = (size_t)t.n_upper_leaves;
    cudaError_t e = cudaSuccess;
    auto dn = [&](void *dst, const void *src, size_t bytes) {
        if (e == cudaSuccess && dst && bytes) e = cudaMemcpy(dst, src, bytes, cudaMemcpyDeviceToHost);
    };
    KDGB_CUDA(cudaDeviceSynchronize());
    dn(d->info, t.info.p, n);
    dn(d->split, t.split.p, 4 * n);
    dn(d->aabb_min, t.bmin.p, 16 * n);
    dn(d->aabb_max, t.bmax.p, 16 * n);
    dn(d->prim_index, t.pidx.p, 4 * n);
    dn(d->bitmap, t.bitmap.p, 4 * n);
    dn(d->children, t.children.p, 8 * n);
    dn(d->area, t.area.p, 4 * n);
    dn(d->parent, t.parent.p, 4 * n);
    dn(d->prim_indices, t.prim_indices.p, 4 * r);
    dn(d->leaf_ids, t.leaf_ids.p, 4 * nl);
    dn(d->p0, t.p0.p, 16 * (size_t)t.n_tris);
    dn(d->p1, t.p1.p, 16 * (size_t)t.n_tris);
    dn(d->p2, t.p2.p, 16 * (size_t)t.n_tris);
    if (e != cudaSuccess) return cuda_fail(e, "kdgb_tree_download");
    return KDGB_OK;
}

int kdgb_tree_stats(const kdgb_tree *tree, kdgb_build_stats *stats)
{
    if (!tree || !stats) return fail(KDGB_ERR_INVALID_ARGUMENT, "NULL argument");
    *stats = tree->t.stats;
    return KDGB_OK;
}

int kdgb_trace(const kdgb_tree *tree, const kdgb_trace_params *params, const float *ray_o_dev,
               const float *ray_d_dev, int32_t n, int32_t *hit_dev, float *t_dev, float *u_dev, float *v_dev,
               kdgb_stream_t stream)
{
    if (!tree) return fail(KDGB_ERR_INVALID_ARGUMENT, "tree is NULL");
    kdgb_trace_params p;
    if (params) p = *params; else kdgb_trace_params_default(&p);
    if (n < 0) return fail(KDGB_ERR_INVALID_ARGUMENT, "negative ray count");
    KDGB_CHECK(validate_trace_params(p, n));
    if (n == 0) return KDGB_OK;
    if (!ray_o_dev || !ray_d_dev || !hit_dev || !t_dev || !u_dev || !v_dev)
        return fail(KDGB_ERR_INVALID_ARGUMENT, "NULL ray or output buffer");
    const Tree &t = tree->t;
    if (t.n_meshes > 1) return fail(KDGB_ERR_INVALID_ARGUMENT, "batched tree: use kdgb_trace_batch");
    cudaStream_t s = (cudaStream_t)stream;
    if (p.tracer == KDGB_TRACER_BRUTE) {
        const float4 *woop = nullptr;
        if (p.intersection == KDGB_ISECT_WOOP) {
            KDGB_CHECK(woop_values(t, s));
            woop = t.woop.p;
        }
        return brute_launch(t.p0.p, t.p1.p, t.p2.p, woop, t.n_tris, p.tie, ray_o_dev, ray_d_dev, n, hit_dev, t_dev,
                            u_dev, v_dev, s);
    }
    return trace_launch(t, p, ray_o_dev, ray_d_dev, n, hit_dev, t_dev, u_dev, v_dev, nullptr, nullptr, s);
}

int kdgb_trace_shadow(const kdgb_tree *tree, const kdgb_trace_params *params, const float *points_dev, int32_t n,
                      const float light[3], int32_t *occluded_dev, kdgb_stream_t stream)
{
    if (!tree || !light) return fail(KDGB_ERR_INVALID_ARGUMENT, "NULL argument");
    kdgb_trace_params p;
    if (params) p = *params; else kdgb_trace_params_default(&p);
    if (n < 0) return fail(KDGB_ERR_INVALID_ARGUMENT, "negative point count");
    p.tile_width = 0;
    KDGB_CHECK(validate_trace_params(p, n));
    if (n == 0) return KDGB_OK;
    if (!points_dev || !occluded_dev) return fail(KDGB_ERR_INVALID_ARGUMENT, "NULL buffer");
    if (tree->t.n_meshes > 1) return fail(KDGB_ERR_UNSUPPORTED, "shadow rays of a batched tree");
    return shadow_launch(tree->t, p, points_dev, n, light, occluded_dev, (cudaStream_t)stream);
}

int kdgb_trace_primary_shadow(const kdgb_tree *tree, const kdgb_trace_params *params, const float *ray_o_dev,
                              const float *ray_d_dev, int32_t n, const float light[3], int32_t *hit_dev,
                              float *t_dev, float *u_dev, float *v_dev, int32_t *occluded_dev, kdgb_stream_t stream)
{
    if (!tree || !light) return fail(KDGB_ERR_INVALID_ARGUMENT, "NULL argument");
    kdgb_trace_params p;
    if (params) p = *params; else kdgb_trace_params_default(&p);
    if (n < 0) return fail(KDGB_ERR_INVALID_ARGUMENT, "negative ray count");
    KDGB_CHECK(validate_trace_params(p, n));
    if (p.tracer == KDGB_TRACER_BRUTE) return fail(KDGB_ERR_UNSUPPORTED, "fused shadow rays need a kd tracer");
    if (n == 0) return KDGB_OK;
    if (!ray_o_dev || !ray_d_dev || !hit_dev || !t_dev || !u_dev || !v_dev || !occluded_dev)
        return fail(KDGB_ERR_INVALID_ARGUMENT, "NULL ray or output buffer");
    if (tree->t.n_meshes > 1) return fail(KDGB_ERR_UNSUPPORTED, "shadow rays of a batched tree");
    return trace_launch(tree->t, p, ray_o_dev, ray_d_dev, n, hit_dev, t_dev, u_dev, v_dev, occluded_dev, light,
                        (cudaStream_t)stream);
}

int kdgb_trace_count_steps(const kdgb_tree *tree, const kdgb_trace_params *params, const float *ray_o_dev,
                           const float *ray_d_dev, int32_t n, const float light[3], int32_t *hit_dev, float *t_dev,
                           float *u_dev, float *v_dev, int32_t *occluded_dev, uint64_t counts[8], kdgb_stream_t stream)
{
    if (!tree || !light || !counts) return fail(KDGB_ERR_INVALID_ARGUMENT, "NULL argument");
    kdgb_trace_params p;
    if (params) p = *params; else kdgb_trace_params_default(&p);
    if (n < 0) return fail(KDGB_ERR_INVALID_ARGUMENT, "negative ray count");
    KDGB_CHECK(validate_trace_params(p, n));
    if (p.tracer != KDGB_TRACER_SHORTSTACK) return fail(KDGB_ERR_UNSUPPORTED, "step counts need the short-stack tracer");
    if (tree->t.n_meshes > 1) return fail(KDGB_ERR_UNSUPPORTED, "step counts of a batched tree");
    for (int k = 0; k < 8; ++k) counts[k] = 0;
    if (n == 0) return KDGB_OK;
    if (!ray_o_dev || !ray_d_dev || !hit_dev || !t_dev || !u_dev || !v_dev || !occluded_dev)
        return fail(KDGB_ERR_INVALID_ARGUMENT, "NULL ray or output buffer");
    cudaStream_t s = (cudaStream_t)stream;
    unsigned long long *dev = nullptr;
    KDGB_CUDA(cudaMallocAsync(&dev, 8 * sizeof(unsigned long long), s));
    int rc = cudaMemsetAsync(dev, 0, 8 * sizeof(unsigned long long), s) == cudaSuccess
                 ? trace_launch(tree->t, p, ray_o_dev, ray_d_dev, n, hit_dev, t_dev, u_dev, v_dev, occluded_dev,
                                light, s, nullptr, 0, dev)
                 : cuda_fail(cudaGetLastError(), "kdgb_trace_count_steps");
    unsigned long long host[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    if (rc == KDGB_OK) {
        const cudaError_t e = cudaMemcpyAsync(host, dev, sizeof(host), cudaMemcpyDeviceToHost, s);
        if (e != cudaSuccess) rc = cuda_fail(e, "kdgb_trace_count_steps");
    }
    cudaFreeAsync(dev, s);
    const cudaError_t e = cudaStreamSynchronize(s);
    if (rc == KDGB_OK && e != cudaSuccess) rc = cuda_fail(e, "kdgb_trace_count_steps");
    if (rc == KDGB_OK)
        for (int k = 0; k < 8; ++k) counts[k] = host[k];
    return rc;
}

void kdgb_photon_params_default(kdgb_photon_params *p)
{
    if (!p) return;
    p->light[0] = 0.5f;  // the frame's point light, above the unit cube
    p->light[1] = 3.0f;
    p->light[2] = 0.5f;
    p->seed = 3;
    p->bounces = 3;
    p->survival = 0.7f;
}

int kdgb_trace_photons(const kdgb_tree *tree, const kdgb_trace_params *params, const kdgb_photon_params *photons,
                       int32_t n_photons, int32_t *seg_hit_dev, float *seg_t_dev, kdgb_stream_t stream)
{
    if (!tree || !photons) return fail(KDGB_ERR_INVALID_ARGUMENT, "NULL argument");
    kdgb_trace_params p;
    if (params) p = *params; else kdgb_trace_params_default(&p);
    if (n_photons < 0) return fail(KDGB_ERR_INVALID_ARGUMENT, "negative photon count");
    p.tile_width = 0;
    KDGB_CHECK(validate_trace_params(p, n_photons));
    if (p.tracer == KDGB_TRACER_BRUTE) return fail(KDGB_ERR_UNSUPPORTED, "photon tracing needs a kd tracer");
    if (photons->bounces < 0 || photons->bounces > 64) return fail(KDGB_ERR_INVALID_ARGUMENT, "bounces must be in 0..64");
    if (!(photons->survival >= 0.0f && photons->survival <= 1.0f))
        return fail(KDGB_ERR_INVALID_ARGUMENT, "survival must be in [0, 1]");
    for (int k = 0; k < 3; ++k)
        if (!std::isfinite(photons->light[k])) return fail(KDGB_ERR_INVALID_ARGUMENT, "non-finite light");
    if (n_photons == 0) return KDGB_OK;
    if (!seg_hit_dev || !seg_t_dev) return fail(KDGB_ERR_INVALID_ARGUMENT, "NULL output buffer");
    if (tree->t.n_meshes > 1) return fail(KDGB_ERR_UNSUPPORTED, "photons in a batched tree");
    return photon_launch(tree->t, p, *photons, n_photons, seg_hit_dev, seg_t_dev, (cudaStream_t)stream);
}

void kdgb_light_default(kdgb_light *light)
{
    if (!light) return;
    // Raytracer.cu:43-51: light at (0, 4, 0) with colour (1, 0.92, 0.8)
    // scaled 0.3 / 0.7 / 0.3 for ambient / diffuse / specular.
    const float col[3] = {1.0f, 0.92f, 0.8f};
    light->position[0] = 0.0f;
    light->position[1] = 4.0f;
    light->position[2] = 0.0f;
    for (int k = 0; k < 3; ++k) {
        light->ambient[k] = col[k] * 0.3f;
        light->diffuse[k] = col[k] * 0.7f;
        light->specular[k] = col[k] * 0.3f;
    }
}

int kdgb_trace_shaded(const kdgb_tree *tree, const kdgb_trace_params *params, const float *n0_dev,
                      const float *n1_dev, const float *n2_dev, const uint8_t *c0_dev, const kdgb_light *light,
                      int32_t max_bounces, const float *ray_o_dev, const float *ray_d_dev, int32_t n,
                      uint8_t *rgba_dev, kdgb_stream_t stream)
{
    if (!tree) return fail(KDGB_ERR_INVALID_ARGUMENT, "tree is NULL");
    kdgb_trace_params p;
    if (params) p = *params; else kdgb_trace_params_default(&p);
    if (n < 0) return fail(KDGB_ERR_INVALID_ARGUMENT, "negative ray count");
    KDGB_CHECK(validate_trace_params(p, n));
    if (max_bounces < 0 || max_bounces > 1024) return fail(KDGB_ERR_INVALID_ARGUMENT, "max_bounces must be in 0..1024");
    kdgb_light L;
    if (light) L = *light; else kdgb_light_default(&L);
    for (int k = 0; k < 3; ++k)
        if (!std::isfinite(L.position[k]) || !std::isfinite(L.ambient[k]) || !std::isfinite(L.diffuse[k]) ||
            !std::isfinite(L.specular[k]))
            return fail(KDGB_ERR_INVALID_ARGUMENT, "non-finite light");
    if (tree->t.n_meshes > 1) return fail(KDGB_ERR_UNSUPPORTED, "shading a batched tree");
    if (n == 0) return KDGB_OK;
    if (!ray_o_dev || !ray_d_dev || !rgba_dev) return fail(KDGB_ERR_INVALID_ARGUMENT, "NULL ray or output buffer");
    if (tree->t.n_tris > 0 && (!n0_dev || !n1_dev || !n2_dev || !c0_dev))
        return fail(KDGB_ERR_INVALID_ARGUMENT, "NULL normal or colour buffer");
    return shade_launch(tree->t, p, n0_dev, n1_dev, n2_dev, c0_dev, L, max_bounces > 0 ? max_bounces : 64, ray_o_dev,
                        ray_d_dev, n, rgba_dev, (cudaStream_t)stream);
}

int kdgb_trace_brute_shaded(const float *tri_v_dev, int32_t n_tris, const kdgb_trace_params *params,
                            const float *n0_dev, const float *n1_dev, const float *n2_dev, const uint8_t *c0_dev,
                            const kdgb_light *light, int32_t max_bounces, const float *ray_o_dev,
                            const float *ray_d_dev, int32_t n, uint8_t *rgba_dev, kdgb_stream_t stream)
{
    if (n_tris < 0 || n < 0 || (n_tris > 0 && !tri_v_dev)) return fail(KDGB_ERR_INVALID_ARGUMENT, "bad arguments");
    kdgb_trace_params p;
    if (params) p = *params; else kdgb_trace_params_default(&p);
    p.tracer = KDGB_TRACER_BRUTE;
    KDGB_CHECK(validate_trace_params(p, n));
    if (max_bounces < 0 || max_bounces > 1024) return fail(KDGB_ERR_INVALID_ARGUMENT, "max_bounces must be in 0..1024");
    kdgb_light L;
    if (light) L = *light; else kdgb_light_default(&L);
    if (n == 0) return KDGB_OK;
    if (!ray_o_dev || !ray_d_dev || !rgba_dev) return fail(KDGB_ERR_INVALID_ARGUMENT, "NULL ray or output buffer");
    if (n_tris > 0 && (!n0_dev || !n1_dev || !n2_dev || !c0_dev))
        return fail(KDGB_ERR_INVALID_ARGUMENT, "NULL normal or colour buffer");
    KDGB_CHECK(check_device());
    cudaStream_t s = (cudaStream_t)stream;
    Tree t;
    int rc = load_geometry(t, tri_v_dev, n_tris, s);
    if (rc == KDGB_OK)
        rc = shade_launch(t, p, n0_dev, n1_dev, n2_dev, c0_dev, L, max_bounces > 0 ? max_bounces : 64, ray_o_dev,
                          ray_d_dev, n, rgba_dev, s);
    release_all(t, s);
    return rc;
}

int kdgb_trace_brute_ex(const float *tri_v_dev, int32_t n_tris, const kdgb_trace_params *params,
                        const float *ray_o_dev, const float *ray_d_dev, int32_t n, int32_t *hit_dev, float *t_dev,
                        float *u_dev, float *v_dev, kdgb_stream_t stream)
{
    if (n_tris < 0 || n < 0 || (n_tris > 0 && !tri_v_dev)) return fail(KDGB_ERR_INVALID_ARGUMENT, "bad arguments");
    kdgb_trace_params p;
    if (params) p = *params; else kdgb_trace_params_default(&p);
    p.tracer = KDGB_TRACER_BRUTE;
    p.tile_width = 0;
    KDGB_CHECK(validate_trace_params(p, n));
    if (n == 0) return KDGB_OK;
    if (!ray_o_dev || !ray_d_dev || !hit_dev || !t_dev || !u_dev || !v_dev)
        return fail(KDGB_ERR_INVALID_ARGUMENT, "NULL ray or output buffer");
    KDGB_CHECK(check_device());
    cudaStream_t s = (cudaStream_t)stream;
    Tree t;
    int rc = load_geometry(t, tri_v_dev, n_tris, s);
    const float4 *woop = nullptr;
    if (rc == KDGB_OK && p.intersection == KDGB_ISECT_WOOP) {
        rc = woop_values(t, s);
        woop = t.woop.p;
    }
    if (rc == KDGB_OK)
        rc = brute_launch(t.p0.p, t.p1.p, t.p2.p, woop, n_tris, p.tie, ray_o_dev, ray_d_dev, n, hit_dev, t_dev, u_dev,
                          v_dev, s);
    release_all(t, s);
    return rc;
}

int kdgb_build_batch(const float *tri_v_dev, const int32_t *mesh_offsets, int32_t n_meshes,
                     const kdgb_build_params *params, kdgb_tree **out, kdgb_stream_t stream)
{
    if (!out) return fail(KDGB_ERR_INVALID_ARGUMENT, "out is NULL");
    *out = nullptr;
    KDGB_CHECK(validate_offsets(mesh_offsets, n_meshes, "kdgb_build_batch"));
    const int32_t n_tris = mesh_offsets[n_meshes];
    if (n_tris > 0 && !tri_v_dev) return fail(KDGB_ERR_INVALID_ARGUMENT, "bad triangle buffer");
    KDGB_CHECK(check_device());
    kdgb_build_params p;
    if (params) p = *params; else kdgb_build_params_default(&p);
    KDGB_CHECK(validate_build_params(p));
    kdgb_tree *h = new (std::nothrow) kdgb_tree();
    if (!h) return fail(KDGB_ERR_OUT_OF_MEMORY, "host allocation");
    cudaStream_t s = (cudaStream_t)stream;
    const int rc = do_build(h->t, tri_v_dev, n_tris, p, s, mesh_offsets, n_meshes);
    if (rc != KDGB_OK) {
        release_all(h->t, s);
        cudaStreamSynchronize(s);
        delete h;
        return rc;
    }
    *out = h;
    return KDGB_OK;
}

int kdgb_rebuild_batch(kdgb_tree *tree, const float *tri_v_dev, const int32_t *mesh_offsets, int32_t n_meshes,
                       const kdgb_build_params *params, kdgb_stream_t stream)
{
    if (!tree) return fail(KDGB_ERR_INVALID_ARGUMENT, "tree is NULL");
    KDGB_CHECK(validate_offsets(mesh_offsets, n_meshes, "kdgb_rebuild_batch"));
    const int32_t n_tris = mesh_offsets[n_meshes];
    if (n_tris > 0 && !tri_v_dev) return fail(KDGB_ERR_INVALID_ARGUMENT, "bad triangle buffer");
    KDGB_CHECK(check_device());
    kdgb_build_params p;
    if (params) p = *params; else kdgb_build_params_default(&p);
    KDGB_CHECK(validate_build_params(p));
    return do_build(tree->t, tri_v_dev, n_tris, p, (cudaStream_t)stream, mesh_offsets, n_meshes);
}

int kdgb_trace_batch(const kdgb_tree *tree, const kdgb_trace_params *params, const float *ray_o_dev,
                     const float *ray_d_dev, const int32_t *ray_mesh_dev, int32_t rays_per_mesh, int32_t n,
                     int32_t *hit_dev, float *t_dev, float *u_dev, float *v_dev, kdgb_stream_t stream)
{
    if (!tree) return fail(KDGB_ERR_INVALID_ARGUMENT, "tree is NULL");
    kdgb_trace_params p;
    if (params) p = *params; else kdgb_trace_params_default(&p);
    if (n < 0) return fail(KDGB_ERR_INVALID_ARGUMENT, "negative ray count");
    p.tile_width = 0;
    KDGB_CHECK(validate_trace_params(p, n));
    if (p.tracer == KDGB_TRACER_BRUTE) return fail(KDGB_ERR_UNSUPPORTED, "batched tracing needs a kd tracer");
    if (!ray_mesh_dev && rays_per_mesh < 1)
        return fail(KDGB_ERR_INVALID_ARGUMENT, "kdgb_trace_batch: ray_mesh_dev or rays_per_mesh > 0 required");
    if (!ray_mesh_dev && (int64_t)rays_per_mesh * tree->t.n_meshes < n)
        return fail(KDGB_ERR_INVALID_ARGUMENT, "kdgb_trace_batch: more rays than n_meshes * rays_per_mesh");
    if (n == 0) return KDGB_OK;
    if (!ray_o_dev || !ray_d_dev || !hit_dev || !t_dev || !u_dev || !v_dev)
        return fail(KDGB_ERR_INVALID_ARGUMENT, "NULL ray or output buffer");
    if (tree->t.n_meshes == 1)
        return trace_launch(tree->t, p, ray_o_dev, ray_d_dev, n, hit_dev, t_dev, u_dev, v_dev, nullptr, nullptr,
                            (cudaStream_t)stream);
    return trace_launch(tree->t, p, ray_o_dev, ray_d_dev, n, hit_dev, t_dev, u_dev, v_dev, nullptr, nullptr,
                        (cudaStream_t)stream, ray_mesh_dev, rays_per_mesh);
}

int kdgb_trace_brute(const float *tri_v_dev, int32_t n_tris, int32_t tie, const float *ray_o_dev,
                     const float *ray_d_dev, int32_t n, int32_t *hit_dev, float *t_dev, float *u_dev, float *v_dev,
                     kdgb_stream_t stream)
{
    if (n_tris < 0 || n < 0 || (n_tris > 0 && !tri_v_dev)) return fail(KDGB_ERR_INVALID_ARGUMENT, "bad arguments");
    if (tie != KDGB_TIE_LOWEST_ID && tie != KDGB_TIE_REF_LAST) return fail(KDGB_ERR_INVALID_ARGUMENT, "unknown tie rule");
    if (n == 0) return KDGB_OK;
    if (!ray_o_dev || !ray_d_dev || !hit_dev || !t_dev || !u_dev || !v_dev)
        return fail(KDGB_ERR_INVALID_ARGUMENT, "NULL ray or output buffer");
    KDGB_CHECK(check_device());
    cudaStream_t s = (cudaStream_t)stream;
    Tree t;
    int rc = load_geometry(t, tri_v_dev, n_tris, s);
    if (rc == KDGB_OK)
        rc = brute_launch(t.p0.p, t.p1.p, t.p2.p, nullptr, n_tris, tie, ray_o_dev, ray_d_dev, n, hit_dev, t_dev, u_dev,
                          v_dev, s);
    release_all(t, s);
    return rc;
}

int kdgb_graph_create(kdgb_tree *tree, const float *tri_v_dev, int32_t n_tris, const int32_t *mesh_offsets,
                      int32_t n_meshes, const kdgb_build_params *params, float headroom,
                      const kdgb_trace_params *trace, const float *ray_o_dev, const float *ray_d_dev,
                      const int32_t *ray_mesh_dev, int32_t rays_per_mesh, int32_t n_rays, int32_t *hit_dev,
                      float *t_dev, float *u_dev, float *v_dev, kdgb_graph **out, kdgb_stream_t stream)
{
    if (!out) return fail(KDGB_ERR_INVALID_ARGUMENT, "out is NULL");
    *out = nullptr;
    if (!tree) return fail(KDGB_ERR_INVALID_ARGUMENT, "tree is NULL");
    Tree &t = tree->t;
    if (!t.plan.valid) return fail(KDGB_ERR_INVALID_ARGUMENT, "kdgb_graph_create: build the tree once first");
    if (!(headroom >= 1.0f) || !(headroom <= 64.0f))
        return fail(KDGB_ERR_INVALID_ARGUMENT, "kdgb_graph_create: headroom must be in [1, 64]");
    if (n_meshes < 1) return fail(KDGB_ERR_INVALID_ARGUMENT, "kdgb_graph_create: n_meshes must be >= 1");
    if (n_meshes > 1) {
        KDGB_CHECK(validate_offsets(mesh_offsets, n_meshes, "kdgb_graph_create"));
        if (mesh_offsets[n_meshes] != n_tris)
            return fail(KDGB_ERR_INVALID_ARGUMENT, "kdgb_graph_create: mesh_offsets[n_meshes] != n_tris");
    }
    if (n_tris < 0 || (n_tris > 0 && !tri_v_dev)) return fail(KDGB_ERR_INVALID_ARGUMENT, "bad triangle buffer");
    KDGB_CHECK(check_device());
    kdgb_build_params p;
    if (params) p = *params; else kdgb_build_params_default(&p);
    KDGB_CHECK(validate_build_params(p));
    kdgb_trace_params tp;
    if (trace) tp = *trace; else kdgb_trace_params_default(&tp);
    if (n_rays < 0) return fail(KDGB_ERR_INVALID_ARGUMENT, "negative ray count");
    if (n_rays > 0) {
        if (n_meshes > 1) tp.tile_width = 0;
        KDGB_CHECK(validate_trace_params(tp, n_rays));
        if (tp.tracer == KDGB_TRACER_BRUTE) return fail(KDGB_ERR_UNSUPPORTED, "graph traces need a kd tracer");
        if (!ray_o_dev || !ray_d_dev || !hit_dev || !t_dev || !u_dev || !v_dev)
            return fail(KDGB_ERR_INVALID_ARGUMENT, "NULL ray or output buffer");
        if (n_meshes > 1 && !ray_mesh_dev && (rays_per_mesh < 1 || (int64_t)rays_per_mesh * n_meshes < n_rays))
            return fail(KDGB_ERR_INVALID_ARGUMENT, "kdgb_graph_create: ray_mesh_dev or enough rays_per_mesh needed");
    }
    cudaStream_t s = (cudaStream_t)stream;
    // Offsets and every fixed buffer, before capture.
    t.n_meshes = n_meshes;
    if (n_meshes > 1) {
        KDGB_CHECK(ensure(t.mesh_off, (int64_t)n_meshes + 1, s));
        KDGB_CUDA(cudaMemcpyAsync(t.mesh_off.p, mesh_offsets, sizeof(int32_t) * (n_meshes + 1),
                                  cudaMemcpyHostToDevice, s));
        KDGB_CHECK(set_mesh_order(t, mesh_offsets, n_meshes, s));
    }
    KDGB_CHECK(reserve_for_graph(t, n_tris, p, n_meshes, headroom, s));
    // The queue schedule's counters live in the tree, allocated (zeroed)
    // before capture.
    if (n_rays > 0 && tp.schedule == KDGB_SCHEDULE_QUEUE && !t.qctr.p) KDGB_CHECK(ensure(t.qctr, 2, s, 0, true));
    if (n_rays > 0 && tp.intersection == KDGB_ISECT_WOOP) {
        // The graph recomputes the Woop rows from the rebuilt geometry.
        KDGB_CHECK(ensure(t.woop, 3 * (int64_t)std::max(n_tris, 1), s));
        t.woop_valid = false;
    }
    KDGB_CUDA(cudaStreamSynchronize(s));

    kdgb_graph *g = new (std::nothrow) kdgb_graph();
    if (!g) return fail(KDGB_ERR_OUT_OF_MEMORY, "host allocation");
    g->tree = tree;
    int rc = KDGB_OK;
    // Captured in the context of the caller's stream: for a stream of an SM
    // partition the graph's kernels run on that partition's SMs.
    const StreamContext in_ctx(s);
    cudaError_t e = cudaStreamCreateWithFlags(&g->cs, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&g->body, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&g->fork.aux, cudaStreamNonBlocking);
    for (int i = 0; i < 2 && e == cudaSuccess; ++i) e = cudaEventCreateWithFlags(&g->fork.ev[i], cudaEventDisableTiming);
    if (e != cudaSuccess) rc = cuda_fail(e, "graph streams");
    if (rc == KDGB_OK) {
        e = cudaStreamBeginCapture(g->cs, cudaStreamCaptureModeRelaxed);
        if (e != cudaSuccess) rc = cuda_fail(e, "cudaStreamBeginCapture");
    }
    const int64_t launches0 = kdgb_launch_count();
    if (rc == KDGB_OK) {
        rc = capture_build(t, tri_v_dev, n_tris, p, g->cs, g->body, g->fork, n_meshes > 1 ? t.mesh_off.p : nullptr,
                           n_meshes, g->kernels);
        const int64_t before_trace = kdgb_launch_count();
        if (rc == KDGB_OK && n_rays > 0)
            rc = trace_launch(t, tp, ray_o_dev, ray_d_dev, n_rays, hit_dev, t_dev, u_dev, v_dev, nullptr, nullptr,
                              g->cs, n_meshes > 1 ? ray_mesh_dev : nullptr, n_meshes > 1 ? rays_per_mesh : 0);
        g->trace_kernels = kdgb_launch_count() - before_trace;
        cudaGraph_t graph = nullptr;
        e = cudaStreamEndCapture(g->cs, &graph);
        g->graph = graph;
        if (rc == KDGB_OK && e != cudaSuccess) rc = cuda_fail(e, "cudaStreamEndCapture");
    }
    // Capture launched nothing: take the recorded kernels off the counter.
    note_launch((int)-(kdgb_launch_count() - launches0));
    if (rc == KDGB_OK) {
        e = cudaGraphInstantiate(&g->exec, g->graph, 0);
        if (e != cudaSuccess) rc = cuda_fail(e, "cudaGraphInstantiate");
    }
    {
        const GraphKernels &k = g->kernels;
        g->per_launch = k.fixed + k.upper_body * t.plan.levels + g->trace_kernels +
                        (lower_loop(p) ? k.lower_body * std::max(1, t.plan.low_levels) : 0);
    }
    if (rc != KDGB_OK) {
        kdgb_graph_destroy(g);
        return rc;
    }
    g->signature = layout_signature(t);
    *out = g;
    return KDGB_OK;
}

int kdgb_graph_launch(kdgb_graph *graph, kdgb_stream_t stream)
{
    if (!graph || !graph->exec) return fail(KDGB_ERR_INVALID_ARGUMENT, "graph is NULL");
    if (layout_signature(graph->tree->t) != graph->signature)
        return fail(KDGB_ERR_INVALID_ARGUMENT, "the tree's buffers changed since the graph was created");
    KDGB_CUDA(cudaGraphLaunch(graph->exec, (cudaStream_t)stream));
    graph->tree->t.woop_valid = false;  // the geometry may have moved
    note_launch((int)graph->per_launch);
    return KDGB_OK;
}

int kdgb_graph_status(kdgb_graph *graph, kdgb_stream_t stream)
{
    if (!graph) return fail(KDGB_ERR_INVALID_ARGUMENT, "graph is NULL");
    return read_build_state(graph->tree->t, (cudaStream_t)stream);
}

int kdgb_graph_destroy(kdgb_graph *graph)
{
    if (!graph) return KDGB_OK;
    if (graph->exec) cudaGraphExecDestroy(graph->exec);
    if (graph->graph) cudaGraphDestroy(graph->graph);
    if (graph->body) cudaStreamDestroy(graph->body);
    if (graph->cs) cudaStreamDestroy(graph->cs);
    if (graph->fork.aux) cudaStreamDestroy(graph->fork.aux);
    for (cudaEvent_t ev : graph->fork.ev)
        if (ev) cudaEventDestroy(ev);
    delete graph;
    return KDGB_OK;
}

}  // extern "C"


