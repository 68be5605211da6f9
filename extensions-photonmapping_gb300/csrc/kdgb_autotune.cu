// Autotuner (no reference counterpart): picks the leaf threshold, the SAH
// bin count (tuned mode), the short-stack depth and the trace block size for
// a workload by timing real rebuilds and traces on the caller's stream.
//
// Search: coordinate descent from the caller's parameters, one parameter at
// a time in the order leaf_size, sah_bins, stack_depth, block_size,
// schedule; each
// candidate is scored by builds_per_trace * rebuild_ms + trace_ms, the median
// of `reps` timed repetitions after one warm-up.  rebuild_ms is the time of a
// graph rebuild (kdgb_graph_launch: the whole level loop on the device), the
// way a per-frame rebuild runs; the host-driven rebuild before it only sizes
// the graph's buffers.  Candidates that fail (a
// leaf threshold whose tree does not terminate within a few extra levels, or
// runs out of memory) are skipped.  Every trial goes through the library's
// own entry points, so the winner is a parameter set the oracle can replay.
#include <cuda_runtime.h>

#include <algorithm>
#include <vector>

#include "kdgb_internal.cuh"

namespace kdgb {
namespace {

struct Workload {
    const float *tri;
    int32_t n_tris;
    const int32_t *offsets;
    int32_t n_meshes;
    const float *o, *d;
    const int32_t *ray_mesh;
    int32_t rays_per_mesh, n_rays;
    int32_t *hit;
    float *t, *u, *v;
    cudaStream_t s;
};

struct Score {
    bool ok = false;
    float build_ms = 0.0f, trace_ms = 0.0f;
};

float median(std::vector<float> v)
{
    std::sort(v.begin(), v.end());
    return v.empty() ? 0.0f : v[v.size() / 2];
}

int rebuild(kdgb_tree *tree, const Workload &w, const kdgb_build_params &bp)
{
    if (w.n_meshes > 1) return kdgb_rebuild_batch(tree, w.tri, w.offsets, w.n_meshes, &bp, (kdgb_stream_t)w.s);
    return kdgb_rebuild(tree, w.tri, w.n_tris, &bp, (kdgb_stream_t)w.s);
}

int trace(kdgb_tree *tree, const Workload &w, const kdgb_trace_params &tp)
{
    if (w.n_rays == 0) return KDGB_OK;
    if (w.n_meshes > 1)
        return kdgb_trace_batch(tree, &tp, w.o, w.d, w.ray_mesh, w.rays_per_mesh, w.n_rays, w.hit, w.t, w.u, w.v,
                                (kdgb_stream_t)w.s);
    return kdgb_trace(tree, &tp, w.o, w.d, w.n_rays, w.hit, w.t, w.u, w.v, (kdgb_stream_t)w.s);
}

// Times `reps` graph rebuilds (when `build`) and traces.
Score measure(kdgb_tree *tree, const Workload &w, const kdgb_build_params &bp, const kdgb_trace_params &tp,
              bool build, int reps, cudaEvent_t e0, cudaEvent_t e1, cudaEvent_t e2)
{
    Score sc;
    kdgb_graph *g = nullptr;
    if (build) {
        // A host-driven rebuild sizes the graph's buffers for these
        // parameters; the graph then rebuilds with no host round trip.
        if (rebuild(tree, w, bp) != KDGB_OK) return sc;
        if (kdgb_graph_create(tree, w.tri, w.n_tris, w.n_meshes > 1 ? w.offsets : nullptr, w.n_meshes, &bp, 1.1f,
                              nullptr, nullptr, nullptr, nullptr, 0, 0, nullptr, nullptr, nullptr, nullptr, &g,
                              (kdgb_stream_t)w.s) != KDGB_OK)
            return sc;
    }
    std::vector<float> bt, tt;
    bool ok = true;
    for (int r = 0; r <= reps && ok; ++r) {
        ok = cudaEventRecord(e0, w.s) == cudaSuccess;
        if (ok && g) ok = kdgb_graph_launch(g, (kdgb_stream_t)w.s) == KDGB_OK;
        ok = ok && cudaEventRecord(e1, w.s) == cudaSuccess;
        // The trace reads the tree's host-side counts, which a graph rebuild
        // refreshes at kdgb_graph_status; they equal the sizing rebuild's.
        ok = ok && trace(tree, w, tp) == KDGB_OK;
        ok = ok && cudaEventRecord(e2, w.s) == cudaSuccess && cudaEventSynchronize(e2) == cudaSuccess;
        if (!ok) break;
        float b = 0.0f, t = 0.0f;
        cudaEventElapsedTime(&b, e0, e1);
        cudaEventElapsedTime(&t, e1, e2);
        if (r > 0) {  // the first repetition warms up
            bt.push_back(b);
            tt.push_back(t);
        }
    }
    if (g) {
        if (ok && kdgb_graph_status(g, (kdgb_stream_t)w.s) != KDGB_OK) ok = false;
        kdgb_graph_destroy(g);
    }
    if (!ok) return sc;
    sc.ok = true;
    sc.build_ms = median(bt);
    sc.trace_ms = median(tt);
    return sc;
}

}  // namespace
}  // namespace kdgb

using namespace kdgb;

extern "C" {

int kdgb_autotune(const float *tri_v_dev, int32_t n_tris, const int32_t *mesh_offsets, int32_t n_meshes,
                  const float *ray_o_dev, const float *ray_d_dev, const int32_t *ray_mesh_dev, int32_t rays_per_mesh,
                  int32_t n_rays, const kdgb_build_params *build, const kdgb_trace_params *trace_in,
                  float builds_per_trace, int32_t reps, kdgb_autotune_result *out, kdgb_stream_t stream)
{
    if (!out) return fail(KDGB_ERR_INVALID_ARGUMENT, "out is NULL");
    if (n_meshes < 1) return fail(KDGB_ERR_INVALID_ARGUMENT, "n_meshes must be >= 1");
    if ((n_meshes > 1 && !mesh_offsets) || (mesh_offsets && mesh_offsets[n_meshes] != n_tris))
        return fail(KDGB_ERR_INVALID_ARGUMENT, "kdgb_autotune: mesh_offsets[n_meshes] must equal n_tris");
    if (n_rays < 0 || reps < 1 || reps > 100 || !(builds_per_trace >= 0.0f))
        return fail(KDGB_ERR_INVALID_ARGUMENT, "kdgb_autotune: bad n_rays, reps or builds_per_trace");
    kdgb_build_params bp;
    if (build) bp = *build; else kdgb_build_params_default(&bp);
    kdgb_trace_params tp;
    if (trace_in) tp = *trace_in; else kdgb_trace_params_default(&tp);
    if (tp.tracer == KDGB_TRACER_BRUTE) return fail(KDGB_ERR_UNSUPPORTED, "kdgb_autotune tunes the kd tracers");
    if (n_meshes > 1) tp.tile_width = 0;
    cudaStream_t s = (cudaStream_t)stream;

    Workload w{tri_v_dev, n_tris, mesh_offsets, n_meshes, ray_o_dev, ray_d_dev, ray_mesh_dev, rays_per_mesh,
               n_rays, nullptr, nullptr, nullptr, nullptr, s};
    kdgb_tree *tree = nullptr;
    int rc = n_meshes > 1 ? kdgb_build_batch(tri_v_dev, mesh_offsets, n_meshes, &bp, &tree, stream)
                          : kdgb_build(tri_v_dev, n_tris, &bp, &tree, stream);
    if (rc != KDGB_OK) return rc;
    // Trial builds may use at most a few more levels than the caller's tree
    // needed, so a leaf threshold whose tree keeps duplicating references
    // fails fast instead of filling the device.
    kdgb_build_stats st0;
    kdgb_tree_stats(tree, &st0);
    const int32_t trial_levels = std::min(bp.max_levels, st0.upper_levels + 4);

    void *scratch = nullptr;
    if (n_rays > 0) {
        const cudaError_t e = cudaMallocAsync(&scratch, (size_t)n_rays * 16, s);
        if (e != cudaSuccess) {
            kdgb_tree_destroy(tree);
            return cuda_fail(e, "autotune scratch");
        }
        w.hit = (int32_t *)scratch;
        w.t = (float *)scratch + n_rays;
        w.u = (float *)scratch + 2 * (int64_t)n_rays;
        w.v = (float *)scratch + 3 * (int64_t)n_rays;
    }
    cudaEvent_t e0 = nullptr, e1 = nullptr, e2 = nullptr;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventCreate(&e2);

    auto objective = [&](const Score &sc) { return builds_per_trace * sc.build_ms + sc.trace_ms; };
    kdgb_build_params best_b = bp;
    kdgb_trace_params best_t = tp;
    Score best = measure(tree, w, best_b, best_t, true, reps, e0, e1, e2);
    int trials = 1;
    rc = best.ok ? KDGB_OK : KDGB_ERR_CUDA;
    const float baseline = objective(best);

    auto try_build = [&](kdgb_build_params cand) {
        cand.max_levels = trial_levels;
        ++trials;
        const Score sc = measure(tree, w, cand, best_t, true, reps, e0, e1, e2);
        if (sc.ok && objective(sc) < objective(best)) {
            best = sc;
            cand.max_levels = bp.max_levels;
            best_b = cand;
        }
    };
    auto try_trace = [&](const kdgb_trace_params &cand) {
        ++trials;
        Score sc = measure(tree, w, best_b, cand, false, reps, e0, e1, e2);
        sc.build_ms = best.build_ms;
        if (sc.ok && objective(sc) < objective(best)) {
            best = sc;
            best_t = cand;
        }
    };
    if (rc == KDGB_OK) {
        for (int ls : {16, 24, 32}) {
            if (ls == best_b.leaf_size) continue;
            kdgb_build_params c = best_b;
            c.leaf_size = ls;
            try_build(c);
        }
        if (best_b.mode == KDGB_BUILD_TUNED) {
            for (int b : {8, 16, 32}) {
                if (b == best_b.sah_bins) continue;
                kdgb_build_params c = best_b;
                c.sah_bins = b;
                try_build(c);
            }
        }
        // The trace candidates run on the best tree.
        if (rebuild(tree, w, best_b) != KDGB_OK) rc = KDGB_ERR_CUDA;
    }
    if (rc == KDGB_OK && n_rays > 0) {
        if (best_t.tracer == KDGB_TRACER_SHORTSTACK) {
            for (int dpt : {2, 4, 8}) {
                if (dpt == best_t.stack_depth) continue;
                kdgb_trace_params c = best_t;
                c.stack_depth = dpt;
                try_trace(c);
            }
        }
        for (int bs : {64, 128, 256}) {
            if (bs == (best_t.block_size > 0 ? best_t.block_size : 128)) continue;
            kdgb_trace_params c = best_t;
            c.block_size = bs;
            try_trace(c);
        }
        // The schedule: one thread per ray, or the persistent queue that
        // hands out the largest meshes' rays first.
        {
            kdgb_trace_params c = best_t;
            c.schedule = best_t.schedule == KDGB_SCHEDULE_QUEUE ? KDGB_SCHEDULE_GRID : KDGB_SCHEDULE_QUEUE;
            try_trace(c);
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaEventDestroy(e2);
    if (scratch) cudaFreeAsync(scratch, s);
    kdgb_tree_destroy(tree);
    if (rc != KDGB_OK) return fail(rc, "kdgb_autotune: the starting parameters failed");
    out->build = best_b;
    out->trace = best_t;
    out->build_ms = best.build_ms;
    out->trace_ms = best.trace_ms;
    out->baseline = baseline;
    out->objective = objective(best);
    out->trials = trials;
    set_error("");
    return KDGB_OK;
}

}  // extern "C"
