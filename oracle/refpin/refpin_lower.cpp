// The reference's lower creators run on the host: its own kernels
// (Utils/CUDA/Kernels/LowerTriangleMap.h, compiled unmodified) executed one
// thread at a time, driven level by level as TriangleMapSAHCreator.cu:67-260
// and TriangleMapBalancedCreator.cu:60-248 drive them (their CUDPP scans are
// plain prefix sums here).  CreateSplittingPlanes reads the other threads'
// shared-memory boxes without a barrier (warp-synchronous); each of its
// blocks therefore runs twice, the first pass filling shared memory.  TEST
// INFRASTRUCTURE ONLY: built into oracle/_ref/, never part of the library.
#include <Meta/CUDA.h>
#include <Utils/CUDA/SharedMemory.h>
#include <Utils/CUDA/Utils.h>
#include <Utils/CUDA/Convert.h>
#include <Utils/CUDA/IntersectionTests.h>
#include <Scene/TriangleNode.h>
#include <Utils/CUDA/Kernels/DeviceVars.h>

#include <vector>

uint3 threadIdx, blockIdx;
dim3 blockDim, gridDim;

namespace OpenEngine {
namespace Utils {
namespace CUDA {
using namespace Kernels;
using namespace Scene;
namespace PinLower {
#include <Utils/CUDA/Kernels/LowerTriangleMap.h>
}  // namespace PinLower
}  // namespace CUDA
}  // namespace Utils
}  // namespace OpenEngine

using namespace OpenEngine::Utils::CUDA;
using namespace OpenEngine::Utils::CUDA::PinLower;
using OpenEngine::Scene::KDNode;

template <class Body>
static void launch(int n_threads, int block, Body body, int passes = 1)
{
    const int blocks = (n_threads + block - 1) / block;
    blockDim = {(unsigned)block, 1, 1};
    gridDim = {(unsigned)(blocks > 0 ? blocks : 1), 1, 1};
    for (int b = 0; b < blocks; ++b) {
        blockIdx = {(unsigned)b, 0, 0};
        for (int p = 0; p < passes; ++p)
            for (int t = 0; t < block; ++t) {
                threadIdx = {(unsigned)t, 0, 0};
                body();
            }
    }
}

static void exclusive_scan(const std::vector<int> &in, std::vector<int> &out, int n)
{
    out.assign(n + 1, 0);
    for (int i = 0; i < n; ++i) out[i + 1] = out[i] + in[i];
}

extern "C" {

// Runs the SAH (creator 1) or balanced (creator 2) lower creator over the
// upper leaves of a tree whose upper phase is done.  Node arrays have room
// for max_nodes; on entry they hold n_nodes nodes (upper leaves with their
// reference counts in `bitmap`).  Returns the node count, or -1 when
// max_nodes is too small.
int ref_lower(int creator, int propagate, float traversal_cost, const float *tri, int T, int n_nodes, int max_nodes,
              signed char *info, float *split, float *aabb_min, float *aabb_max, int *prim_index, int *bitmap,
              int *children, float *area, const int *prim_indices, const float *prim_min, const float *prim_max,
              int n_refs, const int *leaf_ids, int n_leaves, int *levels)
{
    std::vector<float4> p0(T), p1(T), p2(T);
    for (int i = 0; i < T; ++i) {
        p0[i] = make_float4(tri[9 * i], tri[9 * i + 1], tri[9 * i + 2], 1.0f);
        p1[i] = make_float4(tri[9 * i + 3], tri[9 * i + 4], tri[9 * i + 5], 1.0f);
        p2[i] = make_float4(tri[9 * i + 6], tri[9 * i + 7], tri[9 * i + 8], 1.0f);
    }
    char *ninfo = reinterpret_cast<char *>(info);
    float4 *nmin = reinterpret_cast<float4 *>(aabb_min), *nmax = reinterpret_cast<float4 *>(aabb_max);
    int2 *nch = reinterpret_cast<int2 *>(children);
    std::vector<int> idx(prim_indices, prim_indices + n_refs), ids(leaf_ids, leaf_ids + n_leaves);
    std::vector<float4> pmin(reinterpret_cast<const float4 *>(prim_min), reinterpret_cast<const float4 *>(prim_min) + n_refs);
    std::vector<float4> pmax(reinterpret_cast<const float4 *>(prim_max), reinterpret_cast<const float4 *>(prim_max) + n_refs);
    std::vector<float> areas(n_refs > 0 ? n_refs : 1);
    std::vector<int4> sets(3 * (size_t)(n_refs > 0 ? n_refs : 1));
    d_triangles = n_refs;

    // Preprocessing (PreprocessLowerNodes of each creator).
    int range = n_leaves;
    if (creator == 1) {
        launch(n_refs, 128, [&] { CalcSurfaceArea(idx.data(), p0.data(), p1.data(), p2.data(), areas.data(), n_refs); });
        launch(range, 128, [&] { PreprocesLowerNodes(ids.data(), prim_index, bitmap, area, areas.data(), range); });
    } else {
        launch(range, 128, [&] { PreprocessLeafNodes(ids.data(), bitmap, range); });
    }
    launch(range * KDNode::MAX_LOWER_SIZE, 128,
           [&] { CreateSplittingPlanes(ids.data(), prim_index, bitmap, pmin.data(), pmax.data(), sets.data(), range); },
           2);

    // The level loop (ProcessLowerNodes).
    int active = n_nodes, lv = 0;
    bool first = true;
    while (range > 0) {
        ++lv;
        d_activeNodeIndex = active;
        d_activeNodeRange = range;
        std::vector<float2> careas(range);
        std::vector<int2> csets(range);
        std::vector<int> side(range + 1, 0), addr;
        const int block = creator == 1 ? 96 : 128;
        if (creator == 1) {
            if (first)
                launch(range, block, [&] {
                    CalcSAH<true>(ids.data(), ninfo, split, prim_index, bitmap, area, areas.data(), pmin.data(),
                                  pmax.data(), sets.data(), careas.data(), csets.data(), side.data(), traversal_cost);
                });
            else
                launch(range, block, [&] {
                    CalcSAH<false>(nullptr, ninfo, split, prim_index, bitmap, area, areas.data(), pmin.data(),
                                   pmax.data(), sets.data(), careas.data(), csets.data(), side.data(), traversal_cost);
                });
        } else {
            if (first)
                launch(range, block, [&] {
                    CalcSplit<true>(ids.data(), ninfo, split, prim_index, bitmap, pmin.data(), pmax.data(),
                                    sets.data(), csets.data(), side.data(), traversal_cost);
                });
            else
                launch(range, block, [&] {
                    CalcSplit<false>(nullptr, ninfo, split, prim_index, bitmap, pmin.data(), pmax.data(),
                                     sets.data(), csets.data(), side.data(), traversal_cost);
                });
        }
        exclusive_scan(side, addr, range);
        const int splits = addr[range];
        if (n_nodes + 2 * splits > max_nodes) return -1;
        n_nodes += 2 * splits;
        if (creator == 1) {
            if (first)
                launch(range, 128, [&] {
                    CreateLowerSAHChildren<true>(ids.data(), side.data(), addr.data(), careas.data(), csets.data(),
                                                 area, prim_index, bitmap, nch, splits);
                });
            else
                launch(range, 128, [&] {
                    CreateLowerSAHChildren<false>(nullptr, side.data(), addr.data(), careas.data(), csets.data(),
                                                  area, prim_index, bitmap, nch, splits);
                });
        } else {
            if (first)
                launch(range, 128, [&] {
                    CreateChildren<true>(ids.data(), side.data(), addr.data(), csets.data(), prim_index, bitmap, nch,
                                         splits);
                });
            else
                launch(range, 128, [&] {
                    CreateChildren<false>(nullptr, side.data(), addr.data(), csets.data(), prim_index, bitmap, nch,
                                          splits);
                });
        }
        const int created = 2 * splits;
        if (propagate && created > 0) {
            if (first)
                launch(range, 128, [&] { PropagateAabbToChildren<true>(ids.data(), ninfo, split, nmin, nmax, nch); });
            else
                launch(range, 128, [&] { PropagateAabbToChildren<false>(nullptr, ninfo, split, nmin, nmax, nch); });
        }
        first = false;
        active = n_nodes - created;
        range = created;
    }
    *levels = lv;
    return n_nodes;
}

}  // extern "C"
