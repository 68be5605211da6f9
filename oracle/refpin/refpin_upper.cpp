// The reference's upper creator run on the host: its own kernels
// (Utils/CUDA/Kernels/TriangleUpper.h, TriangleUpperSegment.h,
// TriangleUpperChildren.h, EmptySpaceSplitting.h, ReduceSegments.h, compiled
// unmodified) executed one thread at a time, driven level by level as
// TriangleMapUpperCreator.cu:100-700 drives them (Create, ProcessNodes,
// Segment, ReduceAabb, CreateEmptySplits, CreateChildren).  Its CUDPP scans
// are plain prefix sums here.  TEST INFRASTRUCTURE ONLY: built into
// oracle/_ref/, never part of the library.
//
// Two kernels are not replayed thread by thread: ReduceSegmentsUnrolled
// (warp-synchronous) and FinalSegmentedReduce (barrier rounds across the
// block).  What they compute is the per-segment and then per-node minimum
// and maximum of the reference boxes, padded with +-fInfinity; min and max
// are exact and order-free, so the driver computes those values directly.
// ReduceSegmentsUnrolled leaves the w of its segment boxes unset, which makes
// the w of the reduced node boxes undefined in the reference; here they come
// out as 0 and callers compare x, y, z only.
//
// Node and reference arrays the reference allocates without initialising
// (CUDADataBlock Extend / Resize) are zero-filled here.  The unit is a library
// of its own, built with hidden visibility: DeviceVars.h defines the device
// variables it shares with the lower kernels as plain globals here.
#include <Meta/CUDA.h>
#include <Utils/CUDA/SharedMemory.h>
#include <Utils/CUDA/Utils.h>
#include <Utils/CUDA/Convert.h>
#include <Utils/CUDA/IntersectionTests.h>
#include <Utils/CUDA/Segments.h>
#include <Scene/TriangleNode.h>
#include <Utils/CUDA/Kernels/DeviceVars.h>

#include <algorithm>
#include <vector>

namespace OpenEngine {
namespace Utils {
namespace CUDA {
using namespace Kernels;
using namespace Scene;
namespace PinUpper {
#include <Utils/CUDA/Kernels/TriangleUpper.h>
#include <Utils/CUDA/Kernels/TriangleUpperSegment.h>
#include <Utils/CUDA/Kernels/ReduceSegments.h>
#include <Utils/CUDA/Kernels/TriangleUpperChildren.h>
#include <Utils/CUDA/Kernels/TriangleKernels.h>
#include <Utils/CUDA/Kernels/EmptySpaceSplitting.h>
}  // namespace PinUpper
}  // namespace CUDA
}  // namespace Utils
}  // namespace OpenEngine

using namespace OpenEngine::Utils::CUDA;
using namespace OpenEngine::Utils::CUDA::PinUpper;
using OpenEngine::Scene::KDNode;
using OpenEngine::Scene::TriangleNode;

namespace {

// A grid of `blocks` x `threads`, every thread run to completion in turn.
template <class Body>
void launch_grid(unsigned blocks, unsigned threads, Body body)
{
    blockDim = {threads, 1, 1};
    gridDim = {blocks, 1, 1};
    for (unsigned b = 0; b < blocks; ++b) {
        blockIdx = {b, 0, 0};
        for (unsigned t = 0; t < threads; ++t) {
            threadIdx = {t, 0, 0};
            body();
        }
    }
}

// The grid Calc1DKernelDimensions (Utils/CUDA/Utils.h:127-142) picks.
template <class Body>
void launch_1d(int size, Body body, unsigned max_threads = 0)
{
    unsigned blocks = 0, threads = 0;
    Calc1DKernelDimensions(size, blocks, threads, max_threads);
    launch_grid(blocks, threads, body);
}

// The grid KernelConf1D (Utils/CUDA/Utils.h:101-125) picks.
template <class Body>
void launch_conf(int size, Body body)
{
    const KernelConf conf = KernelConf1D(size);
    launch_grid(conf.blocks, conf.threads, body);
}

void exclusive_scan(const int *in, int *out, int n)
{
    int acc = 0;
    for (int i = 0; i < n; ++i) {
        const int v = in[i];
        out[i] = acc;
        acc += v;
    }
}

template <class T>
void grow(std::vector<T> &v, size_t n)
{
    v.resize(n, T());
}

struct Upper {
    // TriangleNode SoA (KDNode.h:64-74, TriangleNode.h:20-21).
    std::vector<char> info;
    std::vector<float> split;
    std::vector<float4> nmin, nmax;
    std::vector<int> pidx, amount, parent;
    std::vector<int2> children;
    // TriangleMap's upper-leaf references and leaf list (TriangleMap.h:52-57).
    std::vector<float4> prim_min, prim_max;
    std::vector<int> leaf_ids;
    // The creator's working arrays (TriangleMapUpperCreator.h:41-66).
    std::vector<float4> aabb_min, aabb_max, temp_min, temp_max;
    std::vector<int> node_segments, owner, split_side, split_addr, leaf_side, leaf_addr, es_nodes, es_addrs;
    std::vector<int2> seg_info, child_size;
    std::vector<float4> seg_min, seg_max;
    std::vector<char> es_planes;
    std::vector<float4> p0, p1, p2;
    int split_method = 0;
    bool ess = true, propagate = true;

    int size() const { return (int)info.size(); }
    void resize_nodes(int n)
    {
        grow(info, n); grow(split, n); grow(nmin, n); grow(nmax, n);
        grow(pidx, n); grow(amount, n); grow(parent, n); grow(children, n);
    }

    // Segment (TriangleMapUpperCreator.cu:154-190).
    void segment(int active_index, int active_range)
    {
        grow(node_segments, active_range + 1);
        launch_1d(active_range, [&] { NodeSegments(amount.data() + active_index, node_segments.data()); });
        exclusive_scan(node_segments.data(), node_segments.data(), active_range + 1);
        const int segments = node_segments[active_range];
        d_segments = segments;
        owner.assign(segments, 0);
        launch_1d(active_range, [&] { MarkOwnerStart(owner.data(), node_segments.data()); });
        for (int i = 1; i < segments; ++i) owner[i] += owner[i - 1];  // inclusive scan
        grow(seg_info, segments);
        launch_1d(segments, [&] {
            CalcSegmentPrimitives(owner.data(), node_segments.data(), pidx.data(), amount.data(), seg_info.data());
        });
    }

    // ReduceAabb (TriangleMapUpperCreator.cu:192-258).
    void reduce_aabb(int active_index, int active_range)
    {
        const int segments = (int)owner.size();
        const float inf = fInfinity;
        // ReduceSegmentsUnrolled: each segment's box, padded with +-fInfinity.
        seg_min.assign(segments, make_float4(0.0f));
        seg_max.assign(segments, make_float4(0.0f));
        for (int s = 0; s < segments; ++s) {
            float3 lo = make_float3(inf), hi = make_float3(-1.0f * inf);
            for (int k = 0; k < seg_info[s].y; ++k) {
                lo = min(lo, make_float3(aabb_min[seg_info[s].x + k]));
                hi = max(hi, make_float3(aabb_max[seg_info[s].x + k]));
            }
            seg_min[s] = make_float4(lo, 0.0f);
            seg_max[s] = make_float4(hi, 0.0f);
        }
        if (ess) {
            temp_min.assign(nmin.begin() + active_index, nmin.begin() + active_index + active_range);
            temp_max.assign(nmax.begin() + active_index, nmax.begin() + active_index + active_range);
        }
        launch_1d(active_range, [&] { AabbMemset(nmin.data() + active_index, nmax.data() + active_index); });
        // FinalSegmentedReduce: each node's box from its segments.
        for (int s = 0; s < segments; ++s) {
            const int n = owner[s];
            nmin[n] = make_float4(min(make_float3(nmin[n]), make_float3(seg_min[s])), 0.0f);
            nmax[n] = make_float4(max(make_float3(nmax[n]), make_float3(seg_max[s])), 0.0f);
        }
        d_segments = segments;
        if (ess && active_index != 0) create_empty_splits(active_index, active_range);
        launch_1d(active_range, [&] {
            CalcUpperNodeSplitInfo(nmin.data() + active_index, nmax.data() + active_index, split.data() + active_index,
                                   info.data() + active_index);
        });
    }

    // CreateEmptySplits (TriangleMapUpperCreator.cu:260-320).
    void create_empty_splits(int active_index, int active_range)
    {
        d_createdEmptySplits = false;
        grow(es_planes, active_range);
        grow(es_nodes, active_range + 1);
        launch_conf(active_range, [&] {
            CalcEmptySpaceSplits(temp_min.data(), temp_max.data(), nmin.data() + active_index,
                                 nmax.data() + active_index, es_planes.data(), es_nodes.data());
        });
        if (!d_createdEmptySplits) return;
        grow(es_addrs, active_range + 1);
        exclusive_scan(es_nodes.data(), es_addrs.data(), active_range + 1);
        const int empty_nodes = es_addrs[active_range];
        resize_nodes(size() + empty_nodes);
        launch_conf(active_range, [&] {
            EmptySpaceSplitting2(info.data(), split.data(), amount.data(), parent.data(), children.data(),
                                 es_planes.data(), es_addrs.data(), nmin.data() + active_index,
                                 nmax.data() + active_index, empty_nodes);
        });
    }

    // CreateChildren (TriangleMapUpperCreator.cu:440-700).
    int create_children(int active_index, int active_range)
    {
        const int triangles = (int)aabb_min.size();
        const unsigned blocks = (unsigned)owner.size(), threads = Segments::SEGMENT_SIZE;
        grow(split_side, 2 * triangles + 1);
        grow(split_addr, 2 * triangles + 1);
        grow(leaf_side, 2 * triangles + 1);
        grow(leaf_addr, 2 * triangles + 1);
        grow(child_size, active_range);
        const int child_start = size();
        resize_nodes(size() + 2 * active_range);
        if (split_method == 0)
            launch_grid(blocks, threads, [&] {
                SetSplitSide(seg_info.data(), owner.data(), info.data(), split.data(), aabb_min.data(),
                             aabb_max.data(), split_side.data());
            });
        else
            launch_grid(blocks, threads, [&] {
                SetDivideSide<false>(seg_info.data(), owner.data(), info.data(), split.data(), aabb_min.data(),
                                     aabb_max.data(), nmin.data(), nmax.data(), p0.data(), p1.data(), p2.data(),
                                     split_side.data());
            });
        exclusive_scan(split_side.data(), split_addr.data(), 2 * triangles + 1);
        int new_triangles = split_addr[2 * triangles];
        d_createdLeafs = false;
        launch_1d(active_range, [&] {
            CalcNodeChildSize(pidx.data() + active_index, amount.data() + active_index, split_addr.data(),
                              child_size.data());
        });
        int created;
        if (d_createdLeafs) {
            launch_grid(blocks, threads, [&] {
                SetPrimitiveLeafSide(seg_info.data(), owner.data(), child_size.data(), split_side.data(),
                                     leaf_side.data());
            });
            exclusive_scan(leaf_side.data(), leaf_addr.data(), 2 * triangles + 1);
            const int leaf_triangles = leaf_addr[2 * triangles];
            new_triangles -= leaf_triangles;
            temp_min.assign(new_triangles, make_float4(0.0f));
            temp_max.assign(new_triangles, make_float4(0.0f));
            const int upper_leaf_prims = (int)prim_min.size();
            grow(prim_min, upper_leaf_prims + leaf_triangles);
            grow(prim_max, upper_leaf_prims + leaf_triangles);
            launch_grid(blocks, threads, [&] {
                SplitTriangles(seg_info.data(), owner.data(), info.data(), split.data(), split_side.data(),
                               split_addr.data(), leaf_side.data(), leaf_addr.data(), aabb_min.data(), aabb_max.data(),
                               temp_min.data(), temp_max.data(), prim_min.data() + upper_leaf_prims,
                               prim_max.data() + upper_leaf_prims);
            });
            std::swap(aabb_min, temp_min);
            std::swap(aabb_max, temp_max);
            launch_1d(active_range, [&] { MarkNodeLeafs(child_size.data(), leaf_side.data()); });
            // The node-leaf marks are scanned into split_side (its reuse in
            // the reference).
            exclusive_scan(leaf_side.data(), split_side.data(), 2 * active_range + 1);
            const int leaf_nodes = split_side[2 * active_range];
            d_leafNodes = leaf_nodes;
            launch_1d(active_range, [&] {
                CreateUpperChildren<false>(nullptr, pidx.data(), amount.data(), child_size.data(), split_addr.data(),
                                           leaf_addr.data(), split_side.data(), children.data(), parent.data(),
                                           upper_leaf_prims, child_start);
            });
            created = 2 * active_range - leaf_nodes;
            const int first_leaf = (int)leaf_ids.size();
            grow(leaf_ids, first_leaf + leaf_nodes);
            const int leaf_index = size() - 2 * active_range;
            launch_1d(leaf_nodes, [&] {
                MarkLeafNodes(leaf_ids.data() + first_leaf, info.data() + leaf_index, leaf_index, leaf_nodes);
            });
        } else {
            temp_min.assign(new_triangles, make_float4(0.0f));
            temp_max.assign(new_triangles, make_float4(0.0f));
            launch_1d(active_range, [&] {
                CreateUpperChildren<false>(nullptr, pidx.data(), amount.data(), child_size.data(), split_addr.data(),
                                           children.data(), parent.data(), child_start);
            });
            launch_grid(blocks, threads, [&] {
                SplitTriangles(seg_info.data(), owner.data(), info.data(), split.data(), split_side.data(),
                               split_addr.data(), aabb_min.data(), aabb_max.data(), temp_min.data(), temp_max.data());
            });
            std::swap(aabb_min, temp_min);
            std::swap(aabb_max, temp_max);
            created = 2 * active_range;
        }
        if (ess)
            launch_1d(active_range, [&] {
                PropagateAabbToChildren<false>(nullptr, info.data(), split.data(), nmin.data(), nmax.data(),
                                               children.data());
            });
        return created;
    }
};

}  // namespace

uint3 threadIdx, blockIdx;
dim3 blockDim, gridDim;

extern "C" {

// TriangleMapUpperCreator::Create (TriangleMapUpperCreator.cu:100-152) over T
// triangles (tri: T*9 floats).  split_method: 0 BOX, 1 DIVIDE.  Outputs have
// room for max_nodes nodes, max_refs upper-leaf references and max_leaves
// upper leaves; node arrays come back with the upper leaves' reference counts
// in `amount`.  Returns the node count, or -1 when a capacity is too small.
__attribute__((visibility("default"))) int ref_upper(int split_method, int empty_space, int propagate, float threshold, const float *tri, int T,
              int max_nodes, int max_refs, int max_leaves, signed char *info, float *split, float *aabb_min,
              float *aabb_max, int *prim_index, int *amount, int *children, int *parent, float *prim_min,
              float *prim_max, int *prim_indices, int *n_refs, int *leaf_ids, int *n_leaves, int *levels)
{
    Upper u;
    u.split_method = split_method;
    u.ess = empty_space != 0;
    u.propagate = propagate != 0;
    u.p0.resize(T); u.p1.resize(T); u.p2.resize(T);
    for (int i = 0; i < T; ++i) {
        u.p0[i] = make_float4(tri[9 * i], tri[9 * i + 1], tri[9 * i + 2], 1.0f);
        u.p1[i] = make_float4(tri[9 * i + 3], tri[9 * i + 4], tri[9 * i + 5], 1.0f);
        u.p2[i] = make_float4(tri[9 * i + 6], tri[9 * i + 7], tri[9 * i + 8], 1.0f);
    }
    d_emptySpaceThreshold = threshold;
    u.resize_nodes(1);
    u.pidx[0] = 0;
    u.amount[0] = T;
    u.parent[0] = 0;
    u.aabb_min.resize(T);
    u.aabb_max.resize(T);
    launch_1d(T, [&] {
        CalcPrimitiveAabb(u.p0.data(), u.p1.data(), u.p2.data(), u.aabb_min.data(), u.aabb_max.data(), T);
    });
    int active_index = 0, active_range = 1, lv = 0;
    while (active_range > 0) {
        // ProcessNodes (TriangleMapUpperCreator.cu:138-152).
        d_activeNodeIndex = active_index;
        d_activeNodeRange = active_range;
        d_triangles = (int)u.aabb_min.size();
        u.segment(active_index, active_range);
        u.reduce_aabb(active_index, active_range);
        const int created = u.create_children(active_index, active_range);
        active_index = u.size() - created;
        active_range = created;
        ++lv;
        if (u.size() > max_nodes) return -1;
    }
    const int refs = (int)u.prim_min.size(), leaves = (int)u.leaf_ids.size();
    if (refs > max_refs || leaves > max_leaves) return -1;
    std::vector<int> idx(refs);
    launch_1d(refs, [&] { ExtractIndexFromAabb(u.prim_min.data(), idx.data(), refs); }, 128);
    if (!u.ess && u.propagate) {
        const KernelConf conf = KernelConf1D(leaves, 128);
        launch_grid(conf.blocks, conf.threads, [&] {
            PropagateParentAabb<true>(u.leaf_ids.data(), u.info.data(), u.split.data(), u.nmin.data(), u.nmax.data(),
                                      u.parent.data(), u.children.data(), leaves);
        });
    }
    const int n = u.size();
    for (int i = 0; i < n; ++i) {
        info[i] = (signed char)u.info[i];
        split[i] = u.split[i];
        memcpy(aabb_min + 4 * i, &u.nmin[i], sizeof(float4));
        memcpy(aabb_max + 4 * i, &u.nmax[i], sizeof(float4));
        prim_index[i] = u.pidx[i];
        amount[i] = u.amount[i];
        children[2 * i] = u.children[i].x;
        children[2 * i + 1] = u.children[i].y;
        parent[i] = u.parent[i];
    }
    if (refs) {
        memcpy(prim_min, u.prim_min.data(), refs * sizeof(float4));
        memcpy(prim_max, u.prim_max.data(), refs * sizeof(float4));
        memcpy(prim_indices, idx.data(), refs * sizeof(int));
    }
    if (leaves) memcpy(leaf_ids, u.leaf_ids.data(), leaves * sizeof(int));
    *n_refs = refs;
    *n_leaves = leaves;
    *levels = lv;
    return n;
}

}  // extern "C"
