// Internal declarations shared by the kdgb CUDA translation units.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

#include "kdgb.h"

namespace kdgb {

// ---------------------------------------------------------------------------
// Status handling: no exception crosses the C ABI.
// ---------------------------------------------------------------------------
void set_error(const std::string &msg);
int fail(int status, const std::string &msg);
int cuda_fail(cudaError_t e, const char *what);

// SMs of the context current on this thread (a green context's share of the
// device for a stream of an SM partition), or 0 when the driver cannot say.
int context_sm_count();

// Makes the context of stream s current for the lifetime of the object when
// another one is current (a stream of an SM partition), so that the streams
// created and the work captured meanwhile belong to that context.
struct StreamContext {
    explicit StreamContext(cudaStream_t s);
    ~StreamContext();
    StreamContext(const StreamContext &) = delete;
    StreamContext &operator=(const StreamContext &) = delete;

private:
    bool pushed_ = false;
};

#define KDGB_CUDA(call)                                        \
    do {                                                       \
        cudaError_t e_ = (call);                               \
        if (e_ != cudaSuccess) return ::kdgb::cuda_fail(e_, #call); \
    } while (0)

#define KDGB_CHECK(call)                 \
    do {                                 \
        int s_ = (call);                 \
        if (s_ != KDGB_OK) return s_;    \
    } while (0)

// Counts kernel launches made by the library (instrumentation only).
void note_launch(int n = 1);

#define KDGB_LAUNCH_CHECK()              \
    do {                                 \
        ::kdgb::note_launch();           \
        KDGB_CUDA(cudaGetLastError());   \
    } while (0)

// kernel<<<grid, block, smem, stream>>>(args...) followed by
// KDGB_LAUNCH_CHECK(); the kernel may be a template-id in parentheses.
#define KDGB_KERNEL(kernel, grid, block, smem, stream, ...)     \
    do {                                                        \
        kernel<<<(grid), (block), (smem), (stream)>>>(__VA_ARGS__); \
        KDGB_LAUNCH_CHECK();                                    \
    } while (0)

// ---------------------------------------------------------------------------
// Device arrays owned by a tree handle.  `cap` counts elements.
// ---------------------------------------------------------------------------
template <class T>
struct DevArray {
    T *p = nullptr;
    int64_t cap = 0;
};

// Grows `a` to hold at least n elements (stream-ordered allocation).  When
// `keep` elements are live they are copied into the new block.  Newly
// allocated storage is zero-filled when `zero` is set.
template <class T>
int ensure(DevArray<T> &a, int64_t n, cudaStream_t s, int64_t keep = 0, bool zero = false);

template <class T>
void release(DevArray<T> &a, cudaStream_t s);

// Scratch storage: grows geometrically (x1.5) and never keeps contents.
template <class T>
int grab(DevArray<T> &a, int64_t n, cudaStream_t s)
{
    if (a.p && n <= a.cap) return KDGB_OK;
    const int64_t want = a.cap + a.cap / 2 > n ? a.cap + a.cap / 2 : n;
    return ensure(a, want, s, 0, false);
}

// Device-resident counters of a build in progress.  Every build kernel reads
// its sizes here, so one launch sequence runs either under host control
// (exact grids, one readback per level) or captured once into a CUDA graph
// whose level loops are conditional WHILE nodes.  Only one thread of the
// block that finishes a level last writes it (advance_upper/advance_lower).
struct BuildState {
    int64_t N;            // references of the current upper level
    int64_t F;            // leaf references written so far
    int32_t R;            // active nodes of the current upper level
    int32_t active;       // id of the first active node
    int32_t n_nodes;      // nodes written so far
    int32_t level;        // upper levels completed
    int32_t ntiles;       // block tiles (kTileRefs references) covering the N references
    int32_t n_leaf_ids;   // upper leaves so far
    int32_t n_ranges;     // upper levels that produced leaves
    int32_t err;          // first failure (a kdgb_status), 0 while healthy
    int32_t err_detail;   // which check failed (see kdgb_build.cu)
    int32_t nonfinite;    // set when a vertex coordinate is NaN or Inf
    int32_t low_R;        // active nodes of the current SAH lower level
    int32_t low_active;   // first of them when low_first == 0
    int32_t low_levels;   // SAH lower levels completed
    int32_t low_first;    // 1 while the lower level is the upper leaves
    int32_t n_leaf_tris;  // leaf records of the traversal layout
    int32_t n_big;        // tuned levels: chunks of large active nodes listed for block-wide SAH binning
    int32_t done;         // blocks of the current level-closing kernel that have finished
    // SAH lower levels: nodes to evaluate, listed by the level before (by
    // level parity): [0] nodes of at most 16 members, [1] larger ones.
    int32_t low_n[2][2];
};

// Sizes seen by the last host-driven build of a handle; a graph rebuild
// sizes its fixed buffers from them.
struct BuildPlan {
    bool valid = false;
    int64_t max_N = 0, F = 0, nodes = 0, max_R = 0, leaves = 0, max_low_R = 0, leaf_tris = 0;
    int32_t levels = 0, low_levels = 0;
};

// Kernels a captured build records: outside the loops and per loop body.
struct GraphKernels {
    int64_t fixed = 0, upper_body = 0, lower_body = 0;
};

// Per-handle build workspace, reused by every level and every rebuild so the
// steady state issues no device allocations.  References ping-pong between
// rmin/rmax[0] and [1] by level parity.
struct Workspace {
    DevArray<float4> rmin[2], rmax[2], fmin, fmax;
    DevArray<unsigned> keys;
    DevArray<int8_t> planes[2];  // empty-space planes of a level, by level parity
    DevArray<int32_t> ess[2];    // empty-space node counts of a level, by level parity
    DevArray<int32_t> cnt, lbase, chunksum, tilesum, tileoff, stats, scan, misc0, misc1, big;
    DevArray<int32_t> bighist;  // per-node SAH histograms of chunked large nodes, zero between uses
    DevArray<float> areas;
    DevArray<int4> sts;
    DevArray<int32_t> ssplit, roff;
    DevArray<int32_t> lcnt[2];  // SAH lower levels: split nodes per tile of nodes, by level parity
    DevArray<int32_t> lowlist[2];  // SAH lower work lists, by level parity (small nodes first, large from the end)
    DevArray<float2> careas;
    DevArray<int2> csets, ranges;
    DevArray<BuildState> state;
    int32_t *host = nullptr;  // pinned record buffer (kHostRec ints)
};
constexpr int kHostRec = 256;

struct Tree {
    int32_t n_tris = 0;
    int32_t n_nodes = 0;
    int32_t n_refs = 0;
    int32_t n_upper_leaves = 0;
    int32_t n_leaf_tris = 0;     // rows of the leaf-ordered triangle records
    int32_t n_meshes = 1;        // forest roots (kdgb_build_batch)
    kdgb_build_stats stats{};
    DevArray<int32_t> mesh_off;  // n_meshes + 1 triangle offsets (batches only)
    DevArray<int32_t> mesh_order;  // batch meshes by triangle count, largest first (queue traces)
    DevArray<unsigned> qctr;       // queue trace state: next chunk, warps done (zero between launches)

    // Geometry (GeometryList SoA) and the packed triangle array used by builds.
    DevArray<float4> p0, p1, p2;
    // The same triangles packed as the traversal layout's 48-byte records,
    // {v0.xyz, e1.x} {e1.yz, e2.xy} {e2.z, id bits, 0, 0}, 3 float4 per
    // triangle: the leaf records are copies of these (one contiguous
    // gather), and the SAH areas read e1 and e2 from them.
    DevArray<float4> prec;

    // TriangleNode SoA (KDNode.h:65-73, TriangleNode.h:20-21).
    DevArray<int8_t> info;
    DevArray<float> split;
    DevArray<float4> bmin, bmax;
    DevArray<int32_t> pidx, bitmap, parent;
    DevArray<int2> children;
    DevArray<float> area;
    DevArray<int32_t> prim_indices, leaf_ids;

    // Traversal layout: one 8-byte record per node, in an order where the
    // two children of a node are adjacent, the leaf boxes in that order (for
    // leaf skipping), and leaf-ordered triangle records (v0, e1, e2, id) of
    // 48 bytes.
    DevArray<int2> tnode;
    DevArray<float4> tbox;  // leaf boxes: min, max of node j at [2j], [2j + 1]
    DevArray<float4> ttri;

    // Woop transform rows (m0, m1, m2) per triangle, computed on the first
    // Woop trace after a build (a cache: traces of a const handle fill it).
    mutable DevArray<float4> woop;
    mutable bool woop_valid = false;

    Workspace ws;
    BuildPlan plan;
};

// Makes t.woop current (kdgb_trace.cu).
int woop_values(const Tree &t, cudaStream_t s);

// Lower creators that split the upper leaves level by level over bitmap
// sets (SAH and balanced); BITMAP only converts the leaves.
inline bool lower_loop(const kdgb_build_params &p)
{
    return p.lower == KDGB_LOWER_SAH || p.lower == KDGB_LOWER_BALANCED;
}

// Builder (kdgb_build.cu), both modes, host-driven.  tri_v_dev: T*9 floats.
// With M > 1 the triangles are M meshes (mesh m = [mesh_off[m],
// mesh_off[m+1]), device offsets) built as one forest whose root of mesh m is
// node m.  Also builds the traversal layout and records t.plan.
int build_tree(Tree &t, const float *tri_v_dev, int32_t T, const kdgb_build_params &p, cudaStream_t s,
               const int32_t *mesh_off_dev = nullptr, int32_t M = 1);

// A side branch of a captured build: work that does not lie on the level
// chain runs on `aux` beside it (fork on ev[0], join on ev[1]).
struct Fork {
    cudaStream_t aux = nullptr;
    cudaEvent_t ev[2] = {nullptr, nullptr};
};

// The same build recorded into the graph being captured on `cs`: fixed
// buffers sized from t.plan x headroom, level loops as WHILE nodes, no host
// synchronisation.  `body` is a second stream used to capture loop bodies;
// the packed triangle records and the leaf records are made on fork.aux.
int capture_build(Tree &t, const float *tri_v_dev, int32_t T, const kdgb_build_params &p, cudaStream_t cs,
                  cudaStream_t body, const Fork &fork, const int32_t *mesh_off_dev, int32_t M, GraphKernels &counts);

// Allocates every buffer capture_build uses, before capture starts.
int reserve_for_graph(Tree &t, int32_t T, const kdgb_build_params &p, int32_t M, double headroom, cudaStream_t s);

// Copies the device build counters into the host mirrors of t (synchronises
// s).  Returns the build's failure status, if any.
int read_build_state(Tree &t, cudaStream_t s);

int load_geometry(Tree &t, const float *tri_v_dev, int32_t T, cudaStream_t s);

// Traversal layout from the SoA arrays of a tree whose host counts are
// current (kdgb_tree_upload).
int pack_for_traversal(Tree &t, cudaStream_t s);

// Scan inputs: a loader fills the K lanes of record r.
template <int K>
struct ScanArray {
    const int32_t *in;  // n records of K consecutive ints
#ifdef __CUDACC__
    __device__ __forceinline__ void load(int64_t r, int32_t (&v)[K]) const
    {
#pragma unroll
        for (int k = 0; k < K; ++k) v[k] = in[r * K + k];
    }
#endif
};

// The seven per-node lanes of an upper level, computed from the node's
// left/right reference counts and its empty-space node count (see
// k_count and k_node_split): left, right, left references that go to a leaf,
// right references that go to a leaf, left-is-leaf, right-is-leaf, empty-space
// nodes (CalcNodeChildSize, SetPrimitiveLeafSide, MarkNodeLeafs:
// TriangleUpperChildren.h:144-201).
struct NodeLanes {
    const int32_t *cnt;     // 2 per node
    const int32_t *ess[2];  // 1 per node, in ess[*level & 1]
    const int32_t *level;   // completed upper levels (device)
    int32_t LS;             // leaf threshold
#ifdef __CUDACC__
    __device__ __forceinline__ void load(int64_t k, int32_t (&v)[7]) const
    {
        // Both parities' counts are loaded with the level, so no load waits
        // for another.
        const int32_t l = cnt[2 * k], r = cnt[2 * k + 1], e0 = ess[0][k], e1 = ess[1][k], lv = *level;
        const int ll = l < LS, rl = r < LS;
        v[0] = l; v[1] = r; v[2] = ll ? l : 0; v[3] = rl ? r : 0; v[4] = ll; v[5] = rl; v[6] = (lv & 1) ? e1 : e0;
    }
#endif
};

// The two per-node lanes of the traversal pack: the node's leaf records
// (its bitmap's members when it is a leaf, else 0) and whether it is an
// interior node.  Their exclusive scans give each leaf its first record and
// each interior node its rank, which places its children.
struct PackLanes {
    const int8_t *info;
    const int32_t *bitmap;
#ifdef __CUDACC__
    __device__ __forceinline__ void load(int64_t k, int32_t (&v)[2]) const
    {
        const bool leaf = (info[k] & 3) == KDGB_LEAF;
        v[0] = leaf ? __popc((unsigned)bitmap[k]) : 0;
        v[1] = leaf ? 0 : 1;
    }
#endif
};

// Device-wide exclusive scan of n records of K int32 lanes (lanes scanned
// independently), one launch.  out has n+1 records; record n holds the
// totals.  `ws` holds the scan's control words and tile status; it persists
// between scans and is grown (zeroed) here when too small.  With n_dev set,
// the kernel reads the length there (at most n, which then only sizes the
// grid and the status).  A bounded wait that gives up stores
// KDGB_ERR_TIMEOUT in *err (when given) if it is still 0.
template <int K, class In>
int scan_exclusive_in(const In &in, int32_t *out, int64_t n, cudaStream_t s, DevArray<int32_t> *ws,
                      const int32_t *n_dev = nullptr, int32_t *err = nullptr);

template <int K>
inline int scan_exclusive(const int32_t *in, int32_t *out, int64_t n, cudaStream_t s, DevArray<int32_t> *ws,
                          const int32_t *n_dev = nullptr, int32_t *err = nullptr)
{
    return scan_exclusive_in<K, ScanArray<K>>(ScanArray<K>{in}, out, n, s, ws, n_dev, err);
}

// Workspace (int32 elements) a scan of n records of K lanes needs.
int64_t scan_partials_needed(int K, int64_t n);

// Runs one look-back wait that must give up (see k_scan_giveup): result[0]
// = the status it recorded, result[1] = the prefix it assumed for the tile
// that never published.  Synchronises `s`.
int scan_giveup_check(int32_t spin_limit, int32_t *result, cudaStream_t s);

// Two independent scans (as scan_exclusive_in each) in one launch.
template <int K1, class In1, int K2, class In2>
int scan_exclusive_pair(const In1 &in1, int32_t *out1, int64_t n1, const int32_t *n1_dev, const In2 &in2,
                        int32_t *out2, int64_t n2, const int32_t *n2_dev, cudaStream_t s, DevArray<int32_t> *ws,
                        int32_t *err = nullptr);

// Workspace (int32 elements) a scan pair of n1 and n2 records needs.
int64_t scan_pair_needed(int64_t n1, int64_t n2);

// Hash of every device buffer's address and capacity: a captured graph is
// valid while this is unchanged.
uint64_t layout_signature(const Tree &t);

// ---------------------------------------------------------------------------
// Device helpers.
// ---------------------------------------------------------------------------
#ifdef __CUDACC__

__device__ __forceinline__ float3 sub3(float3 a, float3 b)
{
    return make_float3(__fsub_rn(a.x, b.x), __fsub_rn(a.y, b.y), __fsub_rn(a.z, b.z));
}
// dot and cross of the CUDA-SDK vector helpers, left to right, no FMA.
__device__ __forceinline__ float dot3(float3 a, float3 b)
{
    float s = __fmul_rn(a.x, b.x);
    s = __fadd_rn(s, __fmul_rn(a.y, b.y));
    s = __fadd_rn(s, __fmul_rn(a.z, b.z));
    return s;
}
__device__ __forceinline__ float3 cross3(float3 a, float3 b)
{
    return make_float3(__fsub_rn(__fmul_rn(a.y, b.z), __fmul_rn(a.z, b.y)),
                       __fsub_rn(__fmul_rn(a.z, b.x), __fmul_rn(a.x, b.z)),
                       __fsub_rn(__fmul_rn(a.x, b.y), __fmul_rn(a.y, b.x)));
}
__device__ __forceinline__ float3 inv3(float3 d)
{
    return make_float3(__frcp_rn(d.x), __frcp_rn(d.y), __frcp_rn(d.z));
}

// min / max with IEEE totalOrder between -0 and +0 (finite inputs).
__device__ __forceinline__ float kmin(float a, float b)
{
    return a < b ? a : (b < a ? b : (signbit(a) ? a : b));
}
__device__ __forceinline__ float kmax(float a, float b)
{
    return a > b ? a : (b > a ? b : (signbit(a) ? b : a));
}

// Order-preserving float <-> uint32 keys (totalOrder on non-NaN values).
__device__ __forceinline__ unsigned fkey(float f)
{
    const unsigned b = __float_as_uint(f);
    return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}
__device__ __forceinline__ float funkey(unsigned k)
{
    return __uint_as_float((k & 0x80000000u) ? (k & 0x7fffffffu) : ~k);
}

__device__ __forceinline__ float axis_of(float3 a, int axis)
{
    return axis == KDGB_X ? a.x : (axis == KDGB_Y ? a.y : a.z);
}
__device__ __forceinline__ float axis_of4(float4 a, int axis)
{
    return axis == KDGB_X ? a.x : (axis == KDGB_Y ? a.y : a.z);
}

// IRayTracer.h:60-65 AdjustRayDirection.
// Leaf boxes of the traversal layout: min then max of node j at [2j] and
// [2j + 1], so one box is one 32-byte sector.
constexpr int kBoxStride = 2;

__device__ __forceinline__ float3 adjust_dir(float3 d)
{
    const float ooeps = 0x1p-80f;
    d.x = fabsf(d.x) > ooeps ? d.x : copysignf(ooeps, d.x);
    d.y = fabsf(d.y) > ooeps ? d.y : copysignf(ooeps, d.y);
    d.z = fabsf(d.z) > ooeps ? d.z : copysignf(ooeps, d.z);
    return d;
}

#endif  // __CUDACC__

}  // namespace kdgb

struct kdgb_tree {
    kdgb::Tree t;
};
