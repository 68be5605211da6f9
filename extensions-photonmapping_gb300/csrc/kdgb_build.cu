// kd-tree build on the GPU, reference mode and tuned mode.
//
// Reproduces TriangleMap::Create (Utils/CUDA/TriangleMap.cu:51-62) with the
// default upper creator (TriangleMapUpperCreator.cu:110-759, BOX split
// method, empty-space splitting) followed by the BITMAP lower creator
// (TriangleMapBitmapCreator.cu:32-65) or the SAH lower creator
// (TriangleMapSAHCreator.cu:67-260, LowerTriangleMap.h).  Node numbering,
// reference order and every float are identical to the reference's; the
// mechanics differ:
//  * one thread per reference with warp-aggregated atomics replaces the
//    256-reference segments, CUDPP scans and the host loop of single-block
//    FinalSegmentedReduce launches (ReduceSegments.h:337-371);
//  * per-node child sizes and leaf decisions come from per-node counts and a
//    seven-lane node scan, and a reference's destination is its node base
//    plus its rank inside the node (ballot scan + chunk offset), which equals
//    the reference's 2N+1-element scans (TriangleMapUpperCreator.cu:557,631);
//  * every size lives in a device-resident BuildState that the last block of
//    each level's closing kernel updates, and every kernel
//    loops over the counts it reads there.  The host-driven build reads the
//    state once per level to size buffers and grids exactly; the graph build
//    (capture_build) records the same launch sequence once, with fixed
//    buffers and the level loops as conditional WHILE nodes, so a rebuild is
//    one graph launch with no host round trip.  Kernels check the fixed
//    capacities before writing and the build stops with KDGB_ERR_CAPACITY
//    rather than write past them.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>

#include "kdgb_internal.cuh"

namespace kdgb {

namespace {

constexpr int kBlock = 256;

__host__ __device__ inline int64_t ceil_div(int64_t a, int64_t b) { return (a + b - 1) / b; }

// The per-reference passes (k_reduce, k_count, k_scatter) walk
// the reference array in warp chunks of kRows rows of 32 consecutive
// references, kWarps consecutive chunks per block tile.  Owners are sorted,
// so most rows belong to one node: a warp keeps per-lane accumulators while
// the owner stays the same and only reduces and issues atomics when it
// changes, which keeps atomic traffic to a few per node per chunk even at the
// root, where every reference has the same owner.
constexpr int kRows = 4;
constexpr int kChunk = 32 * kRows;  // references per warp chunk
constexpr int kWarps = kBlock / 32;
constexpr int kTileRefs = kChunk * kWarps;  // references per block tile
constexpr int kLanes = 7;                   // per-node scan lanes (see NodeLanes)
// Tuned levels: nodes with at least this many references are binned by a
// whole block, smaller ones by one warp (k_sah_bin).
constexpr int kSahBlockRefs = 512;
// A large node is binned in chunks of kSahChunkRefs references, one block
// each; chunk items are {node index in the level, histogram slot, chunk,
// chunks}.  The blocks add their histograms into the node's global slot of
// kSahHist ints (6 x 32 bins and a count of finished chunks); the last one
// picks the split and zeroes the slot again.
constexpr int kSahItem = 4;
// The traversal layout keeps a node index in 30 bits (kdgb_trace.cu).
constexpr int64_t kMaxPackNodes = int64_t(1) << 29;
constexpr int kSahHist = 6 * 32 + 1;
constexpr int kSahChunkRefs = 2048;
// Chunk items a level of `refs` references can list: ceil(cnt / kSahChunkRefs)
// per node of cnt >= kSahBlockRefs references, at most 2 refs / kSahBlockRefs.
inline int64_t sah_items(int64_t refs) { return 2 * refs / kSahBlockRefs + 1; }
constexpr unsigned kFull = 0xffffffffu;
// SAH lower levels: the split decisions are counted per tile of kLowTile
// consecutive nodes of a level; k_sah_children (one block per tile) numbers
// the children from these counts.
constexpr int kLowTile = kBlock;

__host__ __device__ inline int64_t chunks_for(int64_t n) { return (n + kChunk - 1) / kChunk; }

// Failure details recorded in BuildState::err_detail.
enum {
    kErrNonfinite = 1,
    kErrUpperCapacity = 2,
    kErrLeafCapacity = 3,
    kErrFewerRefs = 4,
    kErrMaxLevels = 5,
    kErrLowerCapacity = 6,
    kErrPackCapacity = 7,
};

// Capacities (elements) of the buffers a build writes.  The host-driven
// build grows buffers before each level, so its checks always pass; a graph
// build has fixed buffers and stops when a check fails.
struct Caps {
    int64_t refs[2];  // reference buffers 0 and 1
    int64_t fin;      // leaf references
    int64_t nodes;    // node arrays
    int64_t R;        // next-level node entries written by k_children
    int64_t leaves;   // upper leaf ids
    int64_t ranges;   // leaf-producing levels
    int64_t low_R;    // SAH lower level arrays
    int64_t tris;     // leaf records of the traversal layout
    int64_t big;      // binning chunks listed per tuned level (kSahItem ints each)
    int64_t list[2];  // SAH lower work list entries, by level parity
    int64_t lcnt[2];  // SAH lower tile split counts, by level parity
};

// Everything a build kernel touches; passed by value to every kernel.
struct BuildArgs {
    BuildState *st;
    Caps cap;
    int32_t T, M, LS, B, upper_levels, max_levels, min_leaf;
    int ess, zmax_as_x, propagate, tuned, lower, divide;
    float thr, ct, ci;
    const int32_t *mesh_off;
    float4 *p0, *p1, *p2;
    float4 *prec;  // packed triangle records (Tree::prec)
    float4 *rmin[2], *rmax[2], *fmin, *fmax;
    int8_t *info;
    float *split;
    float4 *bmin, *bmax;
    int32_t *pidx, *amt, *parent;
    int2 *ch;
    float *area;
    int32_t *prim_indices, *leaf_ids;
    unsigned *keys;
    int32_t *cnt, *lbase, *chunksum, *tilesum, *tileoff, *big, *bighist;
    // Empty-space planes and node counts of a level, in buffer (level & 1)
    // (st->level counts the completed levels): k_children writes the next
    // level's while it reads the current one's.
    int32_t *ess_cnt[2];
    int8_t *planes[2];
    int2 *ranges;
    int32_t *roff;
    float *areas;
    int4 *sts;
    int32_t *ssplit;
    int32_t *lcnt[2];  // split nodes per kLowTile nodes of a lower level, by level parity
    float2 *careas;
    int2 *csets;
    int32_t *lowlist[2];
    int32_t *loff;  // PackLanes scan: 2 ints per node and the totals
    int2 *tnode;
    float4 *tbox;
    int32_t *norder;  // each node's index in the traversal order
    float4 *ttri;
    cudaGraphConditionalHandle upper_cond, lower_cond;
    int use_cond;
};

__device__ __forceinline__ void set_err(BuildState *st, int status, int detail)
{
    if (!st->err) {
        st->err = status;
        st->err_detail = detail;
    }
}

__device__ __forceinline__ bool sah_level(const BuildArgs &a, const BuildState *st)
{
    return a.tuned && st->level + 1 > a.upper_levels;
}

// Empty-space splitting runs on every level but the first, in tuned mode
// too (ahead of the binned SAH split of the remaining box).
__device__ __forceinline__ bool do_ess(const BuildArgs &a, const BuildState *st)
{
    return a.ess && st->active != 0;
}

#define GRID_STRIDE(i, n) \
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < (n); i += (int64_t)gridDim.x * blockDim.x)
#define WARP_STRIDE(w, n)                                                          \
    for (int64_t w = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; w < (n); \
         w += ((int64_t)gridDim.x * blockDim.x) >> 5)

// ---------------------------------------------------------------------------
// Geometry and primitive boxes (CalcPrimitiveAabb, TriangleUpper.h:10-28).
// ---------------------------------------------------------------------------
// Index of the mesh owning triangle i (mesh m owns [off[m], off[m+1])).
__device__ __forceinline__ int mesh_of(const int32_t *__restrict__ off, int M, int32_t i)
{
    int lo = 0, hi = M - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (off[mid] <= i) lo = mid; else hi = mid - 1;
    }
    return lo;
}

__global__ void k_load_geometry(const float *__restrict__ tri, int32_t T, float4 *__restrict__ p0,
                                float4 *__restrict__ p1, float4 *__restrict__ p2,
                                float4 *__restrict__ cmin, float4 *__restrict__ cmax,
                                int *__restrict__ err, const int32_t *__restrict__ mesh_off, int M)
{
    GRID_STRIDE(ii, T) {
        const int32_t i = (int32_t)ii;
        const float *tp = tri + 9 * (int64_t)i;
        float v[9];
#pragma unroll
        for (int k = 0; k < 9; ++k) v[k] = tp[k];
        bool finite = true;
#pragma unroll
        for (int k = 0; k < 9; ++k) finite = finite && isfinite(v[k]);
        if (!finite) atomicOr(err, 1);
        p0[i] = make_float4(v[0], v[1], v[2], 1.0f);
        p1[i] = make_float4(v[3], v[4], v[5], 1.0f);
        p2[i] = make_float4(v[6], v[7], v[8], 1.0f);
        if (cmin) {
            float mnx = kmin(v[0], v[3]), mny = kmin(v[1], v[4]), mnz = kmin(v[2], v[5]);
            float mxx = kmax(v[0], v[3]), mxy = kmax(v[1], v[4]), mxz = kmax(v[2], v[5]);
            cmin[i] = make_float4(kmin(mnx, v[6]), kmin(mny, v[7]), kmin(mnz, v[8]), __int_as_float(i));
            // w carries the local index of the owning active node: the root
            // of the triangle's mesh (0 for a single mesh).
            const int owner = M > 1 ? mesh_of(mesh_off, M, i) : 0;
            cmax[i] = make_float4(kmax(mxx, v[6]), kmax(mxy, v[7]), kmax(mxz, v[8]), __int_as_float(owner));
        }
    }
}

// The packed triangle records {v0.xyz, e1.x} {e1.yz, e2.xy} {e2.z, id, 0, 0}
// (e1 = v1 - v0, e2 = v2 - v0, rounded as the tracers compute them), read by
// the SAH areas and copied into the leaf records; nothing on the upper levels
// reads them, so a captured build makes them beside the level chain.
__global__ void k_load_prec(const float *__restrict__ tri, int32_t T, float4 *__restrict__ prec)
{
    GRID_STRIDE(ii, T) {
        const int32_t i = (int32_t)ii;
        const float *tp = tri + 9 * (int64_t)i;
        const float3 v0 = make_float3(tp[0], tp[1], tp[2]);
        const float3 e1 = sub3(make_float3(tp[3], tp[4], tp[5]), v0);
        const float3 e2 = sub3(make_float3(tp[6], tp[7], tp[8]), v0);
        prec[3 * (int64_t)i + 0] = make_float4(v0.x, v0.y, v0.z, e1.x);
        prec[3 * (int64_t)i + 1] = make_float4(e1.y, e1.z, e2.x, e2.y);
        prec[3 * (int64_t)i + 2] = make_float4(e2.z, __int_as_float(i), 0.0f, 0.0f);
    }
}

__device__ __forceinline__ void zero_node(int32_t j, int8_t *info, float *split, float4 *bmin, float4 *bmax,
                                          int32_t *pidx, int32_t *amt, int2 *ch, float *area, int32_t *parent)
{
    info[j] = 0;
    split[j] = 0.0f;
    bmin[j] = make_float4(0.f, 0.f, 0.f, 0.f);
    bmax[j] = make_float4(0.f, 0.f, 0.f, 0.f);
    pidx[j] = 0;
    amt[j] = 0;
    ch[j] = make_int2(0, 0);
    area[j] = 0.0f;
    parent[j] = 0;
}
#define ZERO_NODE(j) zero_node((j), a.info, a.split, a.bmin, a.bmax, a.pidx, a.amt, a.ch, a.area, a.parent)

// Build state, roots and the first level's node arrays.  Roots
// (TriangleMapUpperCreator.cu:128-136): node m is the root of mesh m,
// covering references [off[m], off[m+1]) (a single mesh: node 0, all of
// them).  The first level's tight-box keys are reset to +-fInfinity
// (AabbMemset, ReduceSegments.h:328-335).
__global__ void k_begin(const BuildArgs a)
{
    BuildState *st = a.st;
    const unsigned lo = fkey(KDGB_FINF), hi = fkey(-KDGB_FINF);
    GRID_STRIDE(mm, a.M) {
        const int32_t m = (int32_t)mm;
        ZERO_NODE(m);
        const int32_t b0 = a.M > 1 ? a.mesh_off[m] : 0, b1 = a.M > 1 ? a.mesh_off[m + 1] : a.T;
        a.pidx[m] = b0;
        a.amt[m] = b1 - b0;
        a.parent[m] = m;
        unsigned *kk = a.keys + 6 * (int64_t)m;
        kk[0] = kk[1] = kk[2] = lo;
        kk[3] = kk[4] = kk[5] = hi;
        a.cnt[2 * m] = 0;
        a.cnt[2 * m + 1] = 0;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        BuildState s;
        memset(&s, 0, sizeof(s));
        s.N = a.T;
        s.R = a.M;
        s.n_nodes = a.M;
        s.ntiles = (int32_t)ceil_div(a.T, kTileRefs);
        *st = s;
    }
}

// ---------------------------------------------------------------------------
// Upper level kernels.
// ---------------------------------------------------------------------------

__device__ __forceinline__ void keys_atomic(unsigned *keys, int o, const unsigned (&k)[6])
{
    unsigned *kk = keys + 6 * (int64_t)o;
    atomicMin(kk + 0, k[0]); atomicMin(kk + 1, k[1]); atomicMin(kk + 2, k[2]);
    atomicMax(kk + 3, k[3]); atomicMax(kk + 4, k[4]); atomicMax(kk + 5, k[5]);
}

__device__ __forceinline__ void keys_reduce(unsigned mask, unsigned (&k)[6])
{
    k[0] = __reduce_min_sync(mask, k[0]); k[1] = __reduce_min_sync(mask, k[1]); k[2] = __reduce_min_sync(mask, k[2]);
    k[3] = __reduce_max_sync(mask, k[3]); k[4] = __reduce_max_sync(mask, k[4]); k[5] = __reduce_max_sync(mask, k[5]);
}

__device__ __forceinline__ void keys_neutral(unsigned (&k)[6])
{
    k[0] = k[1] = k[2] = 0xffffffffu;
    k[3] = k[4] = k[5] = 0u;
}

// Tight node boxes of the roots: exact min/max over each node's references,
// as the segmented reduction ReduceSegmentsUnrolled + FinalSegmentedReduce
// (ReduceSegments.h:230-371) computes.  Keys are order-preserving uint32
// images of the floats, so atomicMin/atomicMax give exact results in any order.
__global__ void __launch_bounds__(kBlock) k_reduce(const BuildArgs a)
{
    __shared__ int s_owner[kWarps];
    __shared__ unsigned s_keys[kWarps][6];
    const BuildState *st = a.st;
    const int64_t N = st->N;
    const int cur = st->level & 1;
    const float4 *__restrict__ cmin = a.rmin[cur];
    const float4 *__restrict__ cmax = a.rmax[cur];
    unsigned *__restrict__ keys = a.keys;
    const unsigned lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int64_t ntiles = ceil_div(N, kTileRefs);
    for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const int64_t base = (tile * kWarps + warp) * kChunk;
        int cw = -1;
        unsigned acc[6];
        keys_neutral(acc);
        // Issue every row's loads before using any of them.
        float4 ra[kRows], rb[kRows];
#pragma unroll
        for (int row = 0; row < kRows; ++row) {
            const int64_t r = base + row * 32 + lane;
            if (r < N) { ra[row] = cmin[r]; rb[row] = cmax[r]; }
            else { rb[row].w = __int_as_float(-1); }
        }
#pragma unroll
        for (int row = 0; row < kRows; ++row) {
            if (base + row * 32 >= N) break;
            const int o = __float_as_int(rb[row].w);
            unsigned k[6];
            keys_neutral(k);
            if (o >= 0) {
                const float4 p = ra[row], q = rb[row];
                k[0] = fkey(p.x); k[1] = fkey(p.y); k[2] = fkey(p.z);
                k[3] = fkey(q.x); k[4] = fkey(q.y); k[5] = fkey(q.z);
            }
            const unsigned m = __match_any_sync(kFull, o);
            if (m == kFull && o == cw) {
                acc[0] = min(acc[0], k[0]); acc[1] = min(acc[1], k[1]); acc[2] = min(acc[2], k[2]);
                acc[3] = max(acc[3], k[3]); acc[4] = max(acc[4], k[4]); acc[5] = max(acc[5], k[5]);
                continue;
            }
            if (cw >= 0) {
                keys_reduce(kFull, acc);
                if (lane == 0) keys_atomic(keys, cw, acc);
            }
            if (m == kFull && o >= 0) {
                cw = o;
                for (int j = 0; j < 6; ++j) acc[j] = k[j];
            } else {
                if (o >= 0) {
                    keys_reduce(m, k);
                    if (lane == (unsigned)(__ffs(m) - 1)) keys_atomic(keys, o, k);
                }
                cw = -1;
                keys_neutral(acc);
            }
        }
        if (cw >= 0) keys_reduce(kFull, acc);
        if (lane == 0) {
            s_owner[warp] = cw;
            for (int j = 0; j < 6; ++j) s_keys[warp][j] = acc[j];
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            // Consecutive warps cover consecutive chunks: merge equal owners.
            int o = -1;
            unsigned k[6];
            keys_neutral(k);
            for (int w = 0; w < kWarps; ++w) {
                const int ow = s_owner[w];
                if (ow < 0) continue;
                if (ow != o) {
                    if (o >= 0) keys_atomic(keys, o, k);
                    o = ow;
                    for (int j = 0; j < 6; ++j) k[j] = s_keys[w][j];
                } else {
                    for (int j = 0; j < 3; ++j) k[j] = min(k[j], s_keys[w][j]);
                    for (int j = 3; j < 6; ++j) k[j] = max(k[j], s_keys[w][j]);
                }
            }
            if (o >= 0) keys_atomic(keys, o, k);
        }
        __syncthreads();
    }
}

// One active node's tight box (from its keys), empty-space planes against
// its propagated box [lo, hi] (CalcEmptySpaceSplits,
// EmptySpaceSplitting.h:10-70) and spatial-median split of the longest axis
// (CalcUpperNodeSplitInfo, ReduceSegments.h:466-484); nodes of a binned-SAH
// level with at least kSahBlockRefs references are listed for block-wide
// binning.  k is the node's index in its level, node its id.
__device__ __forceinline__ void node_split_one(const BuildArgs &a, int32_t k, int32_t node, bool ess, float4 lo,
                                               float4 hi, bool sah, int8_t *planes, int32_t *ess_cnt)
{
    const float thr = a.thr;
    const unsigned *kk = a.keys + 6 * (int64_t)k;
    const float3 mn = make_float3(funkey(kk[0]), funkey(kk[1]), funkey(kk[2]));
    const float3 mx = make_float3(funkey(kk[3]), funkey(kk[4]), funkey(kk[5]));
    a.bmin[node] = make_float4(mn.x, mn.y, mn.z, 0.0f);
    a.bmax[node] = make_float4(mx.x, mx.y, mx.z, 0.0f);
    if (ess) {
        int pl = 0, nr = 0;
        if (__fsub_rn(mn.x, lo.x) > __fmul_rn(thr, __fsub_rn(hi.x, lo.x))) { pl |= 1; nr += 2; }
        if (__fsub_rn(mn.y, lo.y) > __fmul_rn(thr, __fsub_rn(hi.y, lo.y))) { pl |= 2; nr += 2; }
        if (__fsub_rn(mn.z, lo.z) > __fmul_rn(thr, __fsub_rn(hi.z, lo.z))) { pl |= 4; nr += 2; }
        if (__fsub_rn(hi.x, mx.x) > __fmul_rn(thr, __fsub_rn(hi.x, lo.x))) { pl |= 8; nr += 2; }
        if (__fsub_rn(hi.y, mx.y) > __fmul_rn(thr, __fsub_rn(hi.y, lo.y))) { pl |= 16; nr += 2; }
        if (__fsub_rn(hi.z, mx.z) > __fmul_rn(thr, __fsub_rn(hi.z, lo.z))) { pl |= 32; nr += 2; }
        planes[k] = (int8_t)pl;
        ess_cnt[k] = nr;
    } else {
        ess_cnt[k] = 0;
    }
    const float sx = __fsub_rn(mx.x, mn.x), sy = __fsub_rn(mx.y, mn.y), sz = __fsub_rn(mx.z, mn.z);
    const float mdx = __fadd_rn(__fmul_rn(sx, 0.5f), mn.x);
    const float mdy = __fadd_rn(__fmul_rn(sy, 0.5f), mn.y);
    const float mdz = __fadd_rn(__fmul_rn(sz, 0.5f), mn.z);
    const bool y_above_x = sx < sy;
    const float mxs = y_above_x ? sy : sx;
    const float sp = y_above_x ? mdy : mdx;
    const int8_t ax = y_above_x ? KDGB_Y : KDGB_X;
    const bool z_higher = mxs < sz;
    a.split[node] = z_higher ? mdz : sp;
    a.info[node] = z_higher ? (int8_t)KDGB_Z : ax;
    const int32_t cnt = a.amt[node];
    if (sah && cnt >= kSahBlockRefs) {
        const int32_t nch = (cnt + kSahChunkRefs - 1) / kSahChunkRefs;
        const int32_t base = atomicAdd(&a.st->n_big, nch);
        if ((int64_t)base + nch > a.cap.big) {
            set_err(a.st, KDGB_ERR_CAPACITY, kErrUpperCapacity);
            return;
        }
        for (int32_t c = 0; c < nch; ++c)
            reinterpret_cast<int4 *>(a.big)[base + c] = make_int4(k, base, c, nch);
    }
}

// The roots' splits (the first level; no empty-space cuts at the root).
// Later levels get theirs from k_children of the level before.
__global__ void k_node_split(const BuildArgs a)
{
    const BuildState *st = a.st;
    const int32_t R = st->R, active = st->active;
    const bool ess = do_ess(a, st), sah = sah_level(a, st);
    const int b = st->level & 1;
    const float4 zero = make_float4(0.f, 0.f, 0.f, 0.f);
    GRID_STRIDE(k64, R) {
        const int32_t k = (int32_t)k64;
        node_split_one(a, k, active + k, ess, zero, zero, sah, a.planes[b], a.ess_cnt[b]);
    }
}

__device__ __forceinline__ void ref_flags(const float4 &lo, const float4 &hi, int axis, float sp, int &L, int &Rf)
{
    // SetSplitSide (TriangleUpperChildren.h:10-62): left = min <= split,
    // right = split < max.
    L = axis_of4(lo, axis) <= sp;
    Rf = sp < axis_of4(hi, axis);
}

// One separating axis of Akenine-Moeller's triangle/box test, step 3 (a
// triangle edge crossed with a box axis), in the two coordinates (s, t)
// perpendicular to the box axis: edge a->b, third vertex c, box half sizes
// hs, ht, all relative to the box centre.  Expressions of a0XTests /
// a1XTests / a2XTests (IntersectionTests.h:23-149) with their slack
// r = (... + 1e-5) * 1.0001 (IntersectionTests.h:20-21), every operation
// rounded separately.
__device__ __forceinline__ bool sat_edge(float as, float at, float bs, float bt, float cs, float ct, float hs,
                                         float ht)
{
    const float p0 = __fsub_rn(__fmul_rn(at, bs), __fmul_rn(as, bt));
    const float p1 = __fsub_rn(__fmul_rn(__fsub_rn(bs, as), ct), __fmul_rn(__fsub_rn(bt, at), cs));
    float r = __fadd_rn(__fmul_rn(ht, fabsf(__fsub_rn(bs, as))), __fmul_rn(hs, fabsf(__fsub_rn(bt, at))));
    r = __fmul_rn(__fadd_rn(r, 0.00001f), 1.0001f);
    return !((p0 > r && p1 > r) || (p0 < -r && p1 < -r));
}

// TriangleAabbIntersectionStep3 (IntersectionTests.h:378-395): the nine
// edge-axis tests of the triangle against the box [lo, hi].
__device__ __forceinline__ bool tri_box_step3(float3 v0, float3 v1, float3 v2, float3 lo, float3 hi)
{
    const float3 h = make_float3(__fmul_rn(__fsub_rn(hi.x, lo.x), 0.5f), __fmul_rn(__fsub_rn(hi.y, lo.y), 0.5f),
                                 __fmul_rn(__fsub_rn(hi.z, lo.z), 0.5f));
    const float3 c = make_float3(__fadd_rn(lo.x, h.x), __fadd_rn(lo.y, h.y), __fadd_rn(lo.z, h.z));
    v0 = sub3(v0, c);
    v1 = sub3(v1, c);
    v2 = sub3(v2, c);
    bool ok = true;
    // box axis x: coordinates (y, z)
    ok &= sat_edge(v0.y, v0.z, v1.y, v1.z, v2.y, v2.z, h.y, h.z);
    ok &= sat_edge(v1.y, v1.z, v2.y, v2.z, v0.y, v0.z, h.y, h.z);
    ok &= sat_edge(v2.y, v2.z, v0.y, v0.z, v1.y, v1.z, h.y, h.z);
    // box axis y: coordinates (z, x)
    ok &= sat_edge(v0.z, v0.x, v1.z, v1.x, v2.z, v2.x, h.z, h.x);
    ok &= sat_edge(v1.z, v1.x, v2.z, v2.x, v0.z, v0.x, h.z, h.x);
    ok &= sat_edge(v2.z, v2.x, v0.z, v0.x, v1.z, v1.x, h.z, h.x);
    // box axis z: coordinates (x, y)
    ok &= sat_edge(v0.x, v0.y, v1.x, v1.y, v2.x, v2.y, h.x, h.y);
    ok &= sat_edge(v1.x, v1.y, v2.x, v2.y, v0.x, v0.y, h.x, h.y);
    ok &= sat_edge(v2.x, v2.y, v0.x, v0.y, v1.x, v1.y, h.x, h.y);
    return ok;
}

// SetDivideSide<false> (TriangleUpperChildren.h:64-142): a reference whose
// box straddles the plane is tested with its triangle against the two halves
// of the node's tight box; it may go to one side only, or to none when the
// triangle misses the node box although its clipped box does not.
__device__ __forceinline__ void divide_flags(const BuildArgs &a, int32_t prim, int32_t node, int axis, float sp,
                                            int &L, int &Rf)
{
    const float4 q0 = __ldg(a.p0 + prim), q1 = __ldg(a.p1 + prim), q2 = __ldg(a.p2 + prim);
    const float3 v0 = make_float3(q0.x, q0.y, q0.z), v1 = make_float3(q1.x, q1.y, q1.z),
                 v2 = make_float3(q2.x, q2.y, q2.z);
    const float4 mn = a.bmin[node], mx = a.bmax[node];
    const float3 lo = make_float3(mn.x, mn.y, mn.z), hi = make_float3(mx.x, mx.y, mx.z);
    const float3 lhi = make_float3(axis == KDGB_X ? sp : hi.x, axis == KDGB_Y ? sp : hi.y, axis == KDGB_Z ? sp : hi.z);
    const float3 rlo = make_float3(axis == KDGB_X ? sp : lo.x, axis == KDGB_Y ? sp : lo.y, axis == KDGB_Z ? sp : lo.z);
    L = tri_box_step3(v0, v1, v2, lo, lhi);
    Rf = tri_box_step3(v0, v1, v2, rlo, hi);
}

// Per-node left/right counts, per-chunk totals of the flags and per-tile
// totals (the tile totals are scanned into tile offsets; k_scatter adds the
// chunk totals of the earlier warps of its tile).  Also resets the tight-box
// keys of the next level's nodes (at most 2R of them) to the +-fInfinity box
// (AabbMemset, ReduceSegments.h:328-335): this level's keys were consumed
// when its splits were made, and k_scatter reduces the children's boxes into
// them.
template <bool DIVIDE>
__global__ void __launch_bounds__(kBlock, DIVIDE ? 2 : 4) k_count(const BuildArgs a)
{
    {
        const int64_t next = min(2 * (int64_t)a.st->R, a.cap.R);
        const unsigned lo_key = fkey(KDGB_FINF), hi_key = fkey(-KDGB_FINF);
        GRID_STRIDE(i, 6 * next) a.keys[i] = (i % 6) < 3 ? lo_key : hi_key;
        // This level's list of large nodes has been binned; k_children lists
        // the next level's.
        if (blockIdx.x == 0 && threadIdx.x == 0) a.st->n_big = 0;
    }
    __shared__ int s_owner[kWarps], s_l[kWarps], s_r[kWarps], s_tl[kWarps], s_tr[kWarps];
    const BuildState *st = a.st;
    const int64_t N = st->N;
    const int32_t active = st->active;
    const int cur = st->level & 1;
    const float4 *__restrict__ cmin = a.rmin[cur];
    const float4 *__restrict__ cmax = a.rmax[cur];
    int32_t *__restrict__ cnt = a.cnt;
    const unsigned lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int64_t ntiles = ceil_div(N, kTileRefs);
    for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const int64_t chunk = tile * kWarps + warp;
        const int64_t base = chunk * kChunk;
        int cw = -1, al = 0, ar = 0, tl = 0, tr = 0;
        float4 ra[kRows], rb[kRows];
#pragma unroll
        for (int row = 0; row < kRows; ++row) {
            const int64_t r = base + row * 32 + lane;
            if (r < N) { ra[row] = cmin[r]; rb[row] = cmax[r]; }
            else { rb[row].w = __int_as_float(-1); }
        }
        int ax[kRows];
        float sp[kRows];
#pragma unroll
        for (int row = 0; row < kRows; ++row) {
            const int o = __float_as_int(rb[row].w);
            ax[row] = o >= 0 ? a.info[active + o] : 0;
            sp[row] = o >= 0 ? a.split[active + o] : 0.0f;
        }
#pragma unroll
        for (int row = 0; row < kRows; ++row) {
            if (base + row * 32 >= N) break;
            const int o = __float_as_int(rb[row].w);
            int L = 0, Rf = 0;
            if (o >= 0) ref_flags(ra[row], rb[row], ax[row], sp[row], L, Rf);
            if (DIVIDE && L && Rf) divide_flags(a, __float_as_int(ra[row].w), active + o, ax[row], sp[row], L, Rf);
            tl += L;
            tr += Rf;
            const unsigned m = __match_any_sync(kFull, o);
            if (m == kFull && o == cw) {
                al += L;
                ar += Rf;
                continue;
            }
            // As in k_scatter: the run's lanes add to it before it is
            // flushed, whole parents in between are flushed here, and the
            // row's last parent starts the next run.
            if (cw >= 0 && o == cw) {
                al += L;
                ar += Rf;
            }
            if (cw >= 0) {
                al = __reduce_add_sync(kFull, al);
                ar = __reduce_add_sync(kFull, ar);
                if (lane == 0) { atomicAdd(cnt + 2 * cw, al); atomicAdd(cnt + 2 * cw + 1, ar); }
            }
            const int last = __shfl_sync(kFull, o, 31);
            if (o >= 0 && o != cw && o != last) {
                const int gl = __reduce_add_sync(m, L), gr = __reduce_add_sync(m, Rf);
                if (lane == (unsigned)(__ffs(m) - 1)) { atomicAdd(cnt + 2 * o, gl); atomicAdd(cnt + 2 * o + 1, gr); }
            }
            cw = last >= 0 && last != cw ? last : -1;
            if (cw >= 0 && o == cw) {
                al = L;
                ar = Rf;
            } else {
                al = 0;
                ar = 0;
            }
        }
        if (cw >= 0) {
            al = __reduce_add_sync(kFull, al);
            ar = __reduce_add_sync(kFull, ar);
        }
        tl = __reduce_add_sync(kFull, tl);
        tr = __reduce_add_sync(kFull, tr);
        if (lane == 0) {
            if (base < N) {
                a.chunksum[2 * chunk] = tl;
                a.chunksum[2 * chunk + 1] = tr;
            }
            s_owner[warp] = cw;
            s_l[warp] = al;
            s_r[warp] = ar;
            s_tl[warp] = tl;
            s_tr[warp] = tr;
        }
        __syncthreads();
        if (threadIdx.x == 32) {
            int sl = 0, sr = 0;
            for (int w = 0; w < kWarps; ++w) { sl += s_tl[w]; sr += s_tr[w]; }
            a.tilesum[2 * tile] = sl;
            a.tilesum[2 * tile + 1] = sr;
        }
        if (threadIdx.x == 0) {
            // Consecutive warps cover consecutive chunks: merge equal owners.
            int o = -1, l = 0, r = 0;
            for (int w = 0; w < kWarps; ++w) {
                const int ow = s_owner[w];
                if (ow < 0) continue;
                if (ow != o) {
                    if (o >= 0) { atomicAdd(cnt + 2 * o, l); atomicAdd(cnt + 2 * o + 1, r); }
                    o = ow; l = s_l[w]; r = s_r[w];
                } else {
                    l += s_l[w]; r += s_r[w];
                }
            }
            if (o >= 0) { atomicAdd(cnt + 2 * o, l); atomicAdd(cnt + 2 * o + 1, r); }
        }
        __syncthreads();
    }
}

// ---------------------------------------------------------------------------
// Tuned mode: binned SAH for the upper levels below `upper_levels` (the
// reference splits every upper level at the median).  Per node and axis with
// extent > 0: B equal bins over the tight box; each reference adds 1 to the
// bin of its box min (left histogram) and of its box max (right histogram).
// The plane at bin boundary k has NL = left counts below k, NR = right counts
// from k up and cost AL*NL + AR*NR (half box areas); the first strict
// minimum over (axis X,Y,Z; k = 1..B-1) wins, skipping planes that leave a
// side empty or keep every reference on both sides; without a qualifying
// plane the median split stays.
// ---------------------------------------------------------------------------

__device__ __forceinline__ int sah_bin(float x, float mn, float scale, int B)
{
    const int b = (int)__fmul_rn(__fsub_rn(x, mn), scale);
    return b < 0 ? 0 : (b > B - 1 ? B - 1 : b);
}


struct SahNode {
    int32_t node, cnt;
    int64_t first;
    float mnv[3], mxv[3], ext[3], scale[3];
    bool valid[3];
};

// Adds the references of rows row0, row0 + step, ... below row_end (32
// references each) of one node to the histograms
// h[(axis * 2 + side) * 32 + bin] (shared memory private to the calling
// warp), one shared atomic per reference, axis and side (cheaper than
// merging equal bins first).  kRows rows of loads are in flight before any
// of them is binned.
__device__ __forceinline__ void sah_rows(const float4 *__restrict__ cmin, const float4 *__restrict__ cmax,
                                         const SahNode &n, int B, int row0, int step, int row_end, int *h)
{
    const int lane = threadIdx.x & 31;
    const int rows = row_end;
    for (int r0 = row0; r0 < rows; r0 += kRows * step) {
        float4 p[kRows], q[kRows];
        bool in[kRows];
#pragma unroll
        for (int u = 0; u < kRows; ++u) {
            const int32_t i = (r0 + u * step) * 32 + lane;
            in[u] = r0 + u * step < rows && i < n.cnt;
            if (in[u]) { p[u] = cmin[n.first + i]; q[u] = cmax[n.first + i]; }
        }
#pragma unroll
        for (int u = 0; u < kRows; ++u) {
            if (!in[u]) continue;
            const float pv[3] = {p[u].x, p[u].y, p[u].z}, qv[3] = {q[u].x, q[u].y, q[u].z};
#pragma unroll
            for (int ax = 0; ax < 3; ++ax) {
                if (!n.valid[ax]) continue;
                atomicAdd(h + (ax * 2 + 0) * 32 + sah_bin(pv[ax], n.mnv[ax], n.scale[ax], B), 1);
                atomicAdd(h + (ax * 2 + 1) * 32 + sah_bin(qv[ax], n.mnv[ax], n.scale[ax], B), 1);
            }
        }
    }
}

// One warp evaluates the planes of a node from its six histograms (lane j
// holds bin j of each): lane k-1 takes the plane at bin boundary k; the first
// strict minimum over (axis, k) wins.  Lane 0 writes the split.
__device__ __forceinline__ void sah_pick(const BuildArgs &a, const SahNode &n, const int (&hv)[6], int lane)
{
    const int B = a.B;
    float best = INFINITY, best_sp = 0.0f;
    int best_ax = -1;
    for (int ax = 0; ax < 3; ++ax) {
        if (!n.valid[ax]) continue;  // warp-uniform
        int32_t plo = lane < B ? hv[ax * 2 + 0] : 0;  // inclusive prefix sums over bins
        int32_t phi = lane < B ? hv[ax * 2 + 1] : 0;
        for (int s = 1; s < 32; s <<= 1) {
            const int32_t x = __shfl_up_sync(kFull, plo, s), y = __shfl_up_sync(kFull, phi, s);
            if (lane >= s) { plo += x; phi += y; }
        }
        const int32_t total_hi = __shfl_sync(kFull, phi, 31);
        const int k = lane + 1;
        float cost = INFINITY, pk = 0.0f;
        if (k < B) {
            const int32_t nl = plo, nr = total_hi - phi;
            const float w = __fdiv_rn(n.ext[ax], (float)B);
            pk = __fadd_rn(n.mnv[ax], __fmul_rn((float)k, w));
            float le[3] = {n.ext[0], n.ext[1], n.ext[2]}, re[3] = {n.ext[0], n.ext[1], n.ext[2]};
            le[ax] = __fsub_rn(pk, n.mnv[ax]);
            re[ax] = __fsub_rn(n.mxv[ax], pk);
            const float al = __fadd_rn(__fadd_rn(__fmul_rn(le[0], le[1]), __fmul_rn(le[1], le[2])), __fmul_rn(le[2], le[0]));
            const float ar = __fadd_rn(__fadd_rn(__fmul_rn(re[0], re[1]), __fmul_rn(re[1], re[2])), __fmul_rn(re[2], re[0]));
            const float c = __fadd_rn(__fmul_rn(al, (float)nl), __fmul_rn(ar, (float)nr));
            if (nl > 0 && nr > 0 && !(nl == n.cnt && nr == n.cnt)) cost = c;
        }
        // First minimum in k order within the axis, then strictly better
        // than the previous axes.
        float c = cost;
        int kk = k;
        for (int s = 16; s > 0; s >>= 1) {
            const float c2 = __shfl_xor_sync(kFull, c, s);
            const int k2 = __shfl_xor_sync(kFull, kk, s);
            if (c2 < c || (c2 == c && k2 < kk)) { c = c2; kk = k2; }
        }
        const float sp = __shfl_sync(kFull, pk, kk - 1);
        if (c < best) { best = c; best_ax = ax; best_sp = sp; }
    }
    if (lane == 0 && best_ax >= 0) {
        a.info[n.node] = (int8_t)(best_ax + 1);
        a.split[n.node] = best_sp;
    }
}

// An active node's references are contiguous: [pidx, pidx + amt) of the
// current reference buffer (k_begin / k_children place them so).
__device__ __forceinline__ SahNode sah_node(const BuildArgs &a, int32_t node)
{
    SahNode n;
    n.node = node;
    n.cnt = a.amt[node];
    n.first = a.pidx[node];
    const float4 mn4 = a.bmin[node], mx4 = a.bmax[node];
    n.mnv[0] = mn4.x; n.mnv[1] = mn4.y; n.mnv[2] = mn4.z;
    n.mxv[0] = mx4.x; n.mxv[1] = mx4.y; n.mxv[2] = mx4.z;
#pragma unroll
    for (int ax = 0; ax < 3; ++ax) {
        n.ext[ax] = __fsub_rn(n.mxv[ax], n.mnv[ax]);
        n.valid[ax] = n.ext[ax] > 0.0f;
        n.scale[ax] = n.valid[ax] ? __fdiv_rn((float)a.B, n.ext[ax]) : 0.0f;
    }
    return n;
}

// Binned SAH of the active nodes, one launch per tuned level.  First the
// chunks of the nodes with kSahBlockRefs references or more (listed with the
// splits), one block each, dealt to the blocks in turn: every warp bins an
// interleaved share of the chunk's rows into its own histograms, the block
// sums them and adds them into the node's global slot, and the block that
// finishes the node's last chunk picks its split (a node of one chunk is
// picked from shared memory directly).  Then the smaller nodes, one warp
// each.  Bin counts are integers, so the order of the additions cannot
// change them.
__global__ void __launch_bounds__(kBlock, 4) k_sah_bin(const BuildArgs a)
{
    __shared__ int s_hist[kWarps][6 * 32];
    __shared__ int32_t s_last;
    BuildState *st = a.st;
    if (!sah_level(a, st)) return;
    const int32_t nb = st->n_big, R = st->R, active = st->active;
    const int cur = st->level & 1;
    const float4 *__restrict__ cmin = a.rmin[cur];
    const float4 *__restrict__ cmax = a.rmax[cur];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int *h = s_hist[warp];
    int hv[6];
    constexpr int kChunkRows = kSahChunkRefs / 32;
    // Chunks are dealt to the blocks in turn (they hold at most kSahChunkRefs
    // references each, so the shares are even); a shared work counter would
    // make every block of the grid contend for one address twice.
    for (int32_t it = blockIdx.x; it < nb; it += gridDim.x) {  // block-uniform
        const int4 item = reinterpret_cast<const int4 *>(a.big)[it];  // {k, slot, chunk, chunks}
        const SahNode n = sah_node(a, active + item.x);
        for (int j = lane; j < 6 * 32; j += 32) h[j] = 0;
        __syncwarp();
        const int rows = (n.cnt + 31) >> 5;
        const int row_end = min(rows, (item.z + 1) * kChunkRows);
        sah_rows(cmin, cmax, n, a.B, item.z * kChunkRows + warp, kWarps, row_end, h);
        __syncthreads();
        if (item.w == 1) {
            if (warp == 0) {
#pragma unroll
                for (int j = 0; j < 6; ++j) {
                    int sum = 0;
#pragma unroll
                    for (int w = 0; w < kWarps; ++w) sum += s_hist[w][j * 32 + lane];
                    hv[j] = sum;
                }
                sah_pick(a, n, hv, lane);
            }
        } else {
            int32_t *g = a.bighist + (int64_t)item.y * kSahHist;
            for (int j = threadIdx.x; j < 6 * 32; j += blockDim.x) {
                int sum = 0;
#pragma unroll
                for (int w = 0; w < kWarps; ++w) sum += s_hist[w][j];
                if (sum) atomicAdd(g + j, sum);
            }
            __threadfence();
            __syncthreads();
            if (threadIdx.x == 0) s_last = atomicAdd(g + 6 * 32, 1) == item.w - 1;
            __syncthreads();
            if (s_last && warp == 0) {  // every chunk of the node is in g
                __threadfence();
#pragma unroll
                for (int j = 0; j < 6; ++j) hv[j] = atomicExch(g + j * 32 + lane, 0);
                if (lane == 0) atomicExch(g + 6 * 32, 0);
                sah_pick(a, n, hv, lane);
            }
        }
        __syncthreads();  // s_hist and s_last are reused
    }
    WARP_STRIDE(gw, R) {
        const int32_t node = active + (int32_t)gw;
        if (a.amt[node] >= kSahBlockRefs) continue;  // warp-uniform
        const SahNode n = sah_node(a, node);
        for (int j = lane; j < 6 * 32; j += 32) h[j] = 0;
        __syncwarp();
        sah_rows(cmin, cmax, n, a.B, 0, 1, (n.cnt + 31) >> 5, h);
        __syncwarp();
#pragma unroll
        for (int j = 0; j < 6; ++j) hv[j] = h[j * 32 + lane];
        sah_pick(a, n, hv, lane);
        __syncwarp();
    }
}

// The totals record of the node scan: {left, right, left leaf refs, right
// leaf refs, left leaf nodes, right leaf nodes, empty-space nodes}.
__device__ __forceinline__ const int32_t *node_totals(const BuildArgs &a, const BuildState *st)
{
    return a.lbase + kLanes * (int64_t)st->R;
}

// Whether this level's outputs fit the buffers: next-level references, leaf
// references, nodes and next-level node entries.
__device__ __forceinline__ bool level_fits(const BuildArgs &a, const BuildState *st, const int32_t *tot)
{
    const int64_t next_refs = (int64_t)tot[0] + tot[1] - tot[2] - tot[3];
    const int64_t fin = st->F + tot[2] + tot[3];
    const int64_t nodes = (int64_t)st->n_nodes + tot[6] + 2 * (int64_t)st->R;
    const int64_t created = 2 * (int64_t)st->R - tot[4] - tot[5];
    return next_refs <= a.cap.refs[(st->level + 1) & 1] && fin <= a.cap.fin && nodes <= a.cap.nodes &&
           created <= a.cap.R;
}

// Writes one reference to its child (or final leaf) slot: destination = node
// base + rank among the node's left (right) references.
__device__ __forceinline__ void scatter_one(const BuildArgs &a, int32_t R, int owner, int32_t upper, int L, int Rf,
                                            float4 lo, float4 hi, float4 h, float4 l, int32_t pl, int32_t pr,
                                            float4 *__restrict__ nmin, float4 *__restrict__ nmax)
{
    const int32_t LS = a.LS;
    const int32_t *lb = a.lbase + kLanes * (int64_t)owner;
    const int32_t *tot = a.lbase + kLanes * (int64_t)R;
    const int32_t total_l = tot[0], leaf_l = tot[2], leafnodes_l = tot[4];
    if (L) {
        const int32_t rank = pl - lb[0];
        const int32_t lcount = (a.lbase + kLanes * (int64_t)(owner + 1))[0] - lb[0];
        if (lcount < LS) {
            const int64_t dst = (int64_t)upper + lb[2] + rank;
            a.fmin[dst] = lo;
            a.fmax[dst] = h;
        } else {
            const int64_t dst = (int64_t)(lb[0] - lb[2]) + rank;
            nmin[dst] = lo;
            nmax[dst] = make_float4(h.x, h.y, h.z, __int_as_float(owner - lb[4]));
        }
    }
    if (Rf) {
        const int32_t rank = pr - lb[1];
        const int32_t rcount = (a.lbase + kLanes * (int64_t)(owner + 1))[1] - lb[1];
        if (rcount < LS) {
            const int64_t dst = (int64_t)upper + leaf_l + lb[3] + rank;
            a.fmin[dst] = l;
            a.fmax[dst] = make_float4(hi.x, hi.y, hi.z, 0.0f);
        } else {
            const int64_t dst = (int64_t)(total_l - leaf_l) + (lb[1] - lb[3]) + rank;
            nmin[dst] = l;
            nmax[dst] = make_float4(hi.x, hi.y, hi.z, __int_as_float(R + owner - (leafnodes_l + lb[5])));
        }
    }
}

// Tight-box keys of a child's references: min corner in k[0..2], max corner
// in k[3..5]; neutral when the reference does not go to that child.
__device__ __forceinline__ void box_keys(bool in, const float4 &mn, const float4 &mx, unsigned (&k)[6])
{
    if (in) {
        k[0] = fkey(mn.x); k[1] = fkey(mn.y); k[2] = fkey(mn.z);
        k[3] = fkey(mx.x); k[4] = fkey(mx.y); k[5] = fkey(mx.z);
    } else {
        keys_neutral(k);
    }
}

__device__ __forceinline__ void keys_merge(unsigned (&acc)[6], const unsigned (&k)[6])
{
    acc[0] = min(acc[0], k[0]); acc[1] = min(acc[1], k[1]); acc[2] = min(acc[2], k[2]);
    acc[3] = max(acc[3], k[3]); acc[4] = max(acc[4], k[4]); acc[5] = max(acc[5], k[5]);
}

// Adds the reduced child keys of parent o to the next level's tight boxes:
// only non-leaf children are next-level nodes (local ids as in k_children).
// A neutral min key (no finite float maps to it) means no contribution.
__device__ __forceinline__ void child_keys_atomic(const BuildArgs &a, int32_t R, int o, const unsigned (&kl)[6],
                                                  const unsigned (&kr)[6])
{
    const int32_t *lb = a.lbase + kLanes * (int64_t)o, *nb = lb + kLanes;
    const int32_t *tot = a.lbase + kLanes * (int64_t)R;
    if (kl[0] != 0xffffffffu && nb[0] - lb[0] >= a.LS) keys_atomic(a.keys, o - lb[4], kl);
    if (kr[0] != 0xffffffffu && nb[1] - lb[1] >= a.LS) keys_atomic(a.keys, R + o - (tot[4] + lb[5]), kr);
}

// Partition + compaction of the references with clipping to the split plane
// (SplitTriangles, TriangleUpperChildren.h:283-383).  Destination = node base
// + rank of the reference among the node's left (right) references; a warp's
// first rank is its tile's offset plus the chunk totals of the tile's earlier
// warps.  The same pass reduces the next level's tight boxes (the segmented
// AABB reduction of ReduceSegments.h:230-371 for the children): references
// are sorted by parent, so a warp keeps running key minima/maxima while its
// rows belong to one parent and issues atomics only when the parent changes;
// the warps of a block merge equal parents before their atomics.
template <bool DIVIDE>
__global__ void __launch_bounds__(kBlock, DIVIDE ? 2 : 4) k_scatter(const BuildArgs a)
{
    __shared__ int s_owner[kWarps];
    __shared__ unsigned s_keys[kWarps][12];
    const BuildState *st = a.st;
    if (!level_fits(a, st, node_totals(a, st))) return;  // advance_upper records the failure
    const int64_t N = st->N;
    const int32_t R = st->R, active = st->active, upper = (int32_t)st->F;
    const int cur = st->level & 1;
    const float4 *__restrict__ cmin = a.rmin[cur];
    const float4 *__restrict__ cmax = a.rmax[cur];
    float4 *__restrict__ nmin = a.rmin[cur ^ 1];
    float4 *__restrict__ nmax = a.rmax[cur ^ 1];
    const unsigned lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const unsigned below = (1u << lane) - 1u;
    const int64_t ntiles = ceil_div(N, kTileRefs);
    for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const int64_t chunk = tile * kWarps + warp;
        const int64_t base = chunk * kChunk;
        // The warp's first ranks: its tile's offsets plus the chunk totals of
        // the tile's earlier warps (lane w < warp loads warp w's), so no warp
        // waits for another.
        int32_t off_l = 0, off_r = 0;
        {
            const int64_t ch = tile * kWarps + lane;
            if (lane < warp && ch * kChunk < N) {
                off_l = a.chunksum[2 * ch];
                off_r = a.chunksum[2 * ch + 1];
            }
            off_l = __reduce_add_sync(kFull, off_l) + a.tileoff[2 * tile];
            off_r = __reduce_add_sync(kFull, off_r) + a.tileoff[2 * tile + 1];
        }
        int run = -1;  // parent whose whole rows this warp is accumulating
        unsigned al[6], ar[6];
        keys_neutral(al);
        keys_neutral(ar);
        if (base < N) {  // warp-uniform
            float4 ra[kRows], rb[kRows];
#pragma unroll
            for (int row = 0; row < kRows; ++row) {
                const int64_t r = base + row * 32 + lane;
                if (r < N) { ra[row] = cmin[r]; rb[row] = cmax[r]; }
                else { ra[row] = make_float4(0.f, 0.f, 0.f, 0.f); rb[row] = make_float4(0.f, 0.f, 0.f, __int_as_float(-1)); }
            }
            int ax[kRows];
            float sps[kRows];
#pragma unroll
            for (int row = 0; row < kRows; ++row) {
                const int o = __float_as_int(rb[row].w);
                ax[row] = o >= 0 ? a.info[active + o] : 0;
                sps[row] = o >= 0 ? a.split[active + o] : 0.0f;
            }
#pragma unroll
            for (int row = 0; row < kRows; ++row) {
                if (base + row * 32 >= N) break;
                const int owner = __float_as_int(rb[row].w);
                const int axis = ax[row];
                const float sp = sps[row];
                const float4 lo = ra[row], hi = rb[row];
                int L = 0, Rf = 0;
                if (owner >= 0) ref_flags(lo, hi, axis, sp, L, Rf);
                if (DIVIDE && L && Rf) divide_flags(a, __float_as_int(lo.w), active + owner, axis, sp, L, Rf);
                const unsigned bl = __ballot_sync(kFull, L), br = __ballot_sync(kFull, Rf);
                const int32_t pl = off_l + __popc(bl & below), pr = off_r + __popc(br & below);
                off_l += __popc(bl);
                off_r += __popc(br);
                // Clipped boxes: the left child's max and the right child's min.
                const float4 h = make_float4(axis == KDGB_X ? kmin(sp, hi.x) : hi.x,
                                             axis == KDGB_Y ? kmin(sp, hi.y) : hi.y,
                                             axis == KDGB_Z ? kmin(sp, hi.z) : hi.z, 0.0f);
                const float4 l = make_float4(axis == KDGB_X ? kmax(sp, lo.x) : lo.x,
                                             axis == KDGB_Y ? kmax(sp, lo.y) : lo.y,
                                             axis == KDGB_Z ? kmax(sp, lo.z) : lo.z, lo.w);
                if (owner >= 0) scatter_one(a, R, owner, upper, L, Rf, lo, hi, h, l, pl, pr, nmin, nmax);
                unsigned kl[6], kr[6];
                box_keys(L, lo, h, kl);
                box_keys(Rf, l, hi, kr);
                const unsigned m = __match_any_sync(kFull, owner);
                if (m == kFull && owner == run) {
                    keys_merge(al, kl);
                    keys_merge(ar, kr);
                    continue;
                }
                // Parents do not decrease along the references, so a row that
                // leaves the run holds: the run's parent first (its lanes add
                // to the run before it is flushed), whole parents in between
                // (reduced and flushed here), and the row's last parent, which
                // starts the next run.
                if (run >= 0 && owner == run) {
                    keys_merge(al, kl);
                    keys_merge(ar, kr);
                }
                if (run >= 0) {
                    keys_reduce(kFull, al);
                    keys_reduce(kFull, ar);
                    if (lane == 0) child_keys_atomic(a, R, run, al, ar);
                }
                const int last = __shfl_sync(kFull, owner, 31);
                if (owner >= 0 && owner != run && owner != last) {
                    keys_reduce(m, kl);
                    keys_reduce(m, kr);
                    if (lane == (unsigned)(__ffs(m) - 1)) child_keys_atomic(a, R, owner, kl, kr);
                }
                run = last >= 0 && last != run ? last : -1;
                if (run >= 0 && owner == run) {
                    for (int j = 0; j < 6; ++j) { al[j] = kl[j]; ar[j] = kr[j]; }
                } else {
                    keys_neutral(al);
                    keys_neutral(ar);
                }
            }
            if (run >= 0) {
                keys_reduce(kFull, al);
                keys_reduce(kFull, ar);
            }
        }
        if (lane == 0) {
            s_owner[warp] = run;
            for (int j = 0; j < 6; ++j) { s_keys[warp][j] = al[j]; s_keys[warp][6 + j] = ar[j]; }
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            // Consecutive warps cover consecutive chunks: merge equal parents.
            int o = -1;
            unsigned kl[6], kr[6];
            keys_neutral(kl);
            keys_neutral(kr);
            for (int w = 0; w < kWarps; ++w) {
                const int ow = s_owner[w];
                if (ow < 0) continue;
                unsigned wl[6], wr[6];
                for (int j = 0; j < 6; ++j) { wl[j] = s_keys[w][j]; wr[j] = s_keys[w][6 + j]; }
                if (ow != o) {
                    if (o >= 0) child_keys_atomic(a, R, o, kl, kr);
                    o = ow;
                    for (int j = 0; j < 6; ++j) { kl[j] = wl[j]; kr[j] = wr[j]; }
                } else {
                    keys_merge(kl, wl);
                    keys_merge(kr, wr);
                }
            }
            if (o >= 0) child_keys_atomic(a, R, o, kl, kr);
        }
        __syncthreads();  // s_owner and s_keys are rewritten by the next tile
    }
}

// EmptySpaceSplitting2 (EmptySpaceSplitting.h:74-184): a chain of split
// nodes, each with an empty leaf, between the parent par0 and the active node
// `leaf` (box [mn, mx]).
__device__ __forceinline__ void ess_chain(const BuildArgs &a, int32_t leaf, int32_t start, int pl, int32_t par0,
                                          float4 mn, float4 mx)
{
    const int nn = 2 * __popc(pl);
    for (int j = 0; j < nn; ++j) ZERO_NODE(start + j);
    const int2 c = a.ch[par0];
    if (c.x == leaf) a.ch[par0].x = start;
    else a.ch[par0].y = start;
    int32_t par = start;
    const int8_t axes[3] = {KDGB_X, KDGB_Y, KDGB_Z};
    for (int b = 0; b < 3; ++b) {
        if (pl & (1 << b)) {
            pl -= (1 << b);
            a.info[par] = axes[b];
            a.split[par] = axis_of4(mn, axes[b]);
            const int32_t l = par + 1, r = pl ? l + 1 : leaf;
            a.ch[par] = make_int2(l, r);
            a.info[l] = KDGB_LEAF;
            a.amt[l] = 0;
            par = r;
        }
    }
    for (int b = 3; b < 5; ++b) {
        if (pl & (1 << b)) {
            pl -= (1 << b);
            a.info[par] = axes[b - 3];
            a.split[par] = axis_of4(mx, axes[b - 3]);
            const int32_t r = par + 1, l = pl ? r + 1 : leaf;
            a.ch[par] = make_int2(l, r);
            a.info[r] = KDGB_LEAF;
            a.amt[r] = 0;
            par = l;
        }
    }
    if (pl & 32) {
        a.info[par] = a.zmax_as_x ? (int8_t)KDGB_X : (int8_t)KDGB_Z;
        a.split[par] = a.zmax_as_x ? mx.x : mx.z;
        const int32_t r = par + 1;
        a.ch[par] = make_int2(leaf, r);
        a.info[r] = KDGB_LEAF;
        a.amt[r] = 0;
    }
}

// Called by every thread at the end of a level-closing kernel: true in one
// thread of the block that finishes last (all other blocks are done with the
// state then), which also resets the counter for the next level.
__device__ __forceinline__ bool last_block(BuildState *st)
{
    __shared__ bool s_last;
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        s_last = atomicAdd(&st->done, 1) == (int)gridDim.x - 1;
        if (s_last) st->done = 0;
    }
    __syncthreads();
    return s_last && threadIdx.x == 0;
}

// End of an upper level (run by one thread of the level's last block):
// records the level's leaf range, advances the counters to the next level
// and decides whether the loop continues.
__device__ void advance_upper(const BuildArgs &a, BuildState *st)
{
    int more = 0;
    do {
        if (st->err) break;
        if (st->nonfinite) { set_err(st, KDGB_ERR_NONFINITE, kErrNonfinite); break; }
        const int32_t R = st->R;
        const int32_t *tot = node_totals(a, st);
        if (!level_fits(a, st, tot)) { set_err(st, KDGB_ERR_CAPACITY, kErrUpperCapacity); break; }
        const int32_t leaf_nodes = tot[4] + tot[5];
        if (leaf_nodes > 0 && (st->n_ranges >= a.cap.ranges || (int64_t)st->n_leaf_ids + leaf_nodes > a.cap.leaves)) {
            set_err(st, KDGB_ERR_CAPACITY, kErrLeafCapacity);
            break;
        }
        const int64_t tl = tot[0], tr = tot[1], ll = tot[2], lr = tot[3];
        // Box sides keep every reference; DIVIDE may drop references whose
        // triangle misses the node box.
        if (!a.divide && tl + tr < st->N) { set_err(st, KDGB_ERR_DEGENERATE, kErrFewerRefs); break; }
        const int32_t empty = tot[6];
        if (leaf_nodes > 0) {
            a.ranges[st->n_ranges] = make_int2(st->n_nodes + empty, leaf_nodes);
            a.roff[st->n_ranges] = st->n_leaf_ids;
            st->n_ranges += 1;
            st->n_leaf_ids += leaf_nodes;
        }
        st->n_nodes += empty + 2 * R;
        st->F += ll + lr;
        const int32_t created = 2 * R - leaf_nodes;
        st->N = tl + tr - ll - lr;
        st->ntiles = (int32_t)ceil_div(st->N, kTileRefs);
        st->active = st->n_nodes - created;
        st->R = created;
        st->level += 1;
        if (created > 0 && st->level >= a.max_levels) { set_err(st, KDGB_ERR_DEGENERATE, kErrMaxLevels); break; }
        more = created > 0;
    } while (0);
    if (a.use_cond) cudaGraphSetConditional(a.upper_cond, more ? 1u : 0u);
}

// CreateUpperChildren (TriangleUpperChildren.h:203-281), the empty-space
// chain of EmptySpaceSplitting2 (its nodes come first, at base + lane-6
// offsets) and, with empty-space splitting on, PropagateAabbToChildren
// (EmptySpaceSplitting.h:299-331; TriangleMapUpperCreator.cu:731-733 runs
// it whenever empty-space splitting is on, whatever propagateAabbs says).
// Non-leaf children are the next level's active nodes: their counts are
// reset and their splits made here (node_split_one against the propagated
// box; their tight-box keys were reset by k_count and filled by k_scatter),
// so the next level starts with its counting pass.  The block that finishes
// last closes the level (advance_upper).
__global__ void k_children(const BuildArgs a)
{
    BuildState *st = a.st;
    const int32_t *tot = node_totals(a, st);
    const bool fits = level_fits(a, st, tot);  // when not, advance_upper records the failure
    const int32_t R = fits ? st->R : 0, active = st->active, base = st->n_nodes, upper = (int32_t)st->F;
    const int32_t LS = a.LS;
    const bool ess = do_ess(a, st);
    // The next level: never the root level, a binned-SAH level once
    // upper_levels are done.
    const bool sah_next = a.tuned && st->level + 2 > a.upper_levels;
    const int cur = st->level & 1;
    const int8_t *planes = a.planes[cur];
    int8_t *planes_next = a.planes[cur ^ 1];
    int32_t *ess_next = a.ess_cnt[cur ^ 1];
    const int32_t empty = tot[6];
    const int32_t child_start = base + empty;
    const int32_t total_l = tot[0], leaf_l = tot[2], ln_l = tot[4], leaf_nodes = tot[4] + tot[5];
    // Two threads per active node, one per child: the dependent chain of
    // node-record loads and stores is halved, which is what bounds the deep
    // levels (few nodes, latency-bound).  The left thread also links the
    // children and builds the node's empty-space chain.
    GRID_STRIDE(i64, 2 * (int64_t)R) {
        const int32_t k = (int32_t)(i64 >> 1);
        const bool right = i64 & 1;
        const int32_t *lb = a.lbase + kLanes * (int64_t)k;
        const int32_t *nb = a.lbase + kLanes * (int64_t)(k + 1);
        const int32_t par = active + k;
        // Every load that depends only on the node is issued before the
        // first store, so that they are in flight together.
        const int32_t lb0 = lb[0], lb1 = lb[1], lb2 = lb[2], lb3 = lb[3], lb4 = lb[4], lb5 = lb[5], lb6 = lb[6];
        const int32_t nb0 = nb[0], nb1 = nb[1];
        const bool chain = !right && ess;
        const int pl = chain ? planes[k] : 0;
        const int32_t par0 = chain ? a.parent[par] : 0;
        int axis = 0;
        float sp = 0.0f;
        float4 mn = make_float4(0.f, 0.f, 0.f, 0.f), mx = mn;
        if (a.ess) {
            axis = a.info[par] & 3;
            sp = a.split[par];
            mn = a.bmin[par];
            mx = a.bmax[par];
        }
        const int32_t la = lb4, ra = ln_l + lb5;
        const int32_t l = nb0 - lb0, r = nb1 - lb1;
        const bool lleaf = l < LS, rleaf = r < LS;
        const int32_t lnext = k - la, rnext = (R + k) - ra;
        const int32_t lid = child_start + (lleaf ? la : lnext + leaf_nodes);
        const int32_t rid = child_start + (rleaf ? ra : rnext + leaf_nodes);
        if (!right) {
            if (pl) ess_chain(a, par, base + lb6, pl, par0, mn, mx);
            a.ch[par] = make_int2(lid, rid);
        }
        const int32_t id = right ? rid : lid;
        const bool leaf = right ? rleaf : lleaf;
        const int32_t next = right ? rnext : lnext;
        ZERO_NODE(id);
        a.pidx[id] = right ? (rleaf ? upper + leaf_l + lb3 : (total_l - leaf_l) + (lb1 - lb3))
                           : (lleaf ? upper + lb2 : lb0 - lb2);
        a.amt[id] = right ? r : l;
        a.parent[id] = par;
        float4 cmin = make_float4(0.f, 0.f, 0.f, 0.f), cmax = cmin;
        if (a.ess) {  // PropagateAabbToChildren runs with empty-space splitting
            if (right) {
                cmin = make_float4(axis == KDGB_X ? sp : mn.x, axis == KDGB_Y ? sp : mn.y, axis == KDGB_Z ? sp : mn.z,
                                   0.0f);
                cmax = mx;
            } else {
                cmin = mn;
                cmax = make_float4(axis == KDGB_X ? sp : mx.x, axis == KDGB_Y ? sp : mx.y, axis == KDGB_Z ? sp : mx.z,
                                   0.0f);
            }
            a.bmin[id] = cmin;
            a.bmax[id] = cmax;
        }
        if (!leaf) {
            a.cnt[2 * next] = 0;
            a.cnt[2 * next + 1] = 0;
            node_split_one(a, next, id, a.ess, cmin, cmax, sah_next, planes_next, ess_next);
        }
    }
    if (last_block(st)) advance_upper(a, st);
}

// MarkLeafNodes (TriangleUpperChildren.h:385-395) over all levels at once:
// each level appended a contiguous range of leaf node ids.
__device__ __forceinline__ int32_t upper_leaf_id(const BuildArgs &a, int32_t nr, int32_t i)
{
    int lo = 0, hi = nr - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (a.roff[mid] <= i) lo = mid; else hi = mid - 1;
    }
    return a.ranges[lo].x + (i - a.roff[lo]);
}

__global__ void k_leaf_ids(const BuildArgs a)
{
    const BuildState *st = a.st;
    if (st->err) return;
    const int32_t total = st->n_leaf_ids, nr = st->n_ranges;
    GRID_STRIDE(ii, total) a.leaf_ids[ii] = upper_leaf_id(a, nr, (int32_t)ii);
}

// ExtractIndexFromAabb (TriangleUpper.h:43-52).
__global__ void k_extract_indices(const BuildArgs a)
{
    const BuildState *st = a.st;
    if (st->err) return;
    GRID_STRIDE(i, st->F) a.prim_indices[i] = __float_as_int(a.fmin[i].w);
}

// PropagateParentAabb<true> (EmptySpaceSplitting.h:333-368).
__global__ void k_propagate_parent(const BuildArgs a)
{
    const BuildState *st = a.st;
    if (st->err) return;
    GRID_STRIDE(i, st->n_leaf_ids) {
        const int32_t c = a.leaf_ids[i];
        const int32_t par = a.parent[c];
        const float4 mn = a.bmin[par], mx = a.bmax[par];
        const int axis = a.info[par] & 3;
        const float sp = a.split[par];
        if (a.ch[par].x == c) {
            a.bmin[c] = make_float4(mn.x, mn.y, mn.z, 0.0f);
            a.bmax[c] = make_float4(axis == KDGB_X ? sp : mx.x, axis == KDGB_Y ? sp : mx.y,
                                    axis == KDGB_Z ? sp : mx.z, 0.0f);
        } else {
            a.bmin[c] = make_float4(axis == KDGB_X ? sp : mn.x, axis == KDGB_Y ? sp : mn.y,
                                    axis == KDGB_Z ? sp : mn.z, 0.0f);
            a.bmax[c] = make_float4(mx.x, mx.y, mx.z, 0.0f);
        }
    }
}

// PreprocessLeafNodes of the BITMAP creator (TriangleMapBitmapCreator.cu:32-49).
__global__ void k_bitmap_leaves(const BuildArgs a)
{
    const BuildState *st = a.st;
    if (st->err) return;
    GRID_STRIDE(i, st->n_leaf_ids) {
        const int32_t leaf = a.leaf_ids[i];
        a.info[leaf] = KDGB_LEAF;
        a.amt[leaf] = (int32_t)((1u << a.amt[leaf]) - 1u);
    }
}

// ---------------------------------------------------------------------------
// Reference SAH lower creator (LowerTriangleMap.h).
// ---------------------------------------------------------------------------

// CalcSurfaceArea (LowerTriangleMap.h:24-38): 0.5 * |e1 x e2|.
// ExtractIndexFromAabb as k_extract_indices does, and each leaf reference's
// triangle area (the SAH lower creator's CalcArea).
__global__ void k_areas(const BuildArgs a)
{
    const BuildState *st = a.st;
    if (st->err) return;
    GRID_STRIDE(i, st->F) {
        const int32_t prim = __float_as_int(a.fmin[i].w);
        a.prim_indices[i] = prim;
        const float4 q = __ldg(a.prec + 3 * (int64_t)prim), r = __ldg(a.prec + 3 * (int64_t)prim + 1),
                     w = __ldg(a.prec + 3 * (int64_t)prim + 2);
        // e1 = v1 - v0 and e2 = v2 - v0 as k_load_geometry rounded them.
        const float3 cr = cross3(make_float3(q.w, r.x, r.y), make_float3(r.z, r.w, w.x));
        a.areas[i] = __fmul_rn(0.5f, __fsqrt_rn(dot3(cr, cr)));
    }
}

// PreprocesLowerNodes (LowerTriangleMap.h:56-81): node area and the bitmap of
// references with non-zero area.
// MarkLeafNodes as k_leaf_ids does, and each upper leaf's area sum and
// bitmap of references with a nonzero area (PreprocessLeafNodes).
__global__ void k_sah_preprocess(const BuildArgs a)
{
    const BuildState *st = a.st;
    if (st->err) return;
    const int32_t nr = st->n_ranges;
    GRID_STRIDE(k, st->n_leaf_ids) {
        const int32_t leaf = upper_leaf_id(a, nr, (int32_t)k);
        a.leaf_ids[k] = leaf;
        const int32_t pi = a.pidx[leaf], n = a.amt[leaf];
        float s = 0.0f;
        unsigned bmp = 0;
        for (int i = 0; i < n; ++i) {
            const float ar = a.areas[pi + i];
            bmp += ar > 0.0f ? (1u << i) : 0u;
            s = __fadd_rn(s, ar);
        }
        a.area[leaf] = s;
        a.amt[leaf] = (int32_t)bmp;
    }
}

// The first SAH lower level is the set of upper leaves.
__global__ void k_lower_begin(const BuildArgs a)
{
    BuildState *st = a.st;
    st->low_levels = 0;
    st->low_active = 0;
    st->low_first = 1;
    st->low_R = 0;
    st->low_n[0][0] = st->low_n[0][1] = st->low_n[1][0] = st->low_n[1][1] = 0;
    if (st->err) return;
    if ((int64_t)st->n_leaf_ids > a.cap.low_R) {
        set_err(st, KDGB_ERR_CAPACITY, kErrLowerCapacity);
        return;
    }
    st->low_R = st->n_leaf_ids;
}

struct SahPick {
    float cost, la, ra;
    unsigned ls, rs;
    int axis;
    int32_t idx;
};

// CalcAreaForSets (LowerTriangleMap.h:412-461) for the planes of one slot:
// ar[0..3] are the area sums of the four sets (accumulated in bit order by
// the caller); low and high plane costs are tried in the reference's order.
__device__ __forceinline__ void pick_planes(const unsigned (&s)[4], const float (&ar)[4], int axis, int32_t set_index,
                                            SahPick &best)
{
    const float low = __fadd_rn(__fmul_rn((float)__popc(s[0]), ar[0]), __fmul_rn((float)__popc(s[1]), ar[1]));
    const float high = __fadd_rn(__fmul_rn((float)__popc(s[2]), ar[2]), __fmul_rn((float)__popc(s[3]), ar[3]));
    if (low < best.cost) {
        best.cost = low; best.ls = s[0]; best.rs = s[1]; best.la = ar[0]; best.ra = ar[1];
        best.axis = axis; best.idx = set_index;
    }
    if (high < best.cost) {
        best.cost = high; best.ls = s[2]; best.rs = s[3]; best.la = ar[2]; best.ra = ar[3];
        best.axis = axis; best.idx = (int32_t)((unsigned)set_index | 0x80000000u);
    }
}

// Predicated set updates of the SAH plane passes, written as one compare (or
// bit test) feeding predicated instructions: acc += aj when bit m of s is
// set; s |= m and acc += aj when x <= y (x < y).  The additions are IEEE
// round-to-nearest single additions, as __fadd_rn.
__device__ __forceinline__ void add_if_bit(float &acc, unsigned s, unsigned m, float aj)
{
    asm("{\n\t.reg .pred p;\n\t.reg .b32 t;\n\tand.b32 t, %1, %2;\n\tsetp.ne.u32 p, t, 0;\n\t"
        "@p add.rn.f32 %0, %0, %3;\n\t}"
        : "+f"(acc)
        : "r"(s), "r"(m), "f"(aj));
}

__device__ __forceinline__ void set_le(unsigned &s, float &acc, float x, float y, unsigned m, float aj)
{
    asm("{\n\t.reg .pred p;\n\tsetp.le.f32 p, %2, %3;\n\t@p or.b32 %0, %0, %4;\n\t@p add.rn.f32 %1, %1, %5;\n\t}"
        : "+r"(s), "+f"(acc)
        : "f"(x), "f"(y), "r"(m), "f"(aj));
}

__device__ __forceinline__ void set_lt(unsigned &s, float &acc, float x, float y, unsigned m, float aj)
{
    asm("{\n\t.reg .pred p;\n\tsetp.lt.f32 p, %2, %3;\n\t@p or.b32 %0, %0, %4;\n\t@p add.rn.f32 %1, %1, %5;\n\t}"
        : "+r"(s), "+f"(acc)
        : "f"(x), "f"(y), "r"(m), "f"(aj));
}

// The split decision of one lower node (CalcSAH, LowerTriangleMap.h:463-555) from the candidates of a group
// of W lanes (the whole warp or one half): lane r of the group holds the best of its own six planes (mb, valid
// when `mine`), lanes in slot order.  The first minimum in (slot, axis, low/high) order wins; one lane of the
// group writes the decision.  A group with bmp == 0 holds no node and writes nothing.
template <int W>
__device__ __forceinline__ void sah_decide(const BuildArgs &a, int64_t gw, int32_t par, unsigned bmp, int lane,
                                           bool mine, const SahPick &mb, int32_t *tcnt)
{
    const int r = lane & (W - 1);
    // Group argmin on (cost, lane); only lanes whose cost beat fInfinity count.
    float c = mine && mb.cost < KDGB_FINF ? mb.cost : INFINITY;
    int owner = mine && mb.cost < KDGB_FINF ? r : W;
#pragma unroll
    for (int o = W / 2; o > 0; o >>= 1) {
        const float c2 = __shfl_xor_sync(kFull, c, o);
        const int w2 = __shfl_xor_sync(kFull, owner, o);
        if (c2 < c || (c2 == c && w2 < owner)) { c = c2; owner = w2; }
    }
    if (bmp != 0u && r == (owner < W ? owner : 0)) {
        const int cnt = __popc(bmp);
        const float ct = a.ct, ci = a.ci;
        const float opt = owner < W ? mb.cost : KDGB_FINF;
        const float node_area = a.area[par];
        bool split_it = __fmul_rn(ci, opt) < __fmul_rn(__fsub_rn(__fmul_rn(ci, (float)cnt), ct), node_area);
        if (cnt <= a.min_leaf) split_it = false;
        if (split_it) {
            a.careas[gw] = make_float2(mb.la, mb.ra);
            a.csets[gw] = make_int2((int)mb.ls, (int)mb.rs);
            const float4 sp4 = ((unsigned)mb.idx & 0x80000000u) ? a.fmax[(unsigned)mb.idx ^ 0x80000000u]
                                                                 : a.fmin[mb.idx];
            a.split[par] = axis_of4(sp4, mb.axis);
        }
        a.info[par] = split_it ? (int8_t)mb.axis : (int8_t)KDGB_LEAF;
        a.ssplit[gw] = split_it;
        if (split_it) atomicAdd(tcnt + gw / kLowTile, 1);
    }
}

__device__ __forceinline__ void sah_pick_init(SahPick &mb)
{
    mb.cost = KDGB_FINF; mb.la = mb.ra = 0.0f; mb.ls = mb.rs = 0; mb.axis = 0; mb.idx = 0;
}

// Bit position of the r-th (from 0) set bit of m, r < popc(m): the largest p
// with fewer than r + 1 set bits below it.
__device__ __forceinline__ int nth_bit(unsigned m, int r)
{
    int pos = 0;
#pragma unroll
    for (int s = 16; s > 0; s >>= 1)
        if (__popc(m & ((1u << (pos + s)) - 1u)) <= r) pos += s;
    return pos;
}

// The plane costs of one lower node by a group of W lanes (a whole warp, or
// a half warp for a node of at most 16 members, so that one warp evaluates
// two such nodes at once): lane r of the group takes the node's r-th member
// in bit order (slot nth_bit(bmp, r)) with its sets {lowLeft, lowRight,
// highLeft, highRight} per axis, and sums the member areas of all twelve
// sets in one pass over the members in bit order.  Only members are added
// (predicated adds: skipping a +0 term is exact), so every sum equals the
// reference's bit-order accumulation (CalcAreaForSets,
// LowerTriangleMap.h:412-461).  Both halves of a warp run the same number of
// steps (the larger member count); a half without a node has bmp == 0.
template <int W>
__device__ __forceinline__ void sah_eval_group(const BuildArgs &a, int64_t gw, int32_t par, int32_t pi, unsigned bmp,
                                               int lane, int64_t F, int32_t *tcnt)
{
    const int r = lane & (W - 1);
    const int cnt = __popc(bmp);
    const bool mine = r < cnt;
    const int slot = mine ? nth_bit(bmp, r) : 0;
    int4 sx = make_int4(0, 0, 0, 0), sy = sx, sz = sx;
    float a_lane = 0.0f;
    if (mine) {
        sx = a.sts[pi + slot];
        sy = a.sts[F + pi + slot];
        sz = a.sts[2 * F + pi + slot];
        a_lane = a.areas[pi + slot];
    }
    const unsigned sets[3][4] = {
        {(unsigned)sx.x & bmp, (unsigned)sx.y & bmp, (unsigned)sx.z & bmp, (unsigned)sx.w & bmp},
        {(unsigned)sy.x & bmp, (unsigned)sy.y & bmp, (unsigned)sy.z & bmp, (unsigned)sy.w & bmp},
        {(unsigned)sz.x & bmp, (unsigned)sz.y & bmp, (unsigned)sz.z & bmp, (unsigned)sz.w & bmp}};
    float ar[3][4] = {{0.f, 0.f, 0.f, 0.f}, {0.f, 0.f, 0.f, 0.f}, {0.f, 0.f, 0.f, 0.f}};
    int steps = cnt;
    if (W < 32) steps = max(steps, __shfl_xor_sync(kFull, steps, 16));
    const int base = lane & ~(W - 1);
    unsigned bits = bmp;
    for (int t = 0; t < steps; ++t) {  // steps is warp-uniform
        const unsigned m = bits & (0u - bits);  // the t-th member's bit (0 past the last member)
        bits ^= m;
        const float aj = __shfl_sync(kFull, a_lane, base | t);
#pragma unroll
        for (int x = 0; x < 3; ++x)
#pragma unroll
            for (int c = 0; c < 4; ++c) add_if_bit(ar[x][c], sets[x][c], m, aj);
    }
    SahPick mb;
    sah_pick_init(mb);
    pick_planes(sets[0], ar[0], KDGB_X, pi + slot, mb);
    pick_planes(sets[1], ar[1], KDGB_Y, pi + slot, mb);
    pick_planes(sets[2], ar[2], KDGB_Z, pi + slot, mb);
    sah_decide<W>(a, gw, par, bmp, lane, mine, mb, tcnt);
}

// CreateSplittingPlanes (LowerTriangleMap.h:84-155): one warp per node, lane
// i owns reference slot i.  Sets per axis: {lowLeft, lowRight, highLeft,
// highRight} of the planes at slot i's box low / high.
// The members' boxes are staged in shared memory in bit order (entry r is
// the r-th member: its box, its bit in the w of the min corner and its area
// in the w of the max corner) and read back as broadcasts, four members per
// step, so each member costs two loads.  With the SAH creator the warp also
// evaluates the first lower level's plane costs for its node (k_calc_sah
// does the later levels): the area sums of the twelve sets are accumulated
// in the same pass over the members, in bit order, as each set bit is found.
__global__ void __launch_bounds__(kBlock, 4) k_sah_planes(const BuildArgs a)
{
    // Entries past the last member (up to three) are sentinels: an empty box
    // that no plane test accepts, bit 0.
    __shared__ float4 s_lo[kWarps][36], s_hi[kWarps][36];
    const BuildState *st = a.st;
    if (st->err) return;
    const int64_t F = st->F;
    const int lane = threadIdx.x & 31, warp = (threadIdx.x >> 5) & (kWarps - 1);
    const unsigned below = (1u << lane) - 1u;
    // With the SAH lower creator the warp also evaluates the node's planes
    // (the first lower level; k_lower_begin checks the same capacity).
    const bool first_sah = a.lower == KDGB_LOWER_SAH && (int64_t)st->n_leaf_ids <= a.cap.low_R;
    WARP_STRIDE(gw, st->n_leaf_ids) {
        const int32_t leaf = a.leaf_ids[gw];
        const int32_t pi = a.pidx[leaf];
        const unsigned bmp = (unsigned)a.amt[leaf];
        const int cnt = __popc(bmp);
        const bool mine = (bmp >> lane) & 1u;
        const bool eval = first_sah && cnt > a.min_leaf;  // warp-uniform
        float4 lo = make_float4(0.f, 0.f, 0.f, 0.f), hi = lo;
        if (mine) {
            lo = a.fmin[pi + lane];
            hi = a.fmax[pi + lane];
            const int r = __popc(bmp & below);
            s_lo[warp][r] = make_float4(lo.x, lo.y, lo.z, __uint_as_float(1u << lane));
            s_hi[warp][r] = make_float4(hi.x, hi.y, hi.z, eval ? a.areas[pi + lane] : 0.0f);
        }
        if (lane < 4) {
            s_lo[warp][cnt + lane] = make_float4(INFINITY, INFINITY, INFINITY, __uint_as_float(0u));
            s_hi[warp][cnt + lane] = make_float4(-INFINITY, -INFINITY, -INFINITY, 0.0f);
        }
        __syncwarp();
        unsigned sx[4] = {0, 0, 0, 0}, sy[4] = {0, 0, 0, 0}, sz[4] = {0, 0, 0, 0};
        if (eval) {
            float ar[3][4] = {{0.f, 0.f, 0.f, 0.f}, {0.f, 0.f, 0.f, 0.f}, {0.f, 0.f, 0.f, 0.f}};
            for (int t = 0; t < cnt; t += 4) {  // cnt is warp-uniform; four members per step
                float4 mn[4], mx[4];
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    mn[q] = s_lo[warp][t + q];
                    mx[q] = s_hi[warp][t + q];
                }
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    const unsigned m = __float_as_uint(mn[q].w);
                    const float aj = mx[q].w;
                    set_le(sx[0], ar[0][0], mn[q].x, lo.x, m, aj);
                    set_lt(sx[1], ar[0][1], lo.x, mx[q].x, m, aj);
                    set_le(sx[2], ar[0][2], mn[q].x, hi.x, m, aj);
                    set_lt(sx[3], ar[0][3], hi.x, mx[q].x, m, aj);
                    set_le(sy[0], ar[1][0], mn[q].y, lo.y, m, aj);
                    set_lt(sy[1], ar[1][1], lo.y, mx[q].y, m, aj);
                    set_le(sy[2], ar[1][2], mn[q].y, hi.y, m, aj);
                    set_lt(sy[3], ar[1][3], hi.y, mx[q].y, m, aj);
                    set_le(sz[0], ar[2][0], mn[q].z, lo.z, m, aj);
                    set_lt(sz[1], ar[2][1], lo.z, mx[q].z, m, aj);
                    set_le(sz[2], ar[2][2], mn[q].z, hi.z, m, aj);
                    set_lt(sz[3], ar[2][3], hi.z, mx[q].z, m, aj);
                }
            }
            SahPick mb;
            sah_pick_init(mb);
            pick_planes(sx, ar[0], KDGB_X, pi + lane, mb);
            pick_planes(sy, ar[1], KDGB_Y, pi + lane, mb);
            pick_planes(sz, ar[2], KDGB_Z, pi + lane, mb);
            sah_decide<32>(a, gw, leaf, bmp, lane, mine, mb, a.lcnt[0]);
        } else {
            for (int t = 0; t < cnt; t += 4) {  // cnt is warp-uniform; four members per step
                float4 mn[4], mx[4];
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    mn[q] = s_lo[warp][t + q];
                    mx[q] = s_hi[warp][t + q];
                }
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    const unsigned m = __float_as_uint(mn[q].w);
                    sx[0] |= mn[q].x <= lo.x ? m : 0; sx[1] |= lo.x < mx[q].x ? m : 0;
                    sx[2] |= mn[q].x <= hi.x ? m : 0; sx[3] |= hi.x < mx[q].x ? m : 0;
                    sy[0] |= mn[q].y <= lo.y ? m : 0; sy[1] |= lo.y < mx[q].y ? m : 0;
                    sy[2] |= mn[q].y <= hi.y ? m : 0; sy[3] |= hi.y < mx[q].y ? m : 0;
                    sz[0] |= mn[q].z <= lo.z ? m : 0; sz[1] |= lo.z < mx[q].z ? m : 0;
                    sz[2] |= mn[q].z <= hi.z ? m : 0; sz[3] |= hi.z < mx[q].z ? m : 0;
                }
            }
            if (first_sah && lane == 0) {  // never split: no plane costs
                a.info[leaf] = (int8_t)KDGB_LEAF;
                a.ssplit[gw] = 0;
            }
        }
        if (mine) {
            a.sts[pi + lane] = make_int4(sx[0], sx[1], sx[2], sx[3]);
            a.sts[F + pi + lane] = make_int4(sy[0], sy[1], sy[2], sy[3]);
            a.sts[2 * F + pi + lane] = make_int4(sz[0], sz[1], sz[2], sz[3]);
        }
        __syncwarp();  // the staged boxes are rewritten by the warp's next node
    }
}

// CalcSAH (LowerTriangleMap.h:463-555) for the later lower levels (the
// first, the upper leaves, is evaluated by k_sah_planes).  Nodes with too
// few members to split are decided one thread each (no plane costs).  The
// others were listed by the level before (k_sah_children): the warps take
// them from the lists, two at a time (one per half warp) from the list of
// nodes of at most 16 members, then one at a time.  The grid is at most one
// resident wave, so every warp takes about as many list items as any other.
__global__ void k_calc_sah(const BuildArgs a)
{
    BuildState *st = a.st;
    if (st->err || st->low_first) return;
    const int32_t R = st->low_R, active = st->low_active;
    const int64_t F = st->F;
    const int b = st->low_levels & 1;
    // k_sah_children of this level lists the next level's nodes in the other
    // parity's lists.
    if (blockIdx.x == 0 && threadIdx.x == 0) st->low_n[b ^ 1][0] = st->low_n[b ^ 1][1] = 0;
    GRID_STRIDE(k64, R) {
        const int32_t k = (int32_t)k64;
        if (__popc((unsigned)a.amt[active + k]) <= a.min_leaf) {
            a.info[active + k] = (int8_t)KDGB_LEAF;
            a.ssplit[k] = 0;
        }
    }
    const int32_t ns = st->low_n[b][0], nb = st->low_n[b][1];
    const int32_t *__restrict__ list = a.lowlist[b];
    const int64_t cap = a.cap.list[b];
    const int64_t pairs = ((int64_t)ns + 1) / 2;
    const int lane = threadIdx.x & 31;
    WARP_STRIDE(it, pairs + nb) {
        if (it < pairs) {  // warp-uniform
            const bool two = 2 * it + 1 < ns;
            const int32_t k = list[lane < 16 || !two ? 2 * it : 2 * it + 1];
            unsigned bmp = (unsigned)a.amt[active + k];
            const int32_t pi = a.pidx[active + k];
            if (lane >= 16 && !two) bmp = 0u;  // no second node: the upper half idles
            sah_eval_group<16>(a, k, active + k, pi, bmp, lane, F, a.lcnt[b]);
        } else {
            const int32_t k = list[cap - 1 - (it - pairs)];
            sah_eval_group<32>(a, k, active + k, a.pidx[active + k], (unsigned)a.amt[active + k], lane, F, a.lcnt[b]);
        }
    }
}

// Balanced ("SSAH") lower creator: CalcSplit (LowerTriangleMap.h:299-369)
// with CalcRelationForSets (:260-295), one warp per node.  Lane i weighs the
// six planes of slot i by small^2 + large^2 of the two set sizes (integers,
// so the order of evaluation cannot change the result); the warp keeps the
// first minimum in (slot, axis, low/high) order, the reference's running
// strict minimum from 32 * 32.  A node of n references splits when
// (traversal_cost + weight) / n < n and a plane was found.  Children carry
// no area (the creator never writes one).
constexpr int kNoPlane = 32 * 32;

__global__ void k_calc_balanced(const BuildArgs a)
{
    const BuildState *st = a.st;
    if (st->err) return;
    const int32_t R = st->low_R, active = st->low_active;
    const int32_t *__restrict__ ids = st->low_first ? a.leaf_ids : nullptr;
    const int64_t F = st->F;
    const int lane = threadIdx.x & 31;
    WARP_STRIDE(gw, R) {
        const int32_t par = ids ? ids[gw] : active + (int32_t)gw;
        const int32_t pi = a.pidx[par];
        const unsigned bmp = (unsigned)a.amt[par];
        int best = kNoPlane, axis = 0, high = 0;
        unsigned ls = 0, rs = 0;
        if ((bmp >> lane) & 1u) {
#pragma unroll
            for (int x = 0; x < 3; ++x) {
                const int4 s4 = a.sts[x * F + pi + lane];
                const unsigned s[4] = {(unsigned)s4.x & bmp, (unsigned)s4.y & bmp, (unsigned)s4.z & bmp,
                                       (unsigned)s4.w & bmp};
#pragma unroll
                for (int h = 0; h < 2; ++h) {
                    const int c0 = __popc(s[2 * h]), c1 = __popc(s[2 * h + 1]);
                    const int w = c0 * c0 + c1 * c1;
                    if (w < best) { best = w; ls = s[2 * h]; rs = s[2 * h + 1]; axis = x + 1; high = h; }
                }
            }
        }
        int c = best, owner = lane;
        for (int o = 16; o > 0; o >>= 1) {
            const int c2 = __shfl_xor_sync(kFull, c, o);
            const int w2 = __shfl_xor_sync(kFull, owner, o);
            if (c2 < c || (c2 == c && w2 < owner)) { c = c2; owner = w2; }
        }
        if (lane == owner) {
            const float n = (float)__popc(bmp);
            const float ssah = __fdiv_rn(__fadd_rn(a.ct, (float)best), n);
            const bool split_it = best < kNoPlane && ssah < n;
            if (split_it) {
                a.careas[gw] = make_float2(0.0f, 0.0f);
                a.csets[gw] = make_int2((int)ls, (int)rs);
                const float4 sp4 = high ? a.fmax[pi + lane] : a.fmin[pi + lane];
                a.split[par] = axis_of4(sp4, axis);
            }
            a.info[par] = split_it ? (int8_t)axis : (int8_t)KDGB_LEAF;
            a.ssplit[gw] = split_it;
            if (split_it) atomicAdd(a.lcnt[st->low_levels & 1] + gw / kLowTile, 1);
        }
    }
}

__device__ __forceinline__ bool lower_fits(const BuildArgs &a, const BuildState *st, int32_t splits)
{
    return (int64_t)st->n_nodes + 2 * (int64_t)splits <= a.cap.nodes;
}

// End of a SAH lower level (one thread of the level's last block).
__device__ void advance_lower(const BuildArgs &a, BuildState *st, int32_t splits)
{
    int more = 0;
    do {
        if (st->err) break;
        const int32_t R = st->low_R;
        if (R == 0) break;
        if (!lower_fits(a, st, splits) || 2 * (int64_t)splits > a.cap.low_R ||
            (a.lower == KDGB_LOWER_SAH && 2 * (int64_t)splits > a.cap.list[(st->low_levels + 1) & 1])) {
            set_err(st, KDGB_ERR_CAPACITY, kErrLowerCapacity);
            break;
        }
        st->low_levels += 1;
        st->n_nodes += 2 * splits;
        st->low_active = st->n_nodes - 2 * splits;
        st->low_R = 2 * splits;
        st->low_first = 0;
        more = splits > 0;
    } while (0);
    if (a.use_cond) cudaGraphSetConditional(a.lower_cond, more ? 1u : 0u);
}

// Appends the next-level positions of this block's children that are to be
// evaluated (pl / pr, with sl / sr when they have at most 16 members) to the
// SAH work lists of the next level: small nodes from the front of the list,
// larger ones from its end.  One global atomic per list and block; every
// thread of the block calls it.
__device__ __forceinline__ void lower_list_push(const BuildArgs &a, BuildState *st, int nb, bool pl, bool sl,
                                                int32_t ql, bool pr, bool sr, int32_t qr)
{
    __shared__ int32_t s_n[2], s_base[2];
    const unsigned lane = threadIdx.x & 31;
    const unsigned m0 = __ballot_sync(kFull, pl && sl), m1 = __ballot_sync(kFull, pl && !sl);
    const unsigned m2 = __ballot_sync(kFull, pr && sr), m3 = __ballot_sync(kFull, pr && !sr);
    if (threadIdx.x == 0) s_n[0] = s_n[1] = 0;
    __syncthreads();
    int32_t ws = 0, wb = 0;
    if (lane == 0) {
        const int cs = __popc(m0) + __popc(m2), cb = __popc(m1) + __popc(m3);
        if (cs) ws = atomicAdd(&s_n[0], cs);
        if (cb) wb = atomicAdd(&s_n[1], cb);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        s_base[0] = s_n[0] ? atomicAdd(&st->low_n[nb][0], s_n[0]) : 0;
        s_base[1] = s_n[1] ? atomicAdd(&st->low_n[nb][1], s_n[1]) : 0;
    }
    __syncthreads();
    ws = __shfl_sync(kFull, ws, 0) + s_base[0];
    wb = __shfl_sync(kFull, wb, 0) + s_base[1];
    const unsigned below = (1u << lane) - 1u;
    const int64_t end = a.cap.list[nb] - 1;
    int32_t *__restrict__ list = a.lowlist[nb];
    if (pl) {
        if (sl) list[ws + __popc(m0 & below)] = ql;
        else list[end - (wb + __popc(m1 & below))] = ql;
    }
    if (pr) {
        if (sr) list[ws + __popc(m0) + __popc(m2 & below)] = qr;
        else list[end - (wb + __popc(m1) + __popc(m3 & below))] = qr;
    }
}

// Sum of v over the block (every thread gets it); s_red holds kWarps ints.
__device__ __forceinline__ int32_t block_sum(int32_t v, int32_t *s_red)
{
    v = __reduce_add_sync(kFull, v);
    __syncthreads();  // s_red may still be read by the previous call
    if ((threadIdx.x & 31) == 0) s_red[threadIdx.x >> 5] = v;
    __syncthreads();
    int32_t t = 0;
#pragma unroll
    for (int w = 0; w < kWarps; ++w) t += s_red[w];
    return t;
}

// CreateLowerSAHChildren (LowerTriangleMap.h:557-600) and, when enabled,
// PropagateAabbToChildren (LowerTriangleMap.h:602-636).  The children of the
// split nodes are numbered as the reference's scan of the split flags does:
// left children in node order, then right children.  The level's split
// decisions were counted per tile of kLowTile nodes; one block takes a tile,
// its first split's number is the sum of the earlier tiles' counts and each
// split's rank inside the tile comes from a block scan of the flags.  With
// the SAH creator the children that have enough members to be split are
// listed for the next level's k_calc_sah.
__global__ void k_sah_children(const BuildArgs a)
{
    __shared__ int32_t s_red[kWarps], s_wc[kWarps];
    BuildState *st = a.st;
    const int32_t R0 = st->low_R;
    const int b = st->low_levels & 1, nb = b ^ 1;
    const int32_t *__restrict__ tc = a.lcnt[b];
    const int64_t ntile = ((int64_t)R0 + kLowTile - 1) / kLowTile;
    int32_t part = 0;
    for (int64_t i = threadIdx.x; i < ntile; i += blockDim.x) part += tc[i];
    const int32_t splits = block_sum(part, s_red);
    // After a failure, or when the children do not fit (advance_lower
    // records that), no block writes.
    const int32_t R = (st->err || !lower_fits(a, st, splits)) ? 0 : R0;
    const int32_t *__restrict__ ids = st->low_first ? a.leaf_ids : nullptr;
    const int32_t active = st->low_active, child_base = st->n_nodes;
    const bool list = a.lower == KDGB_LOWER_SAH && 2 * (int64_t)splits <= a.cap.list[nb];
    {  // the next level counts its splits from zero
        const int64_t nt = min((2 * (int64_t)splits + kLowTile - 1) / kLowTile, a.cap.lcnt[nb]);
        GRID_STRIDE(i, R > 0 ? nt : 0) a.lcnt[nb][i] = 0;
    }
    const unsigned lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int64_t rtiles = ((int64_t)R + kLowTile - 1) / kLowTile;
    for (int64_t t = blockIdx.x; t < rtiles; t += gridDim.x) {  // block-uniform
        int32_t ps = 0;
        for (int64_t i = threadIdx.x; i < t; i += blockDim.x) ps += tc[i];
        const int32_t pre = block_sum(ps, s_red);
        const int32_t k = (int32_t)(t * kLowTile) + (int32_t)threadIdx.x;
        const bool sp = k < R && a.ssplit[k];
        const unsigned bal = __ballot_sync(kFull, sp);
        if (lane == 0) s_wc[warp] = __popc(bal);
        __syncthreads();
        int32_t wo = 0;
        for (unsigned w = 0; w < warp; ++w) wo += s_wc[w];
        bool pl = false, pr = false, sl = false, sr = false;
        int32_t ql = 0, qr = 0;
        if (sp) {
            const int32_t par = ids ? ids[k] : active + k;
            ql = pre + wo + __popc(bal & ((1u << lane) - 1u));
            qr = ql + splits;
            const int32_t l = child_base + ql, r = child_base + qr;
            ZERO_NODE(l);
            ZERO_NODE(r);
            const float2 ca = a.careas[k];
            const int2 cs = a.csets[k];
            a.area[l] = ca.x; a.pidx[l] = a.pidx[par]; a.amt[l] = cs.x;
            a.area[r] = ca.y; a.pidx[r] = a.pidx[par]; a.amt[r] = cs.y;
            a.ch[par] = make_int2(l, r);
            if (a.propagate) {
                const int axis = a.info[par] & 3;
                const float spl = a.split[par];
                const float4 mn = a.bmin[par], mx = a.bmax[par];
                a.bmin[l] = mn;
                a.bmin[r] = make_float4(axis == KDGB_X ? spl : mn.x, axis == KDGB_Y ? spl : mn.y,
                                        axis == KDGB_Z ? spl : mn.z, 0.0f);
                a.bmax[l] = make_float4(axis == KDGB_X ? spl : mx.x, axis == KDGB_Y ? spl : mx.y,
                                        axis == KDGB_Z ? spl : mx.z, 0.0f);
                a.bmax[r] = mx;
            }
            const int cl = __popc((unsigned)cs.x), cr = __popc((unsigned)cs.y);
            pl = list && cl > a.min_leaf;
            pr = list && cr > a.min_leaf;
            sl = cl <= 16;
            sr = cr <= 16;
        }
        if (list) lower_list_push(a, st, nb, pl, sl, ql, pr, sr, qr);  // block-uniform
    }
    if (last_block(st)) advance_lower(a, st, splits);
}

// ---------------------------------------------------------------------------
// Traversal layout (read by kdgb_trace.cu), in traversal order: roots
// 0..M-1, then the two children of interior node p (rank r among the
// interior nodes in node order) at M + 2r (left) and M + 2r + 1 (right).
//   tnode[j]  int2  interior: {split bits, (left << 2) | axis}
//                   leaf:     {first record, (record count << 2) | 0}
//   tbox[2j], tbox[2j+1]  min and max of the leaf's box (leaf skipping), one sector
//   ttri[3r..3r+2]  float4 x3 per leaf record, in leaf order (LSB first):
//                   {v0.xyz, e1.x} {e1.yz, e2.xy} {e2.z, id bits, 0, 0}
// One 8-byte load per traversal step, siblings in one sector, and three
// 16-byte loads per triangle test, with no index indirection; e1 = v1 - v0
// and e2 = v2 - v0 are the same fp32 values the reference computes per test.
// off holds the exclusive scan of PackLanes: off[2i] the first record of
// node i, off[2i + 1] its interior rank; record n holds the totals.  The
// node count is n_host, or *n_dev when given; err (optional) skips the pass
// after a failed build.
// ---------------------------------------------------------------------------
__device__ __forceinline__ bool pack_ok(int32_t n, const int32_t *err, const int32_t *off, int64_t cap_tris)
{
    return !(err && *err) && (int64_t)off[2 * (int64_t)n] <= cap_tris;
}

// Each node's traversal index: roots keep theirs, the children of interior
// node i go to M + 2 rank(i) and the slot after it.  norder starts at -1, so
// a node that no interior node names stays outside [0, n) and is not packed.
__global__ void k_pack_order(int32_t n_host, const int32_t *n_dev, const int32_t *err, int64_t cap_tris, int32_t M,
                             const int8_t *__restrict__ info, const int2 *__restrict__ ch,
                             const int32_t *__restrict__ off, int32_t *__restrict__ norder)
{
    const int32_t n = n_dev ? *n_dev : n_host;
    if (!pack_ok(n, err, off, cap_tris)) return;
    GRID_STRIDE(i, n) {
        if (i < M) norder[i] = (int32_t)i;
        if ((info[i] & 3) == KDGB_LEAF) continue;
        const int2 c = ch[i];
        const int32_t first = M + 2 * off[2 * i + 1];
        if (c.x >= 0 && c.x < n) norder[c.x] = first;
        if (c.y >= 0 && c.y < n) norder[c.y] = first + 1;
    }
}

__global__ void k_pack_nodes(int32_t n_host, const int32_t *n_dev, const int32_t *err, int64_t cap_tris, int32_t M,
                             const int8_t *__restrict__ info, const float *__restrict__ split,
                             const float4 *__restrict__ bmin, const float4 *__restrict__ bmax,
                             const int32_t *__restrict__ off, const int32_t *__restrict__ norder,
                             int2 *__restrict__ tnode, float4 *__restrict__ tbox)
{
    const int32_t n = n_dev ? *n_dev : n_host;
    if (!pack_ok(n, err, off, cap_tris)) return;
    GRID_STRIDE(i, n) {
        const int32_t j = norder[i];
        if (j < 0 || j >= n) continue;  // not reached from a root
        const int ax = info[i] & 3;
        if (ax == KDGB_LEAF) {
            const int32_t first = off[2 * i];
            tnode[j] = make_int2(first, (off[2 * i + 2] - first) << 2);
            tbox[2 * (int64_t)j] = bmin[i];
            tbox[2 * (int64_t)j + 1] = bmax[i];
        } else {
            tnode[j] = make_int2(__float_as_int(split[i]), ((M + 2 * off[2 * i + 1]) << 2) | ax);
        }
    }
}

// Leaf records in leaf order: a warp takes 32 consecutive nodes, whose
// records are contiguous from off[2 * first node], and writes them 32 at a time,
// so the stores are coalesced and every lane has a record whatever the leaf
// sizes.  Record r of the group belongs to the last node j whose exclusive
// count is <= r, and is the (r - excl_j)-th member (bit order) of its bitmap.
__global__ void k_pack_tris(int32_t n_host, const int32_t *n_dev, const int32_t *err, int64_t cap_tris,
                            const int8_t *__restrict__ info, const int32_t *__restrict__ bitmap,
                            const int32_t *__restrict__ pidx, const int32_t *__restrict__ prim_indices,
                            const float4 *__restrict__ prec, const int32_t *__restrict__ off,
                            float4 *__restrict__ ttri)
{
    const int32_t n = n_dev ? *n_dev : n_host;
    if (!pack_ok(n, err, off, cap_tris)) return;
    const int lane = threadIdx.x & 31;
    WARP_STRIDE(w, (n + 31) >> 5) {
        const int32_t node = (int32_t)(w << 5) + lane;
        const bool leaf = node < n && (info[node] & 3) == KDGB_LEAF;  // as PackLanes counts them
        const unsigned bmp = leaf ? (unsigned)bitmap[node] : 0u;
        const int32_t first = leaf ? pidx[node] : 0;
        const int cnt = __popc(bmp);
        int incl = cnt;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(kFull, incl, o);
            if (lane >= o) incl += y;
        }
        const int excl = incl - cnt;
        const int total = __shfl_sync(kFull, incl, 31);
        const int64_t rec0 = off[2 * (w << 5)];
        for (int base = 0; base < total; base += 32) {  // warp-uniform trip count
            const int r = base + lane;
            int j = 0;
#pragma unroll
            for (int step = 16; step > 0; step >>= 1) {
                const int e = __shfl_sync(kFull, excl, j + step);
                if (e <= r) j += step;
            }
            const int ej = __shfl_sync(kFull, excl, j);
            const unsigned m = __shfl_sync(kFull, bmp, j);
            const int32_t fj = __shfl_sync(kFull, first, j);
            if (r < total) {
                const int32_t prim = prim_indices[fj + nth_bit(m, r - ej)];
                const float4 *src = prec + 3 * (int64_t)prim;
                const float4 qa = __ldg(src), qb = __ldg(src + 1), qc = __ldg(src + 2);
                const int64_t rec = rec0 + r;
                ttri[3 * rec + 0] = qa;
                ttri[3 * rec + 1] = qb;
                ttri[3 * rec + 2] = qc;
            }
        }
    }
}

__global__ void k_pack_finish(const BuildArgs a)
{
    BuildState *st = a.st;
    if (st->err) return;
    const int32_t total = a.loff[2 * (int64_t)st->n_nodes];
    if ((int64_t)total > a.cap.tris) {
        set_err(st, KDGB_ERR_CAPACITY, kErrPackCapacity);
        return;
    }
    st->n_leaf_tris = total;
}

// ---------------------------------------------------------------------------
// Host side.
// ---------------------------------------------------------------------------

// Launch extents: the sizes grids are computed for.  Exact in the
// host-driven build, the buffer capacities in a graph build.
struct Extents {
    int64_t N, R, F, nodes, leaves, low_R;
};

int sm_count()
{
    // The current context's SMs: a graph captured for an SM partition sizes
    // its grids for that partition.
    if (const int c = context_sm_count(); c > 0) return c;
    int dev = 0, n = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
        cudaGetLastError();
        return 148;
    }
    return n > 0 ? n : 148;
}

struct Launcher {
    int sms;
    // Grid for `items` work items of `per_block` each, capped at `waves`
    // blocks per SM (the kernels loop over the rest).  Four is one resident
    // wave of the 64-register level kernels: a second wave only queued behind
    // the first, and with frames in flight the blocks of a smaller grid leave
    // more of the GPU to the trace running beside them (end-to-end frames
    // 2.95 -> 2.88 ms; the device-timed rebuild 2.12 -> 2.13 ms).
    unsigned grid(int64_t items, int per_block, int waves = 4) const
    {
        const int64_t b = std::max<int64_t>(1, ceil_div(items, per_block));
        return (unsigned)std::min<int64_t>(b, (int64_t)sms * waves);
    }
};

template <class T>
int reserve_keep(DevArray<T> &a, int64_t n, int64_t keep, cudaStream_t s)
{
    if (a.p && n <= a.cap) return KDGB_OK;
    const int64_t want = a.cap + a.cap / 2 > n ? a.cap + a.cap / 2 : n;
    return ensure(a, want, s, a.p ? keep : 0);
}

int grow_nodes(Tree &t, int64_t need, int64_t keep, cudaStream_t s)
{
    if (need <= t.info.cap) return KDGB_OK;
    int64_t cap = t.info.cap > 0 ? t.info.cap : 1024;
    while (cap < need) cap *= 2;
    KDGB_CHECK(ensure(t.info, cap, s, keep));
    KDGB_CHECK(ensure(t.split, cap, s, keep));
    KDGB_CHECK(ensure(t.bmin, cap, s, keep));
    KDGB_CHECK(ensure(t.bmax, cap, s, keep));
    KDGB_CHECK(ensure(t.pidx, cap, s, keep));
    KDGB_CHECK(ensure(t.bitmap, cap, s, keep));
    KDGB_CHECK(ensure(t.children, cap, s, keep));
    KDGB_CHECK(ensure(t.area, cap, s, keep));
    KDGB_CHECK(ensure(t.parent, cap, s, keep));
    return KDGB_OK;
}

int host_record(Workspace &ws)
{
    if (!ws.host) KDGB_CUDA(cudaMallocHost(&ws.host, kHostRec * sizeof(int32_t)));
    return KDGB_OK;
}

// Arguments for the current buffers, with capacities as allocated.
BuildArgs make_args(Tree &t, const kdgb_build_params &p, int32_t T, int32_t M, const int32_t *mesh_off)
{
    Workspace &w = t.ws;
    BuildArgs a;
    memset(&a, 0, sizeof(a));
    a.st = w.state.p;
    a.T = T;
    a.M = M;
    a.mesh_off = mesh_off;
    a.LS = p.leaf_size;
    a.B = p.sah_bins;
    a.upper_levels = p.upper_levels;
    a.max_levels = p.max_levels;
    a.min_leaf = p.min_leaf;
    a.ess = p.split_empty_space;
    a.zmax_as_x = p.esc_zmax_as_x;
    a.propagate = p.propagate_aabbs;
    a.tuned = p.mode == KDGB_BUILD_TUNED;
    a.lower = p.lower;
    a.divide = p.split_method == KDGB_SPLIT_DIVIDE;
    a.thr = p.empty_space_threshold;
    a.ct = p.traversal_cost;
    a.ci = p.intersection_cost;
    a.prec = t.prec.p;
    a.p0 = t.p0.p;
    a.p1 = t.p1.p;
    a.p2 = t.p2.p;
    for (int b = 0; b < 2; ++b) {
        a.rmin[b] = w.rmin[b].p;
        a.rmax[b] = w.rmax[b].p;
        a.cap.refs[b] = std::min(w.rmin[b].cap, w.rmax[b].cap);
    }
    a.fmin = w.fmin.p;
    a.fmax = w.fmax.p;
    a.cap.fin = std::min(w.fmin.cap, w.fmax.cap);
    a.info = t.info.p;
    a.split = t.split.p;
    a.bmin = t.bmin.p;
    a.bmax = t.bmax.p;
    a.pidx = t.pidx.p;
    a.amt = t.bitmap.p;
    a.parent = t.parent.p;
    a.ch = t.children.p;
    a.area = t.area.p;
    a.cap.nodes = t.info.cap;
    a.prim_indices = t.prim_indices.p;
    a.leaf_ids = t.leaf_ids.p;
    a.keys = w.keys.p;
    a.cnt = w.cnt.p;
    a.lbase = w.lbase.p;
    for (int b = 0; b < 2; ++b) {
        a.ess_cnt[b] = w.ess[b].p;
        a.planes[b] = w.planes[b].p;
    }
    // Next-level node entries are written by k_children into these.
    a.cap.R = std::min({w.keys.cap / 6, w.cnt.cap / 2, w.ess[0].cap, w.ess[1].cap, w.planes[0].cap,
                        w.planes[1].cap});
    a.chunksum = w.chunksum.p;
    a.tilesum = w.tilesum.p;
    a.tileoff = w.tileoff.p;
    a.big = w.big.p;
    a.bighist = w.bighist.p;
    a.cap.big = std::min(w.big.cap / kSahItem, w.bighist.cap / kSahHist);
    a.ranges = w.ranges.p;
    a.roff = w.roff.p;
    a.cap.ranges = std::min(w.ranges.cap, w.roff.cap);
    a.cap.leaves = INT64_MAX;  // leaf ids are written after the loop and sized then
    a.areas = w.areas.p;
    a.sts = w.sts.p;
    a.ssplit = w.ssplit.p;
    for (int b = 0; b < 2; ++b) {
        a.lcnt[b] = w.lcnt[b].p;
        a.cap.lcnt[b] = w.lcnt[b].cap;
    }
    a.careas = w.careas.p;
    a.csets = w.csets.p;
    a.cap.low_R = INT64_MAX;  // the host sizes each lower level before it runs
    for (int b = 0; b < 2; ++b) {
        a.lowlist[b] = w.lowlist[b].p;
        a.cap.list[b] = w.lowlist[b].cap;
    }
    a.norder = w.misc0.p;
    a.loff = w.misc1.p;
    a.tnode = t.tnode.p;
    a.tbox = t.tbox.p;
    a.ttri = t.ttri.p;
    a.cap.tris = t.ttri.cap / 3;
    return a;
}

// Launch sequences shared by the host-driven and the graph build.
// Launches the packed triangle records on fork.aux (joined later with
// fork_join) when there is a side stream, else on s.
int emit_prec(const BuildArgs &a, const Launcher &L, const float *tri_v_dev, cudaStream_t s, const Fork *fork)
{
    if (a.T <= 0) return KDGB_OK;
    cudaStream_t ps = s;
    if (fork && fork->aux) {
        KDGB_CUDA(cudaEventRecord(fork->ev[0], s));
        KDGB_CUDA(cudaStreamWaitEvent(fork->aux, fork->ev[0], 0));
        ps = fork->aux;
    }
    KDGB_KERNEL(k_load_prec, L.grid(a.T, kBlock), kBlock, 0, ps, tri_v_dev, a.T, a.prec);
    if (ps != s) KDGB_CUDA(cudaEventRecord(fork->ev[1], ps));
    return KDGB_OK;
}

// s waits for the side branch (nothing to do without one).
int fork_join(cudaStream_t s, const Fork *fork)
{
    if (fork && fork->aux) KDGB_CUDA(cudaStreamWaitEvent(s, fork->ev[1], 0));
    return KDGB_OK;
}

int emit_begin(const BuildArgs &a, const Launcher &L, const float *tri_v_dev, cudaStream_t s,
               const Fork *fork = nullptr)
{
    KDGB_KERNEL(k_begin, L.grid(a.M, kBlock), kBlock, 0, s, a);
    KDGB_CHECK(emit_prec(a, L, tri_v_dev, s, fork));
    if (a.T > 0) {
        KDGB_KERNEL(k_load_geometry, L.grid(a.T, kBlock), kBlock, 0, s, tri_v_dev, a.T, a.p0, a.p1, a.p2, a.rmin[0],
                                                               a.rmax[0], &a.st->nonfinite, a.mesh_off, a.M);
        // The roots' tight boxes; later levels get theirs from k_scatter.
        KDGB_KERNEL(k_reduce, L.grid(a.T, kTileRefs), kBlock, 0, s, a);
    }
    // The roots' splits; later levels get theirs from k_children.
    KDGB_KERNEL(k_node_split, L.grid(a.M, kBlock), kBlock, 0, s, a);
    return KDGB_OK;
}

int emit_upper_level(const BuildArgs &a, const Launcher &L, const Extents &e, bool tuned_levels, Workspace &w,
                     cudaStream_t s)
{
    const unsigned gN = L.grid(e.N, kTileRefs);
    if (tuned_levels) {
        // Enough blocks for one per large node and one warp per node.
        const int64_t big = ceil_div(e.N, kSahBlockRefs);  // at least the large nodes
        // Two waves: the warps binning small nodes one after another are
        // latency-bound, and the second wave starts as the first drains
        // (rebuild 2.19 -> 2.16 ms).
        KDGB_KERNEL(k_sah_bin, L.grid(std::max<int64_t>(big * kBlock, e.R * 32), kBlock, 8), kBlock, 0, s, a);
    }
    if (e.N > 0) {
        if (a.divide) KDGB_KERNEL(k_count<true>, gN, kBlock, 0, s, a);
        else KDGB_KERNEL(k_count<false>, gN, kBlock, 0, s, a);
    }
    // Tile offsets and node bases: independent scans, one launch.
    const NodeLanes lanes{a.cnt, {a.ess_cnt[0], a.ess_cnt[1]}, &a.st->level, a.LS};
    KDGB_CHECK((scan_exclusive_pair<2, ScanArray<2>, kLanes, NodeLanes>(
        ScanArray<2>{a.tilesum}, a.tileoff, ceil_div(e.N, kTileRefs), &a.st->ntiles, lanes, a.lbase, e.R, &a.st->R, s,
        &w.scan, &a.st->err)));
    if (e.N > 0) {
        if (a.divide) KDGB_KERNEL(k_scatter<true>, gN, kBlock, 0, s, a);
        else KDGB_KERNEL(k_scatter<false>, gN, kBlock, 0, s, a);
    }
    KDGB_KERNEL(k_children, L.grid(2 * e.R, kBlock, 2), kBlock, 0, s, a);  // a thread per child
    return KDGB_OK;
}

int emit_after_upper(const BuildArgs &a, const Launcher &L, const Extents &e, const kdgb_build_params &p,
                     cudaStream_t s)
{
    const bool parent_boxes = !p.split_empty_space && p.propagate_aabbs;
    if (p.lower == KDGB_LOWER_SAH) {
        // k_areas also extracts the triangle indices, k_sah_preprocess also
        // writes the leaf ids.
        KDGB_KERNEL(k_areas, L.grid(e.F, kBlock), kBlock, 0, s, a);
        KDGB_KERNEL(k_sah_preprocess, L.grid(e.leaves, kBlock), kBlock, 0, s, a);
        if (parent_boxes) KDGB_KERNEL(k_propagate_parent, L.grid(e.leaves, kBlock), kBlock, 0, s, a);
    } else {
        KDGB_KERNEL(k_leaf_ids, L.grid(e.leaves, kBlock), kBlock, 0, s, a);
        KDGB_KERNEL(k_extract_indices, L.grid(e.F, kBlock), kBlock, 0, s, a);
        if (parent_boxes) KDGB_KERNEL(k_propagate_parent, L.grid(e.leaves, kBlock), kBlock, 0, s, a);
        // Every reference of an upper leaf (PreprocessLeafNodes,
        // LowerTriangleMap.h:40-53 and TriangleMapBitmapCreator.cu:32-49).
        KDGB_KERNEL(k_bitmap_leaves, L.grid(e.leaves, kBlock), kBlock, 0, s, a);
    }
    if (lower_loop(p)) {
        // The split counters of the first two lower levels start at zero
        // (k_sah_children clears those of every later level).
        for (int b = 0; b < 2; ++b)
            KDGB_CUDA(cudaMemsetAsync(a.lcnt[b], 0, sizeof(int32_t) * (size_t)a.cap.lcnt[b], s));
        KDGB_KERNEL(k_sah_planes, L.grid(e.leaves * 32, kBlock), kBlock, 0, s, a);
        KDGB_KERNEL(k_lower_begin, 1, 1, 0, s, a);
    }
    return KDGB_OK;
}

// Split counters for a lower level of n nodes.
inline int64_t low_tiles(int64_t n) { return std::max<int64_t>(1, ceil_div(n, kLowTile)); }

// k_calc_sah runs at most one resident wave (its warps share the level's
// work lists evenly).
unsigned calc_sah_grid(const Launcher &L, int64_t R)
{
    static int per_sm = 0;
    if (per_sm <= 0) {
        int n = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_calc_sah, kBlock, 0) != cudaSuccess || n < 1) {
            (void)cudaGetLastError();
            n = 1;
        }
        per_sm = n;
    }
    return std::min<unsigned>(L.grid(R, kBlock), (unsigned)(L.sms * per_sm));
}

int emit_lower_level(const BuildArgs &a, const Launcher &L, const Extents &e, cudaStream_t s)
{
    if (a.lower == KDGB_LOWER_BALANCED) KDGB_KERNEL(k_calc_balanced, L.grid(e.low_R * 32, kBlock), kBlock, 0, s, a);
    else KDGB_KERNEL(k_calc_sah, calc_sah_grid(L, e.low_R), kBlock, 0, s, a);
    KDGB_KERNEL(k_sah_children, L.grid(e.low_R, kLowTile), kLowTile, 0, s, a);  // a block per tile of nodes
    return KDGB_OK;
}

// Leaf record counts, their scan and the recorded total.
int emit_pack_counts(const BuildArgs &a, const Launcher &L, const Extents &e, Workspace &w, cudaStream_t s)
{
    KDGB_CHECK((scan_exclusive_in<2, PackLanes>(PackLanes{a.info, a.amt}, a.loff, e.nodes, s, &w.scan,
                                                &a.st->n_nodes, &a.st->err)));
    KDGB_KERNEL(k_pack_finish, 1, 1, 0, s, a);
    return KDGB_OK;
}

int emit_pack(const BuildArgs &a, const Launcher &L, const Extents &e, cudaStream_t s, const Fork *fork = nullptr)
{
    const unsigned g = L.grid(e.nodes, kBlock);
    // The leaf records need only the scanned leaf counts: on a side stream
    // they are copied while the nodes are packed.
    cudaStream_t ts = s;
    if (fork && fork->aux) {
        KDGB_CUDA(cudaEventRecord(fork->ev[0], s));
        KDGB_CUDA(cudaStreamWaitEvent(fork->aux, fork->ev[0], 0));
        ts = fork->aux;
    }
    KDGB_KERNEL(k_pack_tris, L.grid(e.nodes, kBlock), kBlock, 0, ts, 0, &a.st->n_nodes, &a.st->err, a.cap.tris, a.info,
                                                                  a.amt, a.pidx,
                                     a.prim_indices, a.prec, a.loff, a.ttri);
    if (ts != s) KDGB_CUDA(cudaEventRecord(fork->ev[1], ts));
    KDGB_CUDA(cudaMemsetAsync(a.norder, 0xff, sizeof(int32_t) * (size_t)std::max<int64_t>(e.nodes, 1), s));
    KDGB_KERNEL(k_pack_order, g, kBlock, 0, s, 0, &a.st->n_nodes, &a.st->err, a.cap.tris, a.M, a.info, a.ch, a.loff, a.norder);
    KDGB_KERNEL(k_pack_nodes, g, kBlock, 0, s, 0, &a.st->n_nodes, &a.st->err, a.cap.tris, a.M, a.info, a.split, a.bmin, a.bmax,
                                      a.loff, a.norder, a.tnode, a.tbox);
    return fork_join(s, fork);
}

const char *detail_message(int d)
{
    switch (d) {
    case kErrNonfinite: return "non-finite vertex coordinate";
    case kErrUpperCapacity: return "upper level outgrew the build buffers";
    case kErrLeafCapacity: return "upper leaves outgrew the build buffers";
    case kErrFewerRefs: return "split produced fewer references than its input";
    case kErrMaxLevels: return "upper build exceeded max_levels";
    case kErrLowerCapacity: return "SAH lower level outgrew the build buffers";
    case kErrPackCapacity: return "leaf records outgrew the traversal buffers";
    default: return "build failed";
    }
}

// Reads the device state through the pinned record (synchronises s).
int fetch_state(Tree &t, BuildState &out, cudaStream_t s)
{
    Workspace &w = t.ws;
    KDGB_CHECK(host_record(w));
    static_assert(sizeof(BuildState) <= kHostRec * sizeof(int32_t), "pinned record too small");
    KDGB_CUDA(cudaMemcpyAsync(w.host, w.state.p, sizeof(BuildState), cudaMemcpyDeviceToHost, s));
    KDGB_CUDA(cudaStreamSynchronize(s));
    memcpy(&out, w.host, sizeof(BuildState));
    if (out.err) return fail(out.err, detail_message(out.err_detail));
    return KDGB_OK;
}

void apply_state(Tree &t, const BuildState &st)
{
    t.n_nodes = st.n_nodes;
    t.n_refs = (int32_t)st.F;
    t.n_upper_leaves = st.n_leaf_ids;
    t.n_leaf_tris = st.n_leaf_tris;
    t.stats.upper_levels = st.level;
    t.stats.lower_levels = st.low_levels;
    t.stats.n_nodes = st.n_nodes;
    t.stats.n_refs = (int32_t)st.F;
}

int geometry_arrays(Tree &t, int32_t T, cudaStream_t s)
{
    t.woop_valid = false;  // the Woop rows follow the geometry
    KDGB_CHECK(ensure(t.p0, T, s));
    KDGB_CHECK(ensure(t.p1, T, s));
    KDGB_CHECK(ensure(t.p2, T, s));
    KDGB_CHECK(ensure(t.prec, 3 * (int64_t)T, s));
    t.n_tris = T;
    return KDGB_OK;
}

int64_t scaled(int64_t v, double h, int64_t slack) { return (int64_t)std::ceil((double)v * h) + slack; }

// Arguments and extents of a graph build over the buffers reserve_for_graph
// allocated: every extent is the capacity of what it indexes.
void graph_args(Tree &t, const kdgb_build_params &p, int32_t T, int32_t M, const int32_t *mesh_off, BuildArgs &a,
                Extents &e)
{
    Workspace &w = t.ws;
    a = make_args(t, p, T, M, mesh_off);
    const int64_t chunk_refs = std::min({w.chunksum.cap / 2 * kChunk, w.tilesum.cap / 2 * kTileRefs,
                                         (w.tileoff.cap / 2 - 1) * kTileRefs});
    a.cap.refs[0] = std::min(a.cap.refs[0], chunk_refs);
    a.cap.refs[1] = std::min(a.cap.refs[1], chunk_refs);
    a.cap.R = std::min(a.cap.R, w.lbase.cap / kLanes - 1);
    a.cap.leaves = t.leaf_ids.cap;
    a.cap.low_R = std::min({w.ssplit.cap, w.careas.cap, w.csets.cap,
                            std::min(w.lcnt[0].cap, w.lcnt[1].cap) * (int64_t)kLowTile});
    a.cap.fin = std::min({a.cap.fin, t.prim_indices.cap, w.areas.cap, w.sts.cap / 3});
    a.cap.nodes = std::min({a.cap.nodes, w.misc0.cap, w.misc1.cap / 2 - 1, t.tnode.cap, t.tbox.cap / kBoxStride,
                            kMaxPackNodes - 1});
    a.use_cond = 1;
    e.N = std::min(a.cap.refs[0], a.cap.refs[1]);
    e.R = a.cap.R;
    e.F = a.cap.fin;
    e.nodes = a.cap.nodes;
    e.leaves = a.cap.leaves;
    e.low_R = a.cap.low_R;
}

}  // namespace

uint64_t layout_signature(const Tree &t)
{
    uint64_t h = 1469598103934665603ull;
    auto mix = [&h](const void *p, int64_t cap) {
        h = (h ^ (uint64_t)(uintptr_t)p) * 1099511628211ull;
        h = (h ^ (uint64_t)cap) * 1099511628211ull;
    };
#define MIX(arr) mix((arr).p, (arr).cap)
    const Workspace &w = t.ws;
    MIX(t.p0); MIX(t.p1); MIX(t.p2); MIX(t.prec); MIX(t.info); MIX(t.split); MIX(t.bmin); MIX(t.bmax); MIX(t.pidx);
    MIX(t.bitmap); MIX(t.parent); MIX(t.children); MIX(t.area); MIX(t.prim_indices); MIX(t.leaf_ids);
    MIX(t.tnode); MIX(t.tbox); MIX(t.ttri); MIX(t.mesh_off); MIX(t.mesh_order); MIX(t.qctr);
    MIX(w.rmin[0]); MIX(w.rmin[1]); MIX(w.rmax[0]); MIX(w.rmax[1]); MIX(w.fmin); MIX(w.fmax);
    MIX(w.keys); MIX(w.planes[0]); MIX(w.planes[1]); MIX(w.cnt); MIX(w.ess[0]); MIX(w.ess[1]); MIX(w.lbase);
    MIX(w.chunksum);
    MIX(w.tilesum); MIX(w.tileoff); MIX(w.scan); MIX(w.misc0); MIX(w.misc1); MIX(w.big); MIX(w.bighist); MIX(w.areas); MIX(w.sts);
    MIX(w.ssplit); MIX(w.lcnt[0]); MIX(w.lcnt[1]); MIX(w.roff); MIX(w.careas); MIX(w.csets); MIX(w.ranges); MIX(w.state);
    MIX(w.lowlist[0]); MIX(w.lowlist[1]);
#undef MIX
    return h;
}

int read_build_state(Tree &t, cudaStream_t s)
{
    if (!t.ws.state.p) return fail(KDGB_ERR_INVALID_ARGUMENT, "tree has no build state");
    BuildState st;
    KDGB_CHECK(fetch_state(t, st, s));
    apply_state(t, st);
    return KDGB_OK;
}

int load_geometry(Tree &t, const float *tri_v_dev, int32_t T, cudaStream_t s)
{
    KDGB_CHECK(geometry_arrays(t, T, s));
    if (T == 0) return KDGB_OK;
    Workspace &w = t.ws;
    KDGB_CHECK(host_record(w));
    KDGB_CHECK(grab(w.stats, 16, s));
    KDGB_CUDA(cudaMemsetAsync(w.stats.p, 0, sizeof(int), s));
    const Launcher L{sm_count()};
    KDGB_KERNEL(k_load_geometry, L.grid(T, kBlock), kBlock, 0, s, tri_v_dev, T, t.p0.p, t.p1.p, t.p2.p, nullptr,
             nullptr, w.stats.p, nullptr, 1);
    KDGB_KERNEL(k_load_prec, L.grid(T, kBlock), kBlock, 0, s, tri_v_dev, T, t.prec.p);
    KDGB_CUDA(cudaMemcpyAsync(w.host, w.stats.p, sizeof(int), cudaMemcpyDeviceToHost, s));
    KDGB_CUDA(cudaStreamSynchronize(s));
    if (w.host[0]) return fail(KDGB_ERR_NONFINITE, "non-finite vertex coordinate");
    return KDGB_OK;
}

int pack_for_traversal(Tree &t, cudaStream_t s)
{
    const int32_t n = t.n_nodes;
    if ((int64_t)n >= kMaxPackNodes) return fail(KDGB_ERR_CAPACITY, "too many nodes for the traversal layout");
    Workspace &w = t.ws;
    KDGB_CHECK(host_record(w));
    KDGB_CHECK(grab(w.misc0, std::max<int64_t>(n, 1), s));
    KDGB_CHECK(grab(w.misc1, 2 * ((int64_t)n + 1), s));
    const Launcher L{sm_count()};
    int32_t *norder = w.misc0.p, *off = w.misc1.p;
    KDGB_CHECK((scan_exclusive_in<2, PackLanes>(PackLanes{t.info.p, t.bitmap.p}, off, n, s, &w.scan, nullptr,
                                                nullptr)));
    KDGB_CUDA(cudaMemcpyAsync(w.host + kHostRec - 1, off + 2 * (int64_t)n, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
    KDGB_CUDA(cudaStreamSynchronize(s));
    const int32_t total = w.host[kHostRec - 1];
    KDGB_CHECK(ensure(t.tnode, n, s));
    KDGB_CHECK(ensure(t.tbox, kBoxStride * (int64_t)n, s));
    KDGB_CHECK(ensure(t.ttri, 3 * (int64_t)total, s));
    t.n_leaf_tris = total;
    if (n > 0) {
        const unsigned g = L.grid(n, kBlock);
        KDGB_CUDA(cudaMemsetAsync(norder, 0xff, sizeof(int32_t) * (size_t)n, s));
        KDGB_KERNEL(k_pack_order, g, kBlock, 0, s, n, nullptr, nullptr, INT64_MAX, t.n_meshes, t.info.p, t.children.p, off,
                                          norder);
        KDGB_KERNEL(k_pack_nodes, g, kBlock, 0, s, n, nullptr, nullptr, INT64_MAX, t.n_meshes, t.info.p, t.split.p, t.bmin.p,
                                          t.bmax.p, off, norder, t.tnode.p, t.tbox.p);
        KDGB_KERNEL(k_pack_tris, L.grid(n, kBlock), kBlock, 0, s, n, nullptr, nullptr, INT64_MAX, t.info.p,
                                                                        t.bitmap.p, t.pidx.p, t.prim_indices.p,
                                                                        t.prec.p, off, t.ttri.p);
    }
    return KDGB_OK;
}

int build_tree(Tree &t, const float *tri_v_dev, int32_t T, const kdgb_build_params &p, cudaStream_t s,
               const int32_t *mesh_off_dev, int32_t M)
{
    if (M < 1) M = 1;
    Workspace &w = t.ws;
    const Launcher L{sm_count()};
    KDGB_CHECK(host_record(w));
    KDGB_CHECK(geometry_arrays(t, T, s));
    KDGB_CHECK(ensure(w.state, 1, s));
    KDGB_CHECK(grab(w.rmin[0], T, s));
    KDGB_CHECK(grab(w.rmax[0], T, s));
    KDGB_CHECK(grow_nodes(t, M, 0, s));
    KDGB_CHECK(grab(w.planes[0], M, s));
    KDGB_CHECK(grab(w.ess[0], M, s));
    KDGB_CHECK(grab(w.big, kSahItem * sah_items(T), s));
    KDGB_CHECK(ensure(w.bighist, kSahHist * sah_items(T), s, 0, true));
    KDGB_CHECK(reserve_keep(w.keys, 6 * (int64_t)M, 0, s));
    KDGB_CHECK(reserve_keep(w.cnt, 2 * (int64_t)M, 0, s));
    KDGB_CHECK(grab(w.ranges, (int64_t)p.max_levels + 1, s));
    KDGB_CHECK(grab(w.roff, (int64_t)p.max_levels + 1, s));
    KDGB_CHECK(emit_begin(make_args(t, p, T, M, mesh_off_dev), L, tri_v_dev, s));

    BuildPlan plan;
    plan.max_N = T;
    BuildState st;
    memset(&st, 0, sizeof(st));
    st.N = T;
    st.R = M;
    st.n_nodes = M;
    const bool tuned = p.mode == KDGB_BUILD_TUNED;
    while (st.R > 0) {
        const int64_t N = st.N, R = st.R, F = st.F, n_nodes = st.n_nodes;
        const int nxt = (st.level + 1) & 1;
        const bool tuned_level = tuned && st.level + 1 > p.upper_levels;
        plan.max_R = std::max(plan.max_R, R);
        // Room for this level's writes: <= 14R nodes (empty-space chains and
        // children), <= 2N next-level and leaf references, <= 2R next-level
        // node entries (written in place over this level's R).
        KDGB_CHECK(grow_nodes(t, n_nodes + 14 * R, n_nodes, s));
        KDGB_CHECK(grab(w.rmin[nxt], 2 * N, s));
        KDGB_CHECK(grab(w.rmax[nxt], 2 * N, s));
        if (F + 2 * N > w.fmin.cap) {
            const int64_t want = (F + 2 * N) * 3 / 2 + 1024;
            KDGB_CHECK(ensure(w.fmin, want, s, F));
            KDGB_CHECK(ensure(w.fmax, want, s, F));
        }
        KDGB_CHECK(reserve_keep(w.keys, 12 * R, 6 * R, s));
        KDGB_CHECK(reserve_keep(w.cnt, 4 * R, 2 * R, s));
        // This level's planes and counts are in [cur] (kept); k_children
        // writes the next level's (<= 2R) into [nxt].  Both hold 2R, the
        // capacity the level checks its children against.
        const int cur = st.level & 1;
        KDGB_CHECK(reserve_keep(w.ess[cur], 2 * R, R, s));
        KDGB_CHECK(reserve_keep(w.planes[cur], 2 * R, R, s));
        KDGB_CHECK(grab(w.ess[nxt], 2 * R, s));
        KDGB_CHECK(grab(w.planes[nxt], 2 * R, s));
        KDGB_CHECK(grab(w.lbase, kLanes * (R + 1), s));
        KDGB_CHECK(grab(w.chunksum, 2 * chunks_for(N), s));
        KDGB_CHECK(grab(w.tilesum, 2 * ceil_div(N, kTileRefs), s));
        KDGB_CHECK(grab(w.tileoff, 2 * (ceil_div(N, kTileRefs) + 1), s));
        // This level's large-node list is kept; the next level's is listed
        // by k_children.
        KDGB_CHECK(reserve_keep(w.big, kSahItem * sah_items(2 * N), kSahItem * sah_items(N), s));
        KDGB_CHECK(ensure(w.bighist, kSahHist * sah_items(2 * N), s, 0, true));
        const Extents e{N, R, F, n_nodes, 0, 0};
        KDGB_CHECK(emit_upper_level(make_args(t, p, T, M, mesh_off_dev), L, e, tuned_level, w, s));
        KDGB_CHECK(fetch_state(t, st, s));
        plan.max_N = std::max(plan.max_N, st.N);
    }

    // Leaf ids, final reference indices, lower phase.
    const int64_t F = st.F, nl = st.n_leaf_ids;
    KDGB_CHECK(ensure(t.leaf_ids, nl, s));
    KDGB_CHECK(ensure(t.prim_indices, F, s));
    if (p.lower == KDGB_LOWER_SAH) KDGB_CHECK(grab(w.areas, F, s));
    if (lower_loop(p)) {
        KDGB_CHECK(grab(w.sts, 3 * F, s));
        // The first lower level's decision arrays: k_sah_planes already
        // writes them with the SAH creator (the loop's grab keeps them, as
        // the first level needs exactly this size).
        KDGB_CHECK(grab(w.ssplit, nl, s));
        // Split counters of the first two levels (cleared before the first).
        KDGB_CHECK(ensure(w.lcnt[0], low_tiles(nl), s, 0, true));
        KDGB_CHECK(ensure(w.lcnt[1], low_tiles(2 * nl), s, 0, true));
        KDGB_CHECK(grab(w.careas, nl, s));
        KDGB_CHECK(grab(w.csets, nl, s));
    }
    {
        const Extents e{0, 0, F, st.n_nodes, nl, 0};
        KDGB_CHECK(emit_after_upper(make_args(t, p, T, M, mesh_off_dev), L, e, p, s));
    }
    if (lower_loop(p)) {
        KDGB_CHECK(fetch_state(t, st, s));
        bool first = true;
        while (st.low_R > 0) {
            const int64_t R = st.low_R;
            plan.max_low_R = std::max(plan.max_low_R, R);
            KDGB_CHECK(grow_nodes(t, (int64_t)st.n_nodes + 2 * R, st.n_nodes, s));
            if (first) {
                // The first level's decisions may already sit in these
                // arrays (k_sah_planes writes them): they were sized for all
                // upper leaves above and must not be regrown here.
                if (R > w.ssplit.cap || R > w.careas.cap || R > w.csets.cap)
                    return fail(KDGB_ERR_CAPACITY, "first SAH lower level exceeds its decision arrays");
                first = false;
            } else {
                KDGB_CHECK(grab(w.ssplit, R, s));
                // This level's counters: cleared by the level before, or
                // zeroed here when they have to grow.
                KDGB_CHECK(ensure(w.lcnt[st.low_levels & 1], low_tiles(R), s, 0, true));
                KDGB_CHECK(grab(w.careas, R, s));
                KDGB_CHECK(grab(w.csets, R, s));
            }
            // This level lists the next level's nodes (at most 2R) in the
            // other parity's work list; its own list is not touched.
            if (p.lower == KDGB_LOWER_SAH) KDGB_CHECK(ensure(w.lowlist[(st.low_levels + 1) & 1], 2 * R, s));
            const Extents e{0, 0, F, st.n_nodes, nl, R};
            KDGB_CHECK(emit_lower_level(make_args(t, p, T, M, mesh_off_dev), L, e, s));
            KDGB_CHECK(fetch_state(t, st, s));
        }
    }

    // Traversal layout: leaf records sized from the scanned leaf counts.
    const int64_t n = st.n_nodes;
    if (n >= kMaxPackNodes) return fail(KDGB_ERR_CAPACITY, "too many nodes for the traversal layout");
    KDGB_CHECK(grab(w.misc0, std::max<int64_t>(n, 1), s));
    KDGB_CHECK(grab(w.misc1, 2 * (n + 1), s));
    {
        const Extents e{0, 0, F, n, nl, 0};
        BuildArgs a = make_args(t, p, T, M, mesh_off_dev);
        a.cap.tris = INT64_MAX;
        KDGB_CHECK(emit_pack_counts(a, L, e, w, s));
        KDGB_CHECK(fetch_state(t, st, s));
        KDGB_CHECK(ensure(t.tnode, n, s));
        KDGB_CHECK(ensure(t.tbox, kBoxStride * (int64_t)n, s));
        KDGB_CHECK(ensure(t.ttri, 3 * (int64_t)st.n_leaf_tris, s));
        KDGB_CHECK(emit_pack(make_args(t, p, T, M, mesh_off_dev), L, e, s));
    }
    apply_state(t, st);
    plan.F = st.F;
    plan.nodes = st.n_nodes;
    plan.leaves = st.n_leaf_ids;
    plan.leaf_tris = st.n_leaf_tris;
    plan.levels = st.level;
    plan.low_levels = st.low_levels;
    plan.valid = true;
    t.plan = plan;
    return KDGB_OK;
}

int reserve_for_graph(Tree &t, int32_t T, const kdgb_build_params &p, int32_t M, double h, cudaStream_t s)
{
    const BuildPlan &q = t.plan;
    if (!q.valid) return fail(KDGB_ERR_INVALID_ARGUMENT, "graph rebuild needs a completed build of the tree");
    if (M < 1) M = 1;
    const int64_t refs = std::max<int64_t>(scaled(q.max_N, h, 1024), T);
    const int64_t fin = scaled(q.F, h, 1024);
    const int64_t nodes = std::max<int64_t>(scaled(q.nodes, h, 1024), M);
    const int64_t R = std::max<int64_t>(scaled(q.max_R, h, 256), M);
    const int64_t leaves = scaled(q.leaves, h, 256);
    const int64_t low_R = std::max(scaled(q.max_low_R, h, 256), leaves);
    const int64_t tris = scaled(q.leaf_tris, h, 1024);
    Workspace &w = t.ws;
    KDGB_CHECK(host_record(w));
    KDGB_CHECK(geometry_arrays(t, T, s));
    KDGB_CHECK(ensure(w.state, 1, s));
    for (int b = 0; b < 2; ++b) {
        KDGB_CHECK(ensure(w.rmin[b], refs, s));
        KDGB_CHECK(ensure(w.rmax[b], refs, s));
    }
    KDGB_CHECK(ensure(w.fmin, fin, s));
    KDGB_CHECK(ensure(w.fmax, fin, s));
    KDGB_CHECK(grow_nodes(t, nodes, 0, s));
    KDGB_CHECK(ensure(w.keys, 6 * R, s));
    KDGB_CHECK(ensure(w.cnt, 2 * R, s));
    for (int b = 0; b < 2; ++b) {
        KDGB_CHECK(ensure(w.ess[b], R, s));
        KDGB_CHECK(ensure(w.planes[b], R, s));
    }
    KDGB_CHECK(ensure(w.lbase, kLanes * (R + 1), s));
    KDGB_CHECK(ensure(w.chunksum, 2 * chunks_for(refs), s));
    KDGB_CHECK(ensure(w.tilesum, 2 * ceil_div(refs, kTileRefs), s));
    KDGB_CHECK(ensure(w.tileoff, 2 * (ceil_div(refs, kTileRefs) + 1), s));
    KDGB_CHECK(ensure(w.big, kSahItem * sah_items(refs), s));
    KDGB_CHECK(ensure(w.bighist, kSahHist * sah_items(refs), s, 0, true));
    KDGB_CHECK(ensure(w.ranges, (int64_t)p.max_levels + 1, s));
    KDGB_CHECK(ensure(w.roff, (int64_t)p.max_levels + 1, s));
    KDGB_CHECK(ensure(t.leaf_ids, leaves, s));
    KDGB_CHECK(ensure(t.prim_indices, fin, s));
    KDGB_CHECK(ensure(w.areas, fin, s));
    KDGB_CHECK(ensure(w.sts, 3 * fin, s));
    KDGB_CHECK(ensure(w.ssplit, low_R, s));
    KDGB_CHECK(ensure(w.lcnt[0], low_tiles(low_R), s));
    KDGB_CHECK(ensure(w.lcnt[1], low_tiles(low_R), s));
    KDGB_CHECK(ensure(w.careas, low_R, s));
    KDGB_CHECK(ensure(w.csets, low_R, s));
    KDGB_CHECK(ensure(w.lowlist[0], low_R, s));
    KDGB_CHECK(ensure(w.lowlist[1], low_R, s));
    KDGB_CHECK(ensure(w.misc0, nodes, s));
    KDGB_CHECK(ensure(w.misc1, 2 * (nodes + 1), s));
    KDGB_CHECK(ensure(t.tnode, nodes, s));
    KDGB_CHECK(ensure(t.tbox, kBoxStride * (int64_t)nodes, s));
    KDGB_CHECK(ensure(t.ttri, 3 * tris, s));
    // Scan partials for the extents the capture will use.
    BuildArgs a;
    Extents e;
    graph_args(t, p, T, M, nullptr, a, e);
    const int64_t parts = std::max({scan_pair_needed(ceil_div(e.N, kTileRefs), e.R),
                                    scan_partials_needed(1, e.low_R), scan_partials_needed(1, e.nodes),
                                    (int64_t)1});
    KDGB_CHECK(ensure(w.scan, parts, s, 0, true));  // zeroed scan state
    return KDGB_OK;
}

namespace {

// Appends a WHILE node to the graph captured on cs; its body is captured on
// `body` by emit(handle).  The handle's value is 1 at every graph launch; the
// body's last kernel sets it.
template <class Emit>
int capture_while(cudaStream_t cs, cudaStream_t body, Emit emit)
{
    cudaStreamCaptureStatus status;
    cudaGraph_t graph = nullptr;
    const cudaGraphNode_t *deps = nullptr;
    size_t ndeps = 0;
    KDGB_CUDA(cudaStreamGetCaptureInfo(cs, &status, nullptr, &graph, &deps, nullptr, &ndeps));
    if (status != cudaStreamCaptureStatusActive) return fail(KDGB_ERR_CUDA, "stream capture is not active");
    cudaGraphConditionalHandle handle;
    KDGB_CUDA(cudaGraphConditionalHandleCreate(&handle, graph, 1, cudaGraphCondAssignDefault));
    cudaGraphNodeParams np = {cudaGraphNodeTypeConditional};
    np.conditional.handle = handle;
    np.conditional.type = cudaGraphCondTypeWhile;
    np.conditional.size = 1;
    cudaGraphNode_t node;
    KDGB_CUDA(cudaGraphAddNode(&node, graph, deps, nullptr, ndeps, &np));
    KDGB_CUDA(cudaStreamUpdateCaptureDependencies(cs, &node, nullptr, 1, cudaStreamSetCaptureDependencies));
    cudaGraph_t bg = np.conditional.phGraph_out[0];
    KDGB_CUDA(cudaStreamBeginCaptureToGraph(body, bg, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed));
    const int rc = emit(handle);
    cudaGraph_t ended = nullptr;
    const cudaError_t e = cudaStreamEndCapture(body, &ended);
    if (rc != KDGB_OK) return rc;
    if (e != cudaSuccess) return cuda_fail(e, "loop body capture");
    return KDGB_OK;
}

}  // namespace

int capture_build(Tree &t, const float *tri_v_dev, int32_t T, const kdgb_build_params &p, cudaStream_t cs,
                  cudaStream_t body, const Fork &fork, const int32_t *mesh_off_dev, int32_t M, GraphKernels &counts)
{
    if (M < 1) M = 1;
    Workspace &w = t.ws;
    const Launcher L{sm_count()};
    BuildArgs a;
    Extents e;
    graph_args(t, p, T, M, mesh_off_dev, a, e);
    int64_t c0 = kdgb_launch_count();
    KDGB_CHECK(emit_begin(a, L, tri_v_dev, cs, &fork));
    int64_t c1 = kdgb_launch_count();
    counts.fixed = c1 - c0;
    KDGB_CHECK(capture_while(cs, body, [&](cudaGraphConditionalHandle h) {
        BuildArgs b = a;
        b.upper_cond = h;
        return emit_upper_level(b, L, e, p.mode == KDGB_BUILD_TUNED, w, body);
    }));
    c0 = kdgb_launch_count();
    counts.upper_body = c0 - c1;
    KDGB_CHECK(fork_join(cs, &fork));  // the packed triangle records are complete
    KDGB_CHECK(emit_after_upper(a, L, e, p, cs));
    c1 = kdgb_launch_count();
    counts.fixed += c1 - c0;
    if (lower_loop(p)) {
        KDGB_CHECK(capture_while(cs, body, [&](cudaGraphConditionalHandle h) {
            BuildArgs b = a;
            b.lower_cond = h;
            return emit_lower_level(b, L, e, body);
        }));
    }
    c0 = kdgb_launch_count();
    counts.lower_body = c0 - c1;
    KDGB_CHECK(emit_pack_counts(a, L, e, w, cs));
    KDGB_CHECK(emit_pack(a, L, e, cs, &fork));
    counts.fixed += kdgb_launch_count() - c0;
    return KDGB_OK;
}

}  // namespace kdgb
