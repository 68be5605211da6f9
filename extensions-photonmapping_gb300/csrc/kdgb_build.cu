// Reference-mode kd-tree build on the GPU.
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
//    six-lane node scan, and a reference's destination is its node base plus
//    its rank inside the node (block scan + block offset), which equals the
//    reference's 2N+1-element scans (TriangleMapUpperCreator.cu:557,631);
//  * the host reads one 7-int record per level instead of 6-8 blocking
//    scalar copies, and no level allocates more than it needs.
#include <cuda_runtime.h>

#include <vector>

#include "kdgb_internal.cuh"

namespace kdgb {

namespace {

constexpr int kBlock = 256;

inline unsigned blocks_for(int64_t n, int b = kBlock) { return (unsigned)((n + b - 1) / b); }

// ---------------------------------------------------------------------------
// Geometry and primitive boxes (CalcPrimitiveAabb, TriangleUpper.h:10-28).
// ---------------------------------------------------------------------------
__global__ void k_load_geometry(const float *__restrict__ tri, int32_t T, float4 *__restrict__ p0,
                                float4 *__restrict__ p1, float4 *__restrict__ p2,
                                float4 *__restrict__ cmin, float4 *__restrict__ cmax,
                                int *__restrict__ err)
{
    const int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= T) return;
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
        // w carries the local index of the owning active node (0 = root).
        cmax[i] = make_float4(kmax(mxx, v[6]), kmax(mxy, v[7]), kmax(mxz, v[8]), __int_as_float(0));
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

__global__ void k_init_root(int32_t T, int8_t *info, float *split, float4 *bmin, float4 *bmax,
                            int32_t *pidx, int32_t *amt, int2 *ch, float *area, int32_t *parent)
{
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        zero_node(0, info, split, bmin, bmax, pidx, amt, ch, area, parent);
        amt[0] = T;  // TriangleMapUpperCreator.cu:128-136
    }
}

// ---------------------------------------------------------------------------
// Upper level kernels.
// ---------------------------------------------------------------------------

// Saves the propagated boxes and resets the tight-box keys to +-fInfinity
// (AabbMemset, ReduceSegments.h:328-335).
__global__ void k_level_init(int32_t R, int32_t active, const float4 *__restrict__ bmin,
                             const float4 *__restrict__ bmax, float4 *__restrict__ pmin,
                             float4 *__restrict__ pmax, unsigned *__restrict__ keys,
                             int32_t *__restrict__ cnt)
{
    const int32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= R) return;
    pmin[k] = bmin[active + k];
    pmax[k] = bmax[active + k];
    const unsigned lo = fkey(KDGB_FINF), hi = fkey(-KDGB_FINF);
    keys[6 * k + 0] = lo; keys[6 * k + 1] = lo; keys[6 * k + 2] = lo;
    keys[6 * k + 3] = hi; keys[6 * k + 4] = hi; keys[6 * k + 5] = hi;
    cnt[2 * k] = 0;
    cnt[2 * k + 1] = 0;
}

// Tight node boxes: exact min/max over each node's references, as the
// segmented reduction ReduceSegmentsUnrolled + FinalSegmentedReduce
// (ReduceSegments.h:230-371) computes.
__global__ void __launch_bounds__(kBlock) k_reduce(int64_t N, const float4 *__restrict__ cmin,
                                                  const float4 *__restrict__ cmax,
                                                  unsigned *__restrict__ keys)
{
    const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const unsigned lane = threadIdx.x & 31;
    int owner = -1;
    unsigned k[6] = {0xffffffffu, 0xffffffffu, 0xffffffffu, 0u, 0u, 0u};
    if (r < N) {
        const float4 a = cmin[r], b = cmax[r];
        owner = __float_as_int(b.w);
        k[0] = fkey(a.x); k[1] = fkey(a.y); k[2] = fkey(a.z);
        k[3] = fkey(b.x); k[4] = fkey(b.y); k[5] = fkey(b.z);
    }
    const int o0 = __shfl_sync(0xffffffffu, owner, 0);
    if (__all_sync(0xffffffffu, owner == o0) && o0 >= 0) {
        const unsigned m0 = __reduce_min_sync(0xffffffffu, k[0]);
        const unsigned m1 = __reduce_min_sync(0xffffffffu, k[1]);
        const unsigned m2 = __reduce_min_sync(0xffffffffu, k[2]);
        const unsigned x0 = __reduce_max_sync(0xffffffffu, k[3]);
        const unsigned x1 = __reduce_max_sync(0xffffffffu, k[4]);
        const unsigned x2 = __reduce_max_sync(0xffffffffu, k[5]);
        if (lane == 0) {
            unsigned *kk = keys + 6 * (int64_t)o0;
            atomicMin(kk + 0, m0); atomicMin(kk + 1, m1); atomicMin(kk + 2, m2);
            atomicMax(kk + 3, x0); atomicMax(kk + 4, x1); atomicMax(kk + 5, x2);
        }
    } else if (owner >= 0) {
        unsigned *kk = keys + 6 * (int64_t)owner;
        atomicMin(kk + 0, k[0]); atomicMin(kk + 1, k[1]); atomicMin(kk + 2, k[2]);
        atomicMax(kk + 3, k[3]); atomicMax(kk + 4, k[4]); atomicMax(kk + 5, k[5]);
    }
}

// Writes the tight boxes, the empty-space planes (CalcEmptySpaceSplits,
// EmptySpaceSplitting.h:10-70) and the spatial-median split of the longest
// axis (CalcUpperNodeSplitInfo, ReduceSegments.h:466-484).
__global__ void k_node_split(int32_t R, int32_t active, int do_ess, float thr,
                             const float4 *__restrict__ pmin, const float4 *__restrict__ pmax,
                             const unsigned *__restrict__ keys, float4 *__restrict__ bmin,
                             float4 *__restrict__ bmax, float *__restrict__ split, int8_t *__restrict__ info,
                             int8_t *__restrict__ planes, int32_t *__restrict__ req)
{
    const int32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= R) return;
    const unsigned *kk = keys + 6 * (int64_t)k;
    const float3 mn = make_float3(funkey(kk[0]), funkey(kk[1]), funkey(kk[2]));
    const float3 mx = make_float3(funkey(kk[3]), funkey(kk[4]), funkey(kk[5]));
    bmin[active + k] = make_float4(mn.x, mn.y, mn.z, 0.0f);
    bmax[active + k] = make_float4(mx.x, mx.y, mx.z, 0.0f);
    if (do_ess) {
        const float4 a = pmin[k], b = pmax[k];
        int pl = 0, nr = 0;
        if (__fsub_rn(mn.x, a.x) > __fmul_rn(thr, __fsub_rn(b.x, a.x))) { pl |= 1; nr += 2; }
        if (__fsub_rn(mn.y, a.y) > __fmul_rn(thr, __fsub_rn(b.y, a.y))) { pl |= 2; nr += 2; }
        if (__fsub_rn(mn.z, a.z) > __fmul_rn(thr, __fsub_rn(b.z, a.z))) { pl |= 4; nr += 2; }
        if (__fsub_rn(b.x, mx.x) > __fmul_rn(thr, __fsub_rn(b.x, a.x))) { pl |= 8; nr += 2; }
        if (__fsub_rn(b.y, mx.y) > __fmul_rn(thr, __fsub_rn(b.y, a.y))) { pl |= 16; nr += 2; }
        if (__fsub_rn(b.z, mx.z) > __fmul_rn(thr, __fsub_rn(b.z, a.z))) { pl |= 32; nr += 2; }
        planes[k] = (int8_t)pl;
        req[k] = nr;
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
    split[active + k] = z_higher ? mdz : sp;
    info[active + k] = z_higher ? (int8_t)KDGB_Z : ax;
}

// EmptySpaceSplitting2 (EmptySpaceSplitting.h:74-184): a chain of split
// nodes, each with an empty leaf, between the parent and the active node.
__global__ void k_ess_chain(int32_t R, int32_t active, int32_t base, int zmax_as_x,
                            const int8_t *__restrict__ planes, const int32_t *__restrict__ eaddr,
                            int8_t *info, float *split, float4 *bmin, float4 *bmax, int32_t *pidx,
                            int32_t *amt, int2 *ch, float *area, int32_t *parent)
{
    const int32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= R) return;
    int pl = planes[k];
    if (pl == 0) return;
    const int32_t leaf = active + k;
    const int32_t start = base + eaddr[k];
    const int nn = 2 * __popc(pl);
    for (int j = 0; j < nn; ++j) zero_node(start + j, info, split, bmin, bmax, pidx, amt, ch, area, parent);
    const int32_t par0 = parent[leaf];
    const int2 c = ch[par0];
    if (c.x == leaf) ch[par0].x = start;
    else ch[par0].y = start;
    const float4 mn = bmin[leaf], mx = bmax[leaf];
    int32_t par = start;
    const int8_t axes[3] = {KDGB_X, KDGB_Y, KDGB_Z};
    for (int b = 0; b < 3; ++b) {
        if (pl & (1 << b)) {
            pl -= (1 << b);
            info[par] = axes[b];
            split[par] = axis_of4(mn, axes[b]);
            const int32_t l = par + 1, r = pl ? l + 1 : leaf;
            ch[par] = make_int2(l, r);
            info[l] = KDGB_LEAF;
            amt[l] = 0;
            par = r;
        }
    }
    for (int b = 3; b < 5; ++b) {
        if (pl & (1 << b)) {
            pl -= (1 << b);
            info[par] = axes[b - 3];
            split[par] = axis_of4(mx, axes[b - 3]);
            const int32_t r = par + 1, l = pl ? r + 1 : leaf;
            ch[par] = make_int2(l, r);
            info[r] = KDGB_LEAF;
            amt[r] = 0;
            par = l;
        }
    }
    if (pl & 32) {
        info[par] = zmax_as_x ? (int8_t)KDGB_X : (int8_t)KDGB_Z;
        split[par] = zmax_as_x ? mx.x : mx.z;
        const int32_t r = par + 1;
        ch[par] = make_int2(leaf, r);
        info[r] = KDGB_LEAF;
        amt[r] = 0;
    }
}

__device__ __forceinline__ void ref_flags(const float4 &a, const float4 &b, int axis, float sp, int &L, int &Rf)
{
    // SetSplitSide (TriangleUpperChildren.h:10-62): left = min <= split,
    // right = split < max.
    L = axis_of4(a, axis) <= sp;
    Rf = sp < axis_of4(b, axis);
}

// Per-node left/right counts and per-block totals of the flags.
__global__ void __launch_bounds__(kBlock) k_count(int64_t N, int32_t active, const float4 *__restrict__ cmin,
                                                 const float4 *__restrict__ cmax, const float *__restrict__ split,
                                                 const int8_t *__restrict__ info, int32_t *__restrict__ cnt,
                                                 int32_t *__restrict__ blocksum)
{
    const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const unsigned lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int owner = -1, L = 0, Rf = 0;
    if (r < N) {
        const float4 a = cmin[r], b = cmax[r];
        owner = __float_as_int(b.w);
        const int node = active + owner;
        ref_flags(a, b, info[node], split[node], L, Rf);
    }
    const int o0 = __shfl_sync(0xffffffffu, owner, 0);
    const int wl = __reduce_add_sync(0xffffffffu, L), wr = __reduce_add_sync(0xffffffffu, Rf);
    if (__all_sync(0xffffffffu, owner == o0) && o0 >= 0) {
        if (lane == 0) {
            atomicAdd(cnt + 2 * o0, wl);
            atomicAdd(cnt + 2 * o0 + 1, wr);
        }
    } else if (owner >= 0) {
        if (L) atomicAdd(cnt + 2 * owner, 1);
        if (Rf) atomicAdd(cnt + 2 * owner + 1, 1);
    }
    __shared__ int32_t s[2][kBlock / 32];
    if (lane == 0) { s[0][warp] = wl; s[1][warp] = wr; }
    __syncthreads();
    if (threadIdx.x == 0) {
        int32_t tl = 0, tr = 0;
        for (int w = 0; w < kBlock / 32; ++w) { tl += s[0][w]; tr += s[1][w]; }
        blocksum[2 * (int64_t)blockIdx.x] = tl;
        blocksum[2 * (int64_t)blockIdx.x + 1] = tr;
    }
}

// Six scan lanes per node: left/right sizes, left/right references that go
// to leaves, and the left/right leaf-node flags (CalcNodeChildSize,
// SetPrimitiveLeafSide, MarkNodeLeafs: TriangleUpperChildren.h:144-201).
__global__ void k_node_lanes(int32_t R, int32_t LS, const int32_t *__restrict__ cnt, int32_t *__restrict__ lanes)
{
    const int32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= R) return;
    const int32_t l = cnt[2 * k], r = cnt[2 * k + 1];
    const int ll = l < LS, rl = r < LS;
    int32_t *o = lanes + 6 * (int64_t)k;
    o[0] = l; o[1] = r; o[2] = ll ? l : 0; o[3] = rl ? r : 0; o[4] = ll; o[5] = rl;
}

// Partition + compaction of the references with clipping to the split plane
// (SplitTriangles, TriangleUpperChildren.h:283-383).  Destination = node base
// + rank of the reference among the node's left (right) references.
__global__ void __launch_bounds__(kBlock) k_scatter(
    int64_t N, int32_t R, int32_t active, int32_t LS, int32_t upper,
    const float4 *__restrict__ cmin, const float4 *__restrict__ cmax, const float *__restrict__ split,
    const int8_t *__restrict__ info, const int32_t *__restrict__ blockoff, const int32_t *__restrict__ lbase,
    float4 *__restrict__ nmin, float4 *__restrict__ nmax, float4 *__restrict__ fmin, float4 *__restrict__ fmax)
{
    const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const unsigned lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int owner = -1, L = 0, Rf = 0, axis = 0;
    float sp = 0.0f;
    float4 a = make_float4(0.f, 0.f, 0.f, 0.f), b = a;
    if (r < N) {
        a = cmin[r];
        b = cmax[r];
        owner = __float_as_int(b.w);
        const int node = active + owner;
        axis = info[node];
        sp = split[node];
        ref_flags(a, b, axis, sp, L, Rf);
    }
    const unsigned bl = __ballot_sync(0xffffffffu, L), br = __ballot_sync(0xffffffffu, Rf);
    const unsigned below = (1u << lane) - 1u;
    __shared__ int32_t s[2][kBlock / 32];
    if (lane == 0) { s[0][warp] = __popc(bl); s[1][warp] = __popc(br); }
    __syncthreads();
    int32_t pl = blockoff[2 * (int64_t)blockIdx.x] + __popc(bl & below);
    int32_t pr = blockoff[2 * (int64_t)blockIdx.x + 1] + __popc(br & below);
    for (unsigned w = 0; w < warp; ++w) { pl += s[0][w]; pr += s[1][w]; }
    if (owner < 0) return;

    const int32_t *lb = lbase + 6 * (int64_t)owner;
    const int32_t *tot = lbase + 6 * (int64_t)R;
    const int32_t total_l = tot[0], leaf_l = tot[2], leafnodes_l = tot[4];
    if (L) {
        const int32_t rank = pl - lb[0];
        const float4 hi = make_float4(axis == KDGB_X ? kmin(sp, b.x) : b.x, axis == KDGB_Y ? kmin(sp, b.y) : b.y,
                                      axis == KDGB_Z ? kmin(sp, b.z) : b.z, 0.0f);
        const int32_t lcount = (lbase + 6 * (int64_t)(owner + 1))[0] - lb[0];
        if (lcount < LS) {
            const int64_t dst = (int64_t)upper + lb[2] + rank;
            fmin[dst] = a;
            fmax[dst] = hi;
        } else {
            const int64_t dst = (int64_t)(lb[0] - lb[2]) + rank;
            nmin[dst] = a;
            nmax[dst] = make_float4(hi.x, hi.y, hi.z, __int_as_float(owner - lb[4]));
        }
    }
    if (Rf) {
        const int32_t rank = pr - lb[1];
        const float4 lo = make_float4(axis == KDGB_X ? kmax(sp, a.x) : a.x, axis == KDGB_Y ? kmax(sp, a.y) : a.y,
                                      axis == KDGB_Z ? kmax(sp, a.z) : a.z, a.w);
        const int32_t rcount = (lbase + 6 * (int64_t)(owner + 1))[1] - lb[1];
        if (rcount < LS) {
            const int64_t dst = (int64_t)upper + leaf_l + lb[3] + rank;
            fmin[dst] = lo;
            fmax[dst] = make_float4(b.x, b.y, b.z, 0.0f);
        } else {
            const int64_t dst = (int64_t)(total_l - leaf_l) + (lb[1] - lb[3]) + rank;
            nmin[dst] = lo;
            nmax[dst] = make_float4(b.x, b.y, b.z, __int_as_float(R + owner - (leafnodes_l + lb[5])));
        }
    }
}

// CreateUpperChildren (TriangleUpperChildren.h:203-281) and, with empty-space
// splitting on, PropagateAabbToChildren (EmptySpaceSplitting.h:299-331).
__global__ void k_children(int32_t R, int32_t active, int32_t base, const int32_t *__restrict__ empty_total,
                           int32_t LS, int32_t upper, int propagate, const int32_t *__restrict__ lbase,
                           int8_t *info, float *split, float4 *bmin, float4 *bmax, int32_t *pidx,
                           int32_t *amt, int2 *ch, float *area, int32_t *parent, int32_t *stats)
{
    const int32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    const int32_t empty = empty_total ? *empty_total : 0;
    const int32_t *tot = lbase + 6 * (int64_t)R;
    if (k == 0) {
        stats[0] = empty;
        for (int j = 0; j < 6; ++j) stats[1 + j] = tot[j];
    }
    if (k >= R) return;
    const int32_t child_start = base + empty;
    const int32_t total_l = tot[0], leaf_l = tot[2], ln_l = tot[4], leaf_nodes = tot[4] + tot[5];
    const int32_t *lb = lbase + 6 * (int64_t)k;
    const int32_t *nb = lbase + 6 * (int64_t)(k + 1);
    const int32_t l = nb[0] - lb[0], r = nb[1] - lb[1];
    const int32_t par = active + k;

    const bool lleaf = l < LS;
    const int32_t la = lb[4];
    const int32_t lid = child_start + (lleaf ? la : k - la + leaf_nodes);
    const bool rleaf = r < LS;
    const int32_t ra = ln_l + lb[5];
    const int32_t rid = child_start + (rleaf ? ra : (R + k) - ra + leaf_nodes);

    zero_node(lid, info, split, bmin, bmax, pidx, amt, ch, area, parent);
    zero_node(rid, info, split, bmin, bmax, pidx, amt, ch, area, parent);
    pidx[lid] = lleaf ? upper + lb[2] : lb[0] - lb[2];
    pidx[rid] = rleaf ? upper + leaf_l + lb[3] : (total_l - leaf_l) + (lb[1] - lb[3]);
    amt[lid] = l;
    amt[rid] = r;
    parent[lid] = par;
    parent[rid] = par;
    ch[par] = make_int2(lid, rid);
    if (propagate) {
        const int axis = info[par] & 3;
        const float sp = split[par];
        const float4 mn = bmin[par], mx = bmax[par];
        bmin[lid] = mn;
        bmin[rid] = make_float4(axis == KDGB_X ? sp : mn.x, axis == KDGB_Y ? sp : mn.y, axis == KDGB_Z ? sp : mn.z, 0.0f);
        bmax[lid] = make_float4(axis == KDGB_X ? sp : mx.x, axis == KDGB_Y ? sp : mx.y, axis == KDGB_Z ? sp : mx.z, 0.0f);
        bmax[rid] = mx;
    }
}

// MarkLeafNodes (TriangleUpperChildren.h:385-395) over all levels at once:
// each level appends a contiguous range of leaf node ids.
__global__ void k_leaf_ids(const int2 *__restrict__ ranges, int nr, const int32_t *__restrict__ roff,
                           int32_t total, int32_t *__restrict__ leaf_ids)
{
    const int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= total) return;
    int lo = 0, hi = nr - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (roff[mid] <= i) lo = mid; else hi = mid - 1;
    }
    leaf_ids[i] = ranges[lo].x + (i - roff[lo]);
}

// ExtractIndexFromAabb (TriangleUpper.h:43-52).
__global__ void k_extract_indices(int32_t F, const float4 *__restrict__ fmin, int32_t *__restrict__ out)
{
    const int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < F) out[i] = __float_as_int(fmin[i].w);
}

// PropagateParentAabb<true> (EmptySpaceSplitting.h:333-368).
__global__ void k_propagate_parent(int32_t nl, const int32_t *__restrict__ leaf_ids, const int8_t *info,
                                   const float *split, float4 *bmin, float4 *bmax, const int32_t *parent,
                                   const int2 *ch)
{
    const int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nl) return;
    const int32_t c = leaf_ids[i];
    const int32_t par = parent[c];
    const float4 mn = bmin[par], mx = bmax[par];
    const int axis = info[par] & 3;
    const float sp = split[par];
    if (ch[par].x == c) {
        bmin[c] = make_float4(mn.x, mn.y, mn.z, 0.0f);
        bmax[c] = make_float4(axis == KDGB_X ? sp : mx.x, axis == KDGB_Y ? sp : mx.y, axis == KDGB_Z ? sp : mx.z, 0.0f);
    } else {
        bmin[c] = make_float4(axis == KDGB_X ? sp : mn.x, axis == KDGB_Y ? sp : mn.y, axis == KDGB_Z ? sp : mn.z, 0.0f);
        bmax[c] = make_float4(mx.x, mx.y, mx.z, 0.0f);
    }
}

// PreprocessLeafNodes of the BITMAP creator (TriangleMapBitmapCreator.cu:32-49).
__global__ void k_bitmap_leaves(int32_t nl, const int32_t *__restrict__ leaf_ids, int8_t *info, int32_t *amt)
{
    const int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nl) return;
    const int32_t leaf = leaf_ids[i];
    info[leaf] = KDGB_LEAF;
    amt[leaf] = (int32_t)((1u << amt[leaf]) - 1u);
}

// ---------------------------------------------------------------------------
// Reference SAH lower creator (LowerTriangleMap.h).
// ---------------------------------------------------------------------------

// CalcSurfaceArea (LowerTriangleMap.h:24-38): 0.5 * |e1 x e2|.
__global__ void k_areas(int32_t F, const int32_t *__restrict__ prim_indices, const float4 *__restrict__ p0,
                        const float4 *__restrict__ p1, const float4 *__restrict__ p2, float *__restrict__ areas)
{
    const int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= F) return;
    const int32_t prim = prim_indices[i];
    const float4 a = p0[prim], b = p1[prim], c = p2[prim];
    const float3 v0 = make_float3(a.x, a.y, a.z), v1 = make_float3(b.x, b.y, b.z), v2 = make_float3(c.x, c.y, c.z);
    const float3 cr = cross3(sub3(v1, v0), sub3(v2, v0));
    areas[i] = __fmul_rn(0.5f, __fsqrt_rn(dot3(cr, cr)));
}

// PreprocesLowerNodes (LowerTriangleMap.h:56-81): node area and the bitmap of
// references with non-zero area.
__global__ void k_sah_preprocess(int32_t nl, const int32_t *__restrict__ leaf_ids, const int32_t *__restrict__ pidx,
                                 int32_t *amt, float *area, const float *__restrict__ areas)
{
    const int32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nl) return;
    const int32_t leaf = leaf_ids[k];
    const int32_t pi = pidx[leaf], n = amt[leaf];
    float s = 0.0f;
    unsigned bmp = 0;
    for (int i = 0; i < n; ++i) {
        const float a = areas[pi + i];
        bmp += a > 0.0f ? (1u << i) : 0u;
        s = __fadd_rn(s, a);
    }
    area[leaf] = s;
    amt[leaf] = (int32_t)bmp;
}

// CreateSplittingPlanes (LowerTriangleMap.h:84-155): one warp per node, lane
// i owns reference slot i.  Sets per axis: {lowLeft, lowRight, highLeft,
// highRight} of the planes at slot i's box low / high.
__global__ void k_sah_planes(int32_t nl, const int32_t *__restrict__ leaf_ids, const int32_t *__restrict__ pidx,
                             const int32_t *__restrict__ amt, const float4 *__restrict__ fmin,
                             const float4 *__restrict__ fmax, int64_t F, int4 *__restrict__ sts)
{
    const int64_t gw = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (gw >= nl) return;
    const int32_t leaf = leaf_ids[gw];
    const int32_t pi = pidx[leaf];
    const unsigned bmp = (unsigned)amt[leaf];
    const bool mine = (bmp >> lane) & 1u;
    float4 lo = make_float4(0.f, 0.f, 0.f, 0.f), hi = lo;
    if (mine) { lo = fmin[pi + lane]; hi = fmax[pi + lane]; }
    unsigned sx[4] = {0, 0, 0, 0}, sy[4] = {0, 0, 0, 0}, sz[4] = {0, 0, 0, 0};
    for (int j = 0; j < 32; ++j) {
        const float mnx = __shfl_sync(0xffffffffu, lo.x, j), mny = __shfl_sync(0xffffffffu, lo.y, j);
        const float mnz = __shfl_sync(0xffffffffu, lo.z, j), mxx = __shfl_sync(0xffffffffu, hi.x, j);
        const float mxy = __shfl_sync(0xffffffffu, hi.y, j), mxz = __shfl_sync(0xffffffffu, hi.z, j);
        if (!((bmp >> j) & 1u)) continue;
        const unsigned m = 1u << j;
        sx[0] |= mnx <= lo.x ? m : 0; sx[1] |= lo.x < mxx ? m : 0;
        sx[2] |= mnx <= hi.x ? m : 0; sx[3] |= hi.x < mxx ? m : 0;
        sy[0] |= mny <= lo.y ? m : 0; sy[1] |= lo.y < mxy ? m : 0;
        sy[2] |= mny <= hi.y ? m : 0; sy[3] |= hi.y < mxy ? m : 0;
        sz[0] |= mnz <= lo.z ? m : 0; sz[1] |= lo.z < mxz ? m : 0;
        sz[2] |= mnz <= hi.z ? m : 0; sz[3] |= hi.z < mxz ? m : 0;
    }
    if (mine) {
        sts[pi + lane] = make_int4(sx[0], sx[1], sx[2], sx[3]);
        sts[F + pi + lane] = make_int4(sy[0], sy[1], sy[2], sy[3]);
        sts[2 * F + pi + lane] = make_int4(sz[0], sz[1], sz[2], sz[3]);
    }
}

struct SahPick {
    float cost, la, ra;
    unsigned ls, rs;
    int axis;
    int32_t idx;
};

// CalcAreaForSets (LowerTriangleMap.h:412-461) for one candidate slot.
__device__ __forceinline__ void area_for_sets(int4 set, int axis, int32_t set_index, unsigned bmp,
                                              const float a_lane, SahPick &best)
{
    unsigned s0 = (unsigned)set.x & bmp, s1 = (unsigned)set.y & bmp, s2 = (unsigned)set.z & bmp,
             s3 = (unsigned)set.w & bmp;
    float a0 = 0.0f, a1 = 0.0f, a2 = 0.0f, a3 = 0.0f;
    for (int j = 0; j < 32; ++j) {
        const float aj = __shfl_sync(0xffffffffu, a_lane, j);
        if (!((bmp >> j) & 1u)) continue;
        const unsigned m = 1u << j;
        a0 = __fadd_rn(a0, (s0 & m) ? aj : 0.0f);
        a1 = __fadd_rn(a1, (s1 & m) ? aj : 0.0f);
        a2 = __fadd_rn(a2, (s2 & m) ? aj : 0.0f);
        a3 = __fadd_rn(a3, (s3 & m) ? aj : 0.0f);
    }
    const float low = __fadd_rn(__fmul_rn((float)__popc(s0), a0), __fmul_rn((float)__popc(s1), a1));
    const float high = __fadd_rn(__fmul_rn((float)__popc(s2), a2), __fmul_rn((float)__popc(s3), a3));
    if (low < best.cost) {
        best.cost = low; best.ls = s0; best.rs = s1; best.la = a0; best.ra = a1;
        best.axis = axis; best.idx = set_index;
    }
    if (high < best.cost) {
        best.cost = high; best.ls = s2; best.rs = s3; best.la = a2; best.ra = a3;
        best.axis = axis; best.idx = (int32_t)((unsigned)set_index | 0x80000000u);
    }
}

// CalcSAH (LowerTriangleMap.h:463-555), one warp per node: lane i evaluates
// the six planes of slot i in the reference's order; the warp keeps the
// first minimum in (slot, axis, low/high) order.
__global__ void k_calc_sah(int32_t R, const int32_t *__restrict__ ids, int32_t active, const int32_t *pidx,
                           const int32_t *amt, const float *area, const float *__restrict__ areas,
                           const float4 *__restrict__ fmin, const float4 *__restrict__ fmax,
                           const int4 *__restrict__ sts, int64_t F, float ct, float ci, int32_t min_leaf,
                           int8_t *info, float *split, int32_t *__restrict__ ssplit, float2 *__restrict__ careas,
                           int2 *__restrict__ csets)
{
    const int64_t gw = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (gw >= R) return;
    const int32_t par = ids ? ids[gw] : active + (int32_t)gw;
    const int32_t pi = pidx[par];
    const unsigned bmp = (unsigned)amt[par];
    const bool mine = (bmp >> lane) & 1u;
    const float a_lane = mine ? areas[pi + lane] : 0.0f;
    SahPick best;
    best.cost = KDGB_FINF; best.la = best.ra = 0.0f; best.ls = best.rs = 0; best.axis = 0; best.idx = 0;
    const int4 zero4 = make_int4(0, 0, 0, 0);
    const int4 sx = mine ? sts[pi + lane] : zero4;
    const int4 sy = mine ? sts[F + pi + lane] : zero4;
    const int4 sz = mine ? sts[2 * F + pi + lane] : zero4;
    SahPick mb = best;
    area_for_sets(sx, KDGB_X, pi + lane, bmp, a_lane, mb);
    area_for_sets(sy, KDGB_Y, pi + lane, bmp, a_lane, mb);
    area_for_sets(sz, KDGB_Z, pi + lane, bmp, a_lane, mb);
    if (!mine) mb.cost = KDGB_FINF, mb.idx = -1;
    // Warp argmin on (cost, lane); only lanes whose cost beat fInfinity count.
    float c = mine && mb.cost < KDGB_FINF ? mb.cost : INFINITY;
    int owner = mine && mb.cost < KDGB_FINF ? lane : 32;
    for (int o = 16; o > 0; o >>= 1) {
        const float c2 = __shfl_xor_sync(0xffffffffu, c, o);
        const int w2 = __shfl_xor_sync(0xffffffffu, owner, o);
        if (c2 < c || (c2 == c && w2 < owner)) { c = c2; owner = w2; }
    }
    if (lane != (owner < 32 ? owner : 0)) return;
    const int cnt = __popc(bmp);
    const float opt = owner < 32 ? mb.cost : KDGB_FINF;
    const float node_area = area[par];
    bool do_split = __fmul_rn(ci, opt) < __fmul_rn(__fsub_rn(__fmul_rn(ci, (float)cnt), ct), node_area);
    if (cnt <= min_leaf) do_split = false;
    if (do_split) {
        careas[gw] = make_float2(mb.la, mb.ra);
        csets[gw] = make_int2((int)mb.ls, (int)mb.rs);
        const float4 sp4 = ((unsigned)mb.idx & 0x80000000u) ? fmax[(unsigned)mb.idx ^ 0x80000000u] : fmin[mb.idx];
        split[par] = axis_of4(sp4, mb.axis);
    }
    info[par] = do_split ? (int8_t)mb.axis : (int8_t)KDGB_LEAF;
    ssplit[gw] = do_split;
}

// CreateLowerSAHChildren (LowerTriangleMap.h:557-600) and, when enabled,
// PropagateAabbToChildren (LowerTriangleMap.h:602-636).
__global__ void k_sah_children(int32_t R, const int32_t *__restrict__ ids, int32_t active, int32_t child_base,
                               const int32_t *__restrict__ ssplit, const int32_t *__restrict__ saddr,
                               const float2 *__restrict__ careas, const int2 *__restrict__ csets, int propagate,
                               int8_t *info, float *split, float4 *bmin, float4 *bmax, int32_t *pidx, int32_t *amt,
                               int2 *ch, float *area, int32_t *parent)
{
    const int32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= R || !ssplit[k]) return;
    const int32_t splits = saddr[R];
    const int32_t par = ids ? ids[k] : active + k;
    const int32_t l = child_base + saddr[k], r = l + splits;
    zero_node(l, info, split, bmin, bmax, pidx, amt, ch, area, parent);
    zero_node(r, info, split, bmin, bmax, pidx, amt, ch, area, parent);
    const float2 ca = careas[k];
    const int2 cs = csets[k];
    area[l] = ca.x; pidx[l] = pidx[par]; amt[l] = cs.x;
    area[r] = ca.y; pidx[r] = pidx[par]; amt[r] = cs.y;
    ch[par] = make_int2(l, r);
    if (propagate) {
        const int axis = info[par] & 3;
        const float sp = split[par];
        const float4 mn = bmin[par], mx = bmax[par];
        bmin[l] = mn;
        bmin[r] = make_float4(axis == KDGB_X ? sp : mn.x, axis == KDGB_Y ? sp : mn.y, axis == KDGB_Z ? sp : mn.z, 0.0f);
        bmax[l] = make_float4(axis == KDGB_X ? sp : mx.x, axis == KDGB_Y ? sp : mx.y, axis == KDGB_Z ? sp : mx.z, 0.0f);
        bmax[r] = mx;
    }
}

// ---------------------------------------------------------------------------
// Host side.
// ---------------------------------------------------------------------------

struct Pinned {
    int32_t *p = nullptr;
    ~Pinned() { if (p) cudaFreeHost(p); }
};

template <class T>
struct Scratch {
    T *p = nullptr;
    cudaStream_t s = 0;
    ~Scratch() { if (p) cudaFreeAsync(p, s); }
};

template <class T>
int alloc_scratch(Scratch<T> &a, int64_t n, cudaStream_t s)
{
    if (a.p) { cudaFreeAsync(a.p, s); a.p = nullptr; }
    a.s = s;
    KDGB_CUDA(cudaMallocAsync(&a.p, sizeof(T) * (size_t)(n > 0 ? n : 1), s));
    return KDGB_OK;
}

int grow_nodes(Tree &t, int64_t need, cudaStream_t s)
{
    const int64_t keep = t.n_nodes;
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

#define NODE_ARGS t.info.p, t.split.p, t.bmin.p, t.bmax.p, t.pidx.p, t.bitmap.p, t.children.p, t.area.p, t.parent.p

int lower_sah(Tree &t, const kdgb_build_params &p, const float4 *fmin, const float4 *fmax, int32_t F,
              cudaStream_t s, int32_t *host_rec)
{
    const int32_t nl = t.n_upper_leaves;
    Scratch<float> areas;
    Scratch<int4> sts;
    KDGB_CHECK(alloc_scratch(areas, F, s));
    KDGB_CHECK(alloc_scratch(sts, 3 * (int64_t)F, s));
    if (F > 0) {
        k_areas<<<blocks_for(F), kBlock, 0, s>>>(F, t.prim_indices.p, t.p0.p, t.p1.p, t.p2.p, areas.p);
        KDGB_LAUNCH_CHECK();
    }
    if (nl > 0) {
        k_sah_preprocess<<<blocks_for(nl), kBlock, 0, s>>>(nl, t.leaf_ids.p, t.pidx.p, t.bitmap.p, t.area.p, areas.p);
        KDGB_LAUNCH_CHECK();
        k_sah_planes<<<blocks_for((int64_t)nl * 32), kBlock, 0, s>>>(nl, t.leaf_ids.p, t.pidx.p, t.bitmap.p, fmin,
                                                                   fmax, F, sts.p);
        KDGB_LAUNCH_CHECK();
    }
    int32_t R = nl, active = t.n_nodes, lv = 0;
    const int32_t *ids = t.leaf_ids.p;
    Scratch<int32_t> ssplit, saddr;
    Scratch<float2> careas;
    Scratch<int2> csets;
    while (R > 0) {
        ++lv;
        KDGB_CHECK(alloc_scratch(ssplit, R, s));
        KDGB_CHECK(alloc_scratch(saddr, R + 1, s));
        KDGB_CHECK(alloc_scratch(careas, R, s));
        KDGB_CHECK(alloc_scratch(csets, R, s));
        k_calc_sah<<<blocks_for((int64_t)R * 32), kBlock, 0, s>>>(
            R, ids, active, t.pidx.p, t.bitmap.p, t.area.p, areas.p, fmin, fmax, sts.p, F, p.traversal_cost,
            p.intersection_cost, p.min_leaf, t.info.p, t.split.p, ssplit.p, careas.p, csets.p);
        KDGB_LAUNCH_CHECK();
        KDGB_CHECK(scan_exclusive<1>(ssplit.p, saddr.p, R, s));
        KDGB_CUDA(cudaMemcpyAsync(host_rec, saddr.p + R, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
        KDGB_CUDA(cudaStreamSynchronize(s));
        const int32_t splits = host_rec[0];
        const int32_t child_base = t.n_nodes;
        KDGB_CHECK(grow_nodes(t, (int64_t)t.n_nodes + 2 * (int64_t)splits, s));
        if (splits > 0) {
            k_sah_children<<<blocks_for(R), kBlock, 0, s>>>(R, ids, active, child_base, ssplit.p, saddr.p, careas.p,
                                                           csets.p, p.propagate_aabbs, NODE_ARGS);
            KDGB_LAUNCH_CHECK();
        }
        t.n_nodes += 2 * splits;
        ids = nullptr;
        active = t.n_nodes - 2 * splits;
        R = 2 * splits;
    }
    t.stats.lower_levels = lv;
    return KDGB_OK;
}

}  // namespace

int load_geometry(Tree &t, const float *tri_v_dev, int32_t T, cudaStream_t s)
{
    KDGB_CHECK(ensure(t.p0, T, s));
    KDGB_CHECK(ensure(t.p1, T, s));
    KDGB_CHECK(ensure(t.p2, T, s));
    t.n_tris = T;
    if (T == 0) return KDGB_OK;
    Scratch<int> err;
    KDGB_CHECK(alloc_scratch(err, 1, s));
    KDGB_CUDA(cudaMemsetAsync(err.p, 0, sizeof(int), s));
    k_load_geometry<<<blocks_for(T), kBlock, 0, s>>>(tri_v_dev, T, t.p0.p, t.p1.p, t.p2.p, nullptr, nullptr, err.p);
    KDGB_LAUNCH_CHECK();
    int h = 0;
    KDGB_CUDA(cudaMemcpyAsync(&h, err.p, sizeof(int), cudaMemcpyDeviceToHost, s));
    KDGB_CUDA(cudaStreamSynchronize(s));
    if (h) return fail(KDGB_ERR_NONFINITE, "non-finite vertex coordinate");
    return KDGB_OK;
}

int build_reference(Tree &t, const float *tri_v_dev, int32_t T, const kdgb_build_params &p, cudaStream_t s)
{
    const int32_t LS = p.leaf_size;
    Pinned rec;
    KDGB_CUDA(cudaMallocHost(&rec.p, 16 * sizeof(int32_t)));

    // Geometry, primitive boxes and the root node.
    KDGB_CHECK(ensure(t.p0, T, s));
    KDGB_CHECK(ensure(t.p1, T, s));
    KDGB_CHECK(ensure(t.p2, T, s));
    t.n_tris = T;
    Scratch<float4> cmin, cmax, nmin, nmax, fmin, fmax;
    KDGB_CHECK(alloc_scratch(cmin, T, s));
    KDGB_CHECK(alloc_scratch(cmax, T, s));
    Scratch<int32_t> stats;
    KDGB_CHECK(alloc_scratch(stats, 16, s));
    KDGB_CUDA(cudaMemsetAsync(stats.p, 0, 16 * sizeof(int32_t), s));
    if (T > 0) {
        k_load_geometry<<<blocks_for(T), kBlock, 0, s>>>(tri_v_dev, T, t.p0.p, t.p1.p, t.p2.p, cmin.p, cmax.p,
                                                        stats.p + 15);
        KDGB_LAUNCH_CHECK();
    }
    t.n_nodes = 0;
    KDGB_CHECK(grow_nodes(t, 1, s));
    k_init_root<<<1, 32, 0, s>>>(T, NODE_ARGS);
    KDGB_LAUNCH_CHECK();
    t.n_nodes = 1;

    int64_t N = T, F = 0, fcap = 0;
    int32_t active = 0, R = 1, level = 0;
    std::vector<int2> leaf_ranges;
    std::vector<int32_t> leaf_off;
    int32_t n_leaf_ids = 0;

    Scratch<float4> pmin, pmax;
    Scratch<unsigned> keys;
    Scratch<int8_t> planes;
    Scratch<int32_t> req, eaddr, cnt, lanes, lbase, blocksum, blockoff;

    while (R > 0) {
        if (level >= p.max_levels) return fail(KDGB_ERR_DEGENERATE, "upper build exceeded max_levels");
        ++level;
        const bool do_ess = p.split_empty_space && active != 0;
        const int64_t nb = (N + kBlock - 1) / kBlock;
        KDGB_CHECK(grow_nodes(t, (int64_t)t.n_nodes + 14 * (int64_t)R, s));
        KDGB_CHECK(alloc_scratch(pmin, R, s));
        KDGB_CHECK(alloc_scratch(pmax, R, s));
        KDGB_CHECK(alloc_scratch(keys, 6 * (int64_t)R, s));
        KDGB_CHECK(alloc_scratch(cnt, 2 * (int64_t)R, s));
        KDGB_CHECK(alloc_scratch(lanes, 6 * (int64_t)R, s));
        KDGB_CHECK(alloc_scratch(lbase, 6 * ((int64_t)R + 1), s));
        KDGB_CHECK(alloc_scratch(blocksum, 2 * nb, s));
        KDGB_CHECK(alloc_scratch(blockoff, 2 * (nb + 1), s));
        KDGB_CHECK(alloc_scratch(nmin, 2 * N, s));
        KDGB_CHECK(alloc_scratch(nmax, 2 * N, s));
        if (F + 2 * N > fcap) {
            const int64_t ncap = (F + 2 * N) * 3 / 2 + 1024;
            Scratch<float4> a, b;
            KDGB_CHECK(alloc_scratch(a, ncap, s));
            KDGB_CHECK(alloc_scratch(b, ncap, s));
            if (F > 0) {
                KDGB_CUDA(cudaMemcpyAsync(a.p, fmin.p, sizeof(float4) * F, cudaMemcpyDeviceToDevice, s));
                KDGB_CUDA(cudaMemcpyAsync(b.p, fmax.p, sizeof(float4) * F, cudaMemcpyDeviceToDevice, s));
            }
            std::swap(a.p, fmin.p);
            std::swap(b.p, fmax.p);
            fmin.s = fmax.s = s;
            fcap = ncap;
        }

        k_level_init<<<blocks_for(R), kBlock, 0, s>>>(R, active, t.bmin.p, t.bmax.p, pmin.p, pmax.p, keys.p, cnt.p);
        KDGB_LAUNCH_CHECK();
        if (N > 0) {
            k_reduce<<<(unsigned)nb, kBlock, 0, s>>>(N, cmin.p, cmax.p, keys.p);
            KDGB_LAUNCH_CHECK();
        }
        if (do_ess) {
            KDGB_CHECK(alloc_scratch(planes, R, s));
            KDGB_CHECK(alloc_scratch(req, R, s));
            KDGB_CHECK(alloc_scratch(eaddr, (int64_t)R + 1, s));
        }
        k_node_split<<<blocks_for(R), kBlock, 0, s>>>(R, active, do_ess, p.empty_space_threshold, pmin.p, pmax.p,
                                                      keys.p, t.bmin.p, t.bmax.p, t.split.p, t.info.p,
                                                      do_ess ? planes.p : nullptr, do_ess ? req.p : nullptr);
        KDGB_LAUNCH_CHECK();
        if (do_ess) {
            KDGB_CHECK(scan_exclusive<1>(req.p, eaddr.p, R, s));
            k_ess_chain<<<blocks_for(R), kBlock, 0, s>>>(R, active, t.n_nodes, p.esc_zmax_as_x, planes.p, eaddr.p,
                                                         NODE_ARGS);
            KDGB_LAUNCH_CHECK();
        }
        if (N > 0) {
            k_count<<<(unsigned)nb, kBlock, 0, s>>>(N, active, cmin.p, cmax.p, t.split.p, t.info.p, cnt.p,
                                                    blocksum.p);
            KDGB_LAUNCH_CHECK();
        }
        KDGB_CHECK(scan_exclusive<2>(blocksum.p, blockoff.p, nb, s));
        k_node_lanes<<<blocks_for(R), kBlock, 0, s>>>(R, LS, cnt.p, lanes.p);
        KDGB_LAUNCH_CHECK();
        KDGB_CHECK(scan_exclusive<6>(lanes.p, lbase.p, R, s));
        if (N > 0) {
            k_scatter<<<(unsigned)nb, kBlock, 0, s>>>(N, R, active, LS, (int32_t)F, cmin.p, cmax.p, t.split.p,
                                                      t.info.p, blockoff.p, lbase.p, nmin.p, nmax.p, fmin.p, fmax.p);
            KDGB_LAUNCH_CHECK();
        }
        k_children<<<blocks_for(R), kBlock, 0, s>>>(R, active, t.n_nodes, do_ess ? eaddr.p + R : nullptr, LS,
                                                    (int32_t)F, p.split_empty_space, lbase.p, NODE_ARGS, stats.p);
        KDGB_LAUNCH_CHECK();
        KDGB_CUDA(cudaMemcpyAsync(rec.p, stats.p, 16 * sizeof(int32_t), cudaMemcpyDeviceToHost, s));
        KDGB_CUDA(cudaStreamSynchronize(s));
        if (rec.p[15]) return fail(KDGB_ERR_NONFINITE, "non-finite vertex coordinate");

        const int32_t empty = rec.p[0];
        const int64_t total_l = rec.p[1], total_r = rec.p[2], leaf_l = rec.p[3], leaf_r = rec.p[4];
        const int32_t leaf_nodes = rec.p[5] + rec.p[6];
        if (total_l + total_r < N) return fail(KDGB_ERR_DEGENERATE, "split produced fewer references than its input");
        const int32_t child_start = t.n_nodes + empty;
        if (leaf_nodes > 0) {
            leaf_ranges.push_back(make_int2(child_start, leaf_nodes));
            leaf_off.push_back(n_leaf_ids);
            n_leaf_ids += leaf_nodes;
        }
        t.n_nodes += empty + 2 * R;
        F += leaf_l + leaf_r;
        const int32_t created = 2 * R - leaf_nodes;
        std::swap(cmin.p, nmin.p);
        std::swap(cmax.p, nmax.p);
        N = total_l + total_r - leaf_l - leaf_r;
        active = t.n_nodes - created;
        R = created;
    }
    t.stats.upper_levels = level;

    // Leaf ids, final reference indices.
    t.n_upper_leaves = n_leaf_ids;
    t.n_refs = (int32_t)F;
    KDGB_CHECK(ensure(t.leaf_ids, n_leaf_ids, s));
    KDGB_CHECK(ensure(t.prim_indices, F, s));
    if (n_leaf_ids > 0) {
        const int nr = (int)leaf_ranges.size();
        Scratch<int2> dr;
        Scratch<int32_t> doff;
        KDGB_CHECK(alloc_scratch(dr, nr, s));
        KDGB_CHECK(alloc_scratch(doff, nr, s));
        KDGB_CUDA(cudaMemcpyAsync(dr.p, leaf_ranges.data(), sizeof(int2) * nr, cudaMemcpyHostToDevice, s));
        KDGB_CUDA(cudaMemcpyAsync(doff.p, leaf_off.data(), sizeof(int32_t) * nr, cudaMemcpyHostToDevice, s));
        k_leaf_ids<<<blocks_for(n_leaf_ids), kBlock, 0, s>>>(dr.p, nr, doff.p, n_leaf_ids, t.leaf_ids.p);
        KDGB_LAUNCH_CHECK();
        KDGB_CUDA(cudaStreamSynchronize(s));  // host tables go out of scope
    }
    if (F > 0) {
        k_extract_indices<<<blocks_for(F), kBlock, 0, s>>>((int32_t)F, fmin.p, t.prim_indices.p);
        KDGB_LAUNCH_CHECK();
    }
    if (!p.split_empty_space && p.propagate_aabbs && n_leaf_ids > 0) {
        k_propagate_parent<<<blocks_for(n_leaf_ids), kBlock, 0, s>>>(n_leaf_ids, t.leaf_ids.p, t.info.p, t.split.p,
                                                                     t.bmin.p, t.bmax.p, t.parent.p, t.children.p);
        KDGB_LAUNCH_CHECK();
    }

    t.stats.lower_levels = 0;
    if (p.lower == KDGB_LOWER_SAH) {
        KDGB_CHECK(lower_sah(t, p, fmin.p, fmax.p, (int32_t)F, s, rec.p));
    } else if (n_leaf_ids > 0) {
        k_bitmap_leaves<<<blocks_for(n_leaf_ids), kBlock, 0, s>>>(n_leaf_ids, t.leaf_ids.p, t.info.p, t.bitmap.p);
        KDGB_LAUNCH_CHECK();
    }
    return KDGB_OK;
}

}  // namespace kdgb
