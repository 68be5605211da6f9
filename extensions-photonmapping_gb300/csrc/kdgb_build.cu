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

#include <cstring>
#include <vector>

#include "kdgb_internal.cuh"

namespace kdgb {

namespace {

constexpr int kBlock = 256;

inline unsigned blocks_for(int64_t n, int b = kBlock) { return (unsigned)((n + b - 1) / b); }

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
                                int *__restrict__ err, const int32_t *__restrict__ mesh_off = nullptr, int M = 1)
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
        // w carries the local index of the owning active node: the root of
        // the triangle's mesh (0 for a single mesh).
        const int owner = M > 1 ? mesh_of(mesh_off, M, i) : 0;
        cmax[i] = make_float4(kmax(mxx, v[6]), kmax(mxy, v[7]), kmax(mxz, v[8]), __int_as_float(owner));
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

// Roots (TriangleMapUpperCreator.cu:128-136): node m is the root of mesh m,
// covering references [off[m], off[m+1]) (a single mesh: node 0, all of them).
__global__ void k_init_roots(int32_t T, int M, const int32_t *__restrict__ mesh_off, int8_t *info, float *split,
                             float4 *bmin, float4 *bmax, int32_t *pidx, int32_t *amt, int2 *ch, float *area,
                             int32_t *parent)
{
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= M) return;
    zero_node(m, info, split, bmin, bmax, pidx, amt, ch, area, parent);
    const int32_t a = M > 1 ? mesh_off[m] : 0, b = M > 1 ? mesh_off[m + 1] : T;
    pidx[m] = a;
    amt[m] = b - a;
    parent[m] = m;
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

// The per-reference passes (k_reduce, k_count, k_scatter) walk the reference
// array in warp chunks of kRows rows of 32 consecutive references.  Owners
// are sorted, so most rows belong to one node: a warp keeps per-lane
// accumulators while the owner stays the same and only reduces and issues
// atomics when it changes, which keeps atomic traffic to a few per node per
// chunk even at the root, where every reference has the same owner.
constexpr int kRows = 4;
constexpr int kChunk = 32 * kRows;                   // references per warp
constexpr int kWarps = kBlock / 32;
constexpr int kLanes = 7;  // per-node scan lanes (see k_node_lanes)
constexpr unsigned kFull = 0xffffffffu;

inline int64_t chunks_for(int64_t n) { return (n + kChunk - 1) / kChunk; }
inline unsigned chunk_blocks(int64_t nch) { return (unsigned)((nch + kWarps - 1) / kWarps); }

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

// Tight node boxes: exact min/max over each node's references, as the
// segmented reduction ReduceSegmentsUnrolled + FinalSegmentedReduce
// (ReduceSegments.h:230-371) computes.  Keys are order-preserving uint32
// images of the floats, so atomicMin/atomicMax give exact results in any order.
__global__ void __launch_bounds__(kBlock) k_reduce(int64_t N, const float4 *__restrict__ cmin,
                                                  const float4 *__restrict__ cmax,
                                                  unsigned *__restrict__ keys)
{
    __shared__ int s_owner[kWarps];
    __shared__ unsigned s_keys[kWarps][6];
    const unsigned lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int64_t base = (((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5) * kChunk;
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
            const float4 a = ra[row], b = rb[row];
            k[0] = fkey(a.x); k[1] = fkey(a.y); k[2] = fkey(a.z);
            k[3] = fkey(b.x); k[4] = fkey(b.y); k[5] = fkey(b.z);
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
}

// Writes the tight boxes, the empty-space planes (CalcEmptySpaceSplits,
// EmptySpaceSplitting.h:10-70) and the spatial-median split of the longest
// axis (CalcUpperNodeSplitInfo, ReduceSegments.h:466-484).
__global__ void k_node_split(int32_t R, int32_t active, int do_ess, float thr,
                             const float4 *__restrict__ pmin, const float4 *__restrict__ pmax,
                             const unsigned *__restrict__ keys, float4 *__restrict__ bmin,
                             float4 *__restrict__ bmax, float *__restrict__ split, int8_t *__restrict__ info,
                             int8_t *__restrict__ planes, int32_t *__restrict__ lanes)
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
        lanes[kLanes * (int64_t)k + 6] = nr;
    } else {
        lanes[kLanes * (int64_t)k + 6] = 0;
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

__device__ __forceinline__ void ref_flags(const float4 &a, const float4 &b, int axis, float sp, int &L, int &Rf)
{
    // SetSplitSide (TriangleUpperChildren.h:10-62): left = min <= split,
    // right = split < max.
    L = axis_of4(a, axis) <= sp;
    Rf = sp < axis_of4(b, axis);
}

// Per-node left/right counts and per-chunk totals of the flags (the chunk
// totals are scanned into each warp chunk's global offsets for k_scatter).
__global__ void __launch_bounds__(kBlock) k_count(int64_t N, int32_t active, const float4 *__restrict__ cmin,
                                                 const float4 *__restrict__ cmax, const float *__restrict__ split,
                                                 const int8_t *__restrict__ info, int32_t *__restrict__ cnt,
                                                 int32_t *__restrict__ chunksum)
{
    __shared__ int s_owner[kWarps], s_l[kWarps], s_r[kWarps];
    const unsigned lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int64_t chunk = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
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
        ax[row] = o >= 0 ? info[active + o] : 0;
        sp[row] = o >= 0 ? split[active + o] : 0.0f;
    }
#pragma unroll
    for (int row = 0; row < kRows; ++row) {
        if (base + row * 32 >= N) break;
        const int o = __float_as_int(rb[row].w);
        int L = 0, Rf = 0;
        if (o >= 0) ref_flags(ra[row], rb[row], ax[row], sp[row], L, Rf);
        tl += L;
        tr += Rf;
        const unsigned m = __match_any_sync(kFull, o);
        if (m == kFull && o == cw) {
            al += L;
            ar += Rf;
            continue;
        }
        if (cw >= 0) {
            al = __reduce_add_sync(kFull, al);
            ar = __reduce_add_sync(kFull, ar);
            if (lane == 0) { atomicAdd(cnt + 2 * cw, al); atomicAdd(cnt + 2 * cw + 1, ar); }
        }
        if (m == kFull && o >= 0) {
            cw = o; al = L; ar = Rf;
        } else {
            if (o >= 0) {
                const int gl = __reduce_add_sync(m, L), gr = __reduce_add_sync(m, Rf);
                if (lane == (unsigned)(__ffs(m) - 1)) { atomicAdd(cnt + 2 * o, gl); atomicAdd(cnt + 2 * o + 1, gr); }
            }
            cw = -1; al = 0; ar = 0;
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
            chunksum[2 * chunk] = tl;
            chunksum[2 * chunk + 1] = tr;
        }
        s_owner[warp] = cw;
        s_l[warp] = al;
        s_r[warp] = ar;
    }
    __syncthreads();
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
    int32_t *o = lanes + kLanes * (int64_t)k;
    o[0] = l; o[1] = r; o[2] = ll ? l : 0; o[3] = rl ? r : 0; o[4] = ll; o[5] = rl;
}

// ---------------------------------------------------------------------------
// Tuned mode: binned SAH for the upper levels below `upper_levels` (new in
// this build; the reference splits every upper level at the median).  Per
// node and axis with extent > 0: B equal bins over the tight box; each
// reference adds 1 to the bin of its box min (left histogram) and of its box
// max (right histogram).  The plane at bin boundary k has NL = left counts
// below k, NR = right counts from k up and cost AL*NL + AR*NR (half box
// areas); the first strict minimum over (axis X,Y,Z; k = 1..B-1) wins,
// skipping planes that leave a side empty or keep every reference on both
// sides; without a qualifying plane the median split stays.
// ---------------------------------------------------------------------------

__device__ __forceinline__ int sah_bin(float x, float mn, float scale, int B)
{
    const int b = (int)__fmul_rn(__fsub_rn(x, mn), scale);
    return b < 0 ? 0 : (b > B - 1 ? B - 1 : b);
}

// Histograms hist[((node * 3 + axis) * 2 + side) * B + bin]; lanes of a
// warp with the same (owner, axis, side, bin) add once.
__global__ void __launch_bounds__(kBlock) k_sah_bin(int64_t N, int32_t active, int B, const float4 *__restrict__ cmin,
                                                   const float4 *__restrict__ cmax, const float4 *__restrict__ bmin,
                                                   const float4 *__restrict__ bmax, int32_t *__restrict__ hist)
{
    const unsigned lane = threadIdx.x & 31;
    const int64_t base = (((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5) * kChunk;
    for (int row = 0; row < kRows; ++row) {
        if (base + row * 32 >= N) break;
        const int64_t r = base + row * 32 + lane;
        int o = -1;
        float4 a = make_float4(0.f, 0.f, 0.f, 0.f), b = a, mn = a, mx = a;
        if (r < N) {
            a = cmin[r];
            b = cmax[r];
            o = __float_as_int(b.w);
            mn = bmin[active + o];
            mx = bmax[active + o];
        }
        for (int ax = 0; ax < 3; ++ax) {
            const float lo = ax == 0 ? mn.x : (ax == 1 ? mn.y : mn.z);
            const float ext = __fsub_rn(ax == 0 ? mx.x : (ax == 1 ? mx.y : mx.z), lo);
            const bool valid = o >= 0 && ext > 0.0f;
            const float scale = valid ? __fdiv_rn((float)B, ext) : 0.0f;
            for (int side = 0; side < 2; ++side) {
                const float4 &src = side == 0 ? a : b;
                const float x = ax == 0 ? src.x : (ax == 1 ? src.y : src.z);
                const int bin = valid ? sah_bin(x, lo, scale, B) : 0;
                // Key: (owner, bin); invalid lanes get a key no valid lane has.
                const long long key = valid ? ((long long)o << 8 | bin) : -1ll;
                const unsigned m = __match_any_sync(kFull, key);
                if (valid && lane == (unsigned)(__ffs(m) - 1))
                    atomicAdd(hist + (((int64_t)o * 3 + ax) * 2 + side) * B + bin, __popc(m));
            }
        }
    }
}

// One warp per node, lane k-1 evaluates the plane at bin boundary k.
__global__ void k_sah_split(int32_t R, int32_t active, int B, const float4 *__restrict__ bmin,
                            const float4 *__restrict__ bmax, const int32_t *__restrict__ amt,
                            const int32_t *__restrict__ hist, float *__restrict__ split, int8_t *__restrict__ info)
{
    const int64_t gw = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (gw >= R) return;
    const int32_t node = active + (int32_t)gw;
    const int32_t a = amt[node];
    const float4 mn4 = bmin[node], mx4 = bmax[node];
    const float mnv[3] = {mn4.x, mn4.y, mn4.z}, mxv[3] = {mx4.x, mx4.y, mx4.z};
    const float ext[3] = {__fsub_rn(mxv[0], mnv[0]), __fsub_rn(mxv[1], mnv[1]), __fsub_rn(mxv[2], mnv[2])};
    float best = INFINITY, best_sp = 0.0f;
    int best_ax = -1;
    for (int ax = 0; ax < 3; ++ax) {
        if (!(ext[ax] > 0.0f)) continue;  // warp-uniform
        const int32_t *h = hist + ((int64_t)gw * 3 + ax) * 2 * B;
        const int32_t lo = lane < B ? h[lane] : 0, hi = lane < B ? h[B + lane] : 0;
        int32_t plo = lo, phi = hi;  // inclusive prefix sums over bins
        for (int s = 1; s < 32; s <<= 1) {
            const int32_t x = __shfl_up_sync(kFull, plo, s), y = __shfl_up_sync(kFull, phi, s);
            if (lane >= s) { plo += x; phi += y; }
        }
        const int32_t total_hi = __shfl_sync(kFull, phi, 31);
        const int k = lane + 1;
        float cost = INFINITY, pk = 0.0f;
        if (k < B) {
            const int32_t nl = plo, nr = total_hi - phi;
            const float w = __fdiv_rn(ext[ax], (float)B);
            pk = __fadd_rn(mnv[ax], __fmul_rn((float)k, w));
            float le[3] = {ext[0], ext[1], ext[2]}, re[3] = {ext[0], ext[1], ext[2]};
            le[ax] = __fsub_rn(pk, mnv[ax]);
            re[ax] = __fsub_rn(mxv[ax], pk);
            const float al = __fadd_rn(__fadd_rn(__fmul_rn(le[0], le[1]), __fmul_rn(le[1], le[2])), __fmul_rn(le[2], le[0]));
            const float ar = __fadd_rn(__fadd_rn(__fmul_rn(re[0], re[1]), __fmul_rn(re[1], re[2])), __fmul_rn(re[2], re[0]));
            const float c = __fadd_rn(__fmul_rn(al, (float)nl), __fmul_rn(ar, (float)nr));
            if (nl > 0 && nr > 0 && !(nl == a && nr == a)) cost = c;
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
        info[node] = (int8_t)(best_ax + 1);
        split[node] = best_sp;
    }
}

// Writes one reference to its child (or final leaf) slot: destination = node
// base + rank among the node's left (right) references.
__device__ __forceinline__ void scatter_one(int32_t R, int owner, int32_t LS, int32_t upper, int L, int Rf, int axis,
                                            float sp, float4 a, float4 b, int32_t pl, int32_t pr,
                                            const int32_t *__restrict__ lbase, float4 *__restrict__ nmin,
                                            float4 *__restrict__ nmax, float4 *__restrict__ fmin,
                                            float4 *__restrict__ fmax)
{
    const int32_t *lb = lbase + kLanes * (int64_t)owner;
    const int32_t *tot = lbase + kLanes * (int64_t)R;
    const int32_t total_l = tot[0], leaf_l = tot[2], leafnodes_l = tot[4];
    if (L) {
        const int32_t rank = pl - lb[0];
        const float4 hi = make_float4(axis == KDGB_X ? kmin(sp, b.x) : b.x, axis == KDGB_Y ? kmin(sp, b.y) : b.y,
                                      axis == KDGB_Z ? kmin(sp, b.z) : b.z, 0.0f);
        const int32_t lcount = (lbase + kLanes * (int64_t)(owner + 1))[0] - lb[0];
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
        const int32_t rcount = (lbase + kLanes * (int64_t)(owner + 1))[1] - lb[1];
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

// Partition + compaction of the references with clipping to the split plane
// (SplitTriangles, TriangleUpperChildren.h:283-383).  Destination = node base
// + rank of the reference among the node's left (right) references.
__global__ void __launch_bounds__(kBlock) k_scatter(
    int64_t N, int32_t R, int32_t active, int32_t LS, int32_t upper,
    const float4 *__restrict__ cmin, const float4 *__restrict__ cmax, const float *__restrict__ split,
    const int8_t *__restrict__ info, const int32_t *__restrict__ chunkoff, const int32_t *__restrict__ lbase,
    float4 *__restrict__ nmin, float4 *__restrict__ nmax, float4 *__restrict__ fmin, float4 *__restrict__ fmax)
{
    const unsigned lane = threadIdx.x & 31;
    const int64_t chunk = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t base = chunk * kChunk;
    if (base >= N) return;  // warp-uniform
    const unsigned below = (1u << lane) - 1u;
    int32_t off_l = chunkoff[2 * chunk], off_r = chunkoff[2 * chunk + 1];
    float4 ra[kRows], rb[kRows];
#pragma unroll
    for (int row = 0; row < kRows; ++row) {
        const int64_t r = base + row * 32 + lane;
        if (r < N) { ra[row] = cmin[r]; rb[row] = cmax[r]; }
        else { rb[row].w = __int_as_float(-1); }
    }
    int ax[kRows];
    float sps[kRows];
#pragma unroll
    for (int row = 0; row < kRows; ++row) {
        const int o = __float_as_int(rb[row].w);
        ax[row] = o >= 0 ? info[active + o] : 0;
        sps[row] = o >= 0 ? split[active + o] : 0.0f;
    }
#pragma unroll
    for (int row = 0; row < kRows; ++row) {
        if (base + row * 32 >= N) break;
        const int owner = __float_as_int(rb[row].w);
        const int axis = ax[row];
        const float sp = sps[row];
        const float4 a = ra[row], b = rb[row];
        int L = 0, Rf = 0;
        if (owner >= 0) ref_flags(a, b, axis, sp, L, Rf);
        const unsigned bl = __ballot_sync(kFull, L), br = __ballot_sync(kFull, Rf);
        const int32_t pl = off_l + __popc(bl & below), pr = off_r + __popc(br & below);
        off_l += __popc(bl);
        off_r += __popc(br);
        if (owner >= 0) scatter_one(R, owner, LS, upper, L, Rf, axis, sp, a, b, pl, pr, lbase, nmin, nmax, fmin, fmax);
    }
}

// EmptySpaceSplitting2 (EmptySpaceSplitting.h:74-184): a chain of split
// nodes, each with an empty leaf, between the parent and the active node.
__device__ __forceinline__ void ess_chain(int32_t k, int32_t active, int32_t start, int pl, int zmax_as_x,
                                          int8_t *info, float *split, float4 *bmin, float4 *bmax, int32_t *pidx,
                                          int32_t *amt, int2 *ch, float *area, int32_t *parent)
{
    const int32_t leaf = active + k;
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

// CreateUpperChildren (TriangleUpperChildren.h:203-281), the empty-space
// chain of EmptySpaceSplitting2 (its nodes come first, at base + lane-6
// offsets) and, with empty-space splitting on, PropagateAabbToChildren
// (EmptySpaceSplitting.h:299-331).  Non-leaf children are the next level's
// active nodes: their tight-box keys, counts and propagated boxes are reset
// here (AabbMemset, ReduceSegments.h:328-335) so the next level needs no
// separate init launch.
__global__ void k_children(int32_t R, int32_t active, int32_t base, int do_ess, int zmax_as_x, int32_t LS,
                           int32_t upper, int propagate, const int8_t *__restrict__ planes,
                           const int32_t *__restrict__ lbase, int8_t *info, float *split, float4 *bmin,
                           float4 *bmax, int32_t *pidx, int32_t *amt, int2 *ch, float *area, int32_t *parent,
                           int32_t *stats, unsigned *__restrict__ next_keys, int32_t *__restrict__ next_cnt,
                           float4 *__restrict__ next_pmin, float4 *__restrict__ next_pmax)
{
    const int32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    const int32_t *tot = lbase + kLanes * (int64_t)R;
    const int32_t empty = tot[6];
    if (k == 0) {
        stats[0] = empty;
        for (int j = 0; j < 6; ++j) stats[1 + j] = tot[j];
    }
    if (k >= R) return;
    const int32_t *lb = lbase + kLanes * (int64_t)k;
    const int32_t *nb = lbase + kLanes * (int64_t)(k + 1);
    if (do_ess) {
        const int pl = planes[k];
        if (pl) ess_chain(k, active, base + lb[6], pl, zmax_as_x, info, split, bmin, bmax, pidx, amt, ch, area, parent);
    }
    const int32_t child_start = base + empty;
    const int32_t total_l = tot[0], leaf_l = tot[2], ln_l = tot[4], leaf_nodes = tot[4] + tot[5];
    const int32_t l = nb[0] - lb[0], r = nb[1] - lb[1];
    const int32_t par = active + k;

    const bool lleaf = l < LS;
    const int32_t la = lb[4];
    const int32_t lnext = k - la;
    const int32_t lid = child_start + (lleaf ? la : lnext + leaf_nodes);
    const bool rleaf = r < LS;
    const int32_t ra = ln_l + lb[5];
    const int32_t rnext = (R + k) - ra;
    const int32_t rid = child_start + (rleaf ? ra : rnext + leaf_nodes);

    zero_node(lid, info, split, bmin, bmax, pidx, amt, ch, area, parent);
    zero_node(rid, info, split, bmin, bmax, pidx, amt, ch, area, parent);
    pidx[lid] = lleaf ? upper + lb[2] : lb[0] - lb[2];
    pidx[rid] = rleaf ? upper + leaf_l + lb[3] : (total_l - leaf_l) + (lb[1] - lb[3]);
    amt[lid] = l;
    amt[rid] = r;
    parent[lid] = par;
    parent[rid] = par;
    ch[par] = make_int2(lid, rid);
    float4 lmin = make_float4(0.f, 0.f, 0.f, 0.f), lmax = lmin, rmin = lmin, rmax = lmin;
    if (propagate) {
        const int axis = info[par] & 3;
        const float sp = split[par];
        const float4 mn = bmin[par], mx = bmax[par];
        lmin = mn;
        rmin = make_float4(axis == KDGB_X ? sp : mn.x, axis == KDGB_Y ? sp : mn.y, axis == KDGB_Z ? sp : mn.z, 0.0f);
        lmax = make_float4(axis == KDGB_X ? sp : mx.x, axis == KDGB_Y ? sp : mx.y, axis == KDGB_Z ? sp : mx.z, 0.0f);
        rmax = mx;
        bmin[lid] = lmin;
        bmin[rid] = rmin;
        bmax[lid] = lmax;
        bmax[rid] = rmax;
    }
    const unsigned lo = fkey(KDGB_FINF), hi = fkey(-KDGB_FINF);
    if (!lleaf) {
        unsigned *kk = next_keys + 6 * (int64_t)lnext;
        kk[0] = kk[1] = kk[2] = lo;
        kk[3] = kk[4] = kk[5] = hi;
        next_cnt[2 * lnext] = 0;
        next_cnt[2 * lnext + 1] = 0;
        next_pmin[lnext] = lmin;
        next_pmax[lnext] = lmax;
    }
    if (!rleaf) {
        unsigned *kk = next_keys + 6 * (int64_t)rnext;
        kk[0] = kk[1] = kk[2] = lo;
        kk[3] = kk[4] = kk[5] = hi;
        next_cnt[2 * rnext] = 0;
        next_cnt[2 * rnext + 1] = 0;
        next_pmin[rnext] = rmin;
        next_pmax[rnext] = rmax;
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
    for (unsigned bits = bmp; bits; bits &= bits - 1u) {  // bmp is warp-uniform
        const int j = __ffs(bits) - 1;
        const float mnx = __shfl_sync(0xffffffffu, lo.x, j), mny = __shfl_sync(0xffffffffu, lo.y, j);
        const float mnz = __shfl_sync(0xffffffffu, lo.z, j), mxx = __shfl_sync(0xffffffffu, hi.x, j);
        const float mxy = __shfl_sync(0xffffffffu, hi.y, j), mxz = __shfl_sync(0xffffffffu, hi.z, j);
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

// CalcAreaForSets (LowerTriangleMap.h:412-461) for the planes of one slot:
// a0..a3 are the area sums of the four sets (accumulated in bit order by the
// caller); low and high plane costs are tried in the reference's order.
__device__ __forceinline__ void pick_planes(const unsigned (&s)[4], const float (&a)[4], int axis, int32_t set_index,
                                            SahPick &best)
{
    const float low = __fadd_rn(__fmul_rn((float)__popc(s[0]), a[0]), __fmul_rn((float)__popc(s[1]), a[1]));
    const float high = __fadd_rn(__fmul_rn((float)__popc(s[2]), a[2]), __fmul_rn((float)__popc(s[3]), a[3]));
    if (low < best.cost) {
        best.cost = low; best.ls = s[0]; best.rs = s[1]; best.la = a[0]; best.ra = a[1];
        best.axis = axis; best.idx = set_index;
    }
    if (high < best.cost) {
        best.cost = high; best.ls = s[2]; best.rs = s[3]; best.la = a[2]; best.ra = a[3];
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
    // One pass over the node's references in bit order accumulates the area
    // sums of all twelve sets (3 axes x {lowLeft, lowRight, highLeft, highRight}).
    unsigned st[3][4] = {{(unsigned)sx.x & bmp, (unsigned)sx.y & bmp, (unsigned)sx.z & bmp, (unsigned)sx.w & bmp},
                         {(unsigned)sy.x & bmp, (unsigned)sy.y & bmp, (unsigned)sy.z & bmp, (unsigned)sy.w & bmp},
                         {(unsigned)sz.x & bmp, (unsigned)sz.y & bmp, (unsigned)sz.z & bmp, (unsigned)sz.w & bmp}};
    float ar[3][4] = {{0.f, 0.f, 0.f, 0.f}, {0.f, 0.f, 0.f, 0.f}, {0.f, 0.f, 0.f, 0.f}};
    for (unsigned bits = bmp; bits; bits &= bits - 1u) {  // bmp is warp-uniform
        const int j = __ffs(bits) - 1;
        const float aj = __shfl_sync(0xffffffffu, a_lane, j);
        const unsigned m = 1u << j;
#pragma unroll
        for (int x = 0; x < 3; ++x)
#pragma unroll
            for (int c = 0; c < 4; ++c) ar[x][c] = __fadd_rn(ar[x][c], (st[x][c] & m) ? aj : 0.0f);
    }
    pick_planes(st[0], ar[0], KDGB_X, pi + lane, mb);
    pick_planes(st[1], ar[1], KDGB_Y, pi + lane, mb);
    pick_planes(st[2], ar[2], KDGB_Z, pi + lane, mb);
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

// Grows a per-node array that carries `keep` live entries into a level.
template <class T>
int reserve_keep(DevArray<T> &a, int64_t n, int64_t keep, cudaStream_t s)
{
    if (a.p && n <= a.cap) return KDGB_OK;
    const int64_t want = a.cap + a.cap / 2 > n ? a.cap + a.cap / 2 : n;
    return ensure(a, want, s, a.p ? keep : 0);
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

int host_record(Workspace &ws)
{
    if (!ws.host) KDGB_CUDA(cudaMallocHost(&ws.host, kHostRec * sizeof(int32_t)));
    return KDGB_OK;
}

int lower_sah(Tree &t, const kdgb_build_params &p, const float4 *fmin, const float4 *fmax, int32_t F,
              cudaStream_t s)
{
    Workspace &w = t.ws;
    const int32_t nl = t.n_upper_leaves;
    KDGB_CHECK(grab(w.areas, F, s));
    KDGB_CHECK(grab(w.sts, 3 * (int64_t)F, s));
    if (F > 0) {
        k_areas<<<blocks_for(F), kBlock, 0, s>>>(F, t.prim_indices.p, t.p0.p, t.p1.p, t.p2.p, w.areas.p);
        KDGB_LAUNCH_CHECK();
    }
    if (nl > 0) {
        k_sah_preprocess<<<blocks_for(nl), kBlock, 0, s>>>(nl, t.leaf_ids.p, t.pidx.p, t.bitmap.p, t.area.p,
                                                           w.areas.p);
        KDGB_LAUNCH_CHECK();
        k_sah_planes<<<blocks_for((int64_t)nl * 32), kBlock, 0, s>>>(nl, t.leaf_ids.p, t.pidx.p, t.bitmap.p, fmin,
                                                                   fmax, F, w.sts.p);
        KDGB_LAUNCH_CHECK();
    }
    int32_t R = nl, active = t.n_nodes, lv = 0;
    const int32_t *ids = t.leaf_ids.p;
    while (R > 0) {
        ++lv;
        KDGB_CHECK(grab(w.ssplit, R, s));
        KDGB_CHECK(grab(w.saddr, (int64_t)R + 1, s));
        KDGB_CHECK(grab(w.careas, R, s));
        KDGB_CHECK(grab(w.csets, R, s));
        k_calc_sah<<<blocks_for((int64_t)R * 32), kBlock, 0, s>>>(
            R, ids, active, t.pidx.p, t.bitmap.p, t.area.p, w.areas.p, fmin, fmax, w.sts.p, F, p.traversal_cost,
            p.intersection_cost, p.min_leaf, t.info.p, t.split.p, w.ssplit.p, w.careas.p, w.csets.p);
        KDGB_LAUNCH_CHECK();
        KDGB_CHECK(scan_exclusive<1>(w.ssplit.p, w.saddr.p, R, s, &w.scan));
        KDGB_CUDA(cudaMemcpyAsync(w.host, w.saddr.p + R, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
        KDGB_CUDA(cudaStreamSynchronize(s));
        const int32_t splits = w.host[0];
        const int32_t child_base = t.n_nodes;
        KDGB_CHECK(grow_nodes(t, (int64_t)t.n_nodes + 2 * (int64_t)splits, s));
        if (splits > 0) {
            k_sah_children<<<blocks_for(R), kBlock, 0, s>>>(R, ids, active, child_base, w.ssplit.p, w.saddr.p,
                                                           w.careas.p, w.csets.p, p.propagate_aabbs, NODE_ARGS);
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
    Workspace &w = t.ws;
    KDGB_CHECK(host_record(w));
    KDGB_CHECK(grab(w.stats, 16, s));
    KDGB_CUDA(cudaMemsetAsync(w.stats.p, 0, sizeof(int), s));
    k_load_geometry<<<blocks_for(T), kBlock, 0, s>>>(tri_v_dev, T, t.p0.p, t.p1.p, t.p2.p, nullptr, nullptr, w.stats.p);
    KDGB_LAUNCH_CHECK();
    KDGB_CUDA(cudaMemcpyAsync(w.host, w.stats.p, sizeof(int), cudaMemcpyDeviceToHost, s));
    KDGB_CUDA(cudaStreamSynchronize(s));
    if (w.host[0]) return fail(KDGB_ERR_NONFINITE, "non-finite vertex coordinate");
    return KDGB_OK;
}

int build_reference(Tree &t, const float *tri_v_dev, int32_t T, const kdgb_build_params &p, cudaStream_t s,
                    const int32_t *mesh_off_dev, int32_t M)
{
    if (M < 1) M = 1;
    const int32_t LS = p.leaf_size;
    Workspace &w = t.ws;
    KDGB_CHECK(host_record(w));
    int32_t *rec = w.host;

    // Geometry, primitive boxes and the root node.
    KDGB_CHECK(ensure(t.p0, T, s));
    KDGB_CHECK(ensure(t.p1, T, s));
    KDGB_CHECK(ensure(t.p2, T, s));
    t.n_tris = T;
    KDGB_CHECK(grab(w.cmin, T, s));
    KDGB_CHECK(grab(w.cmax, T, s));
    KDGB_CHECK(grab(w.stats, 16, s));
    KDGB_CUDA(cudaMemsetAsync(w.stats.p, 0, 16 * sizeof(int32_t), s));
    if (T > 0) {
        k_load_geometry<<<blocks_for(T), kBlock, 0, s>>>(tri_v_dev, T, t.p0.p, t.p1.p, t.p2.p, w.cmin.p, w.cmax.p,
                                                        w.stats.p + 15, mesh_off_dev, M);
        KDGB_LAUNCH_CHECK();
    }
    t.n_nodes = 0;
    KDGB_CHECK(grow_nodes(t, M, s));
    k_init_roots<<<blocks_for(M), kBlock, 0, s>>>(T, M, mesh_off_dev, NODE_ARGS);
    KDGB_LAUNCH_CHECK();
    t.n_nodes = M;

    int64_t N = T, F = 0;
    int32_t active = 0, R = M, level = 0;
    std::vector<int2> leaf_ranges;
    std::vector<int32_t> leaf_off;
    int32_t n_leaf_ids = 0;

    while (R > 0) {
        if (level >= p.max_levels) return fail(KDGB_ERR_DEGENERATE, "upper build exceeded max_levels");
        ++level;
        // Tuned mode: median/empty-space splits on the first upper_levels
        // levels, binned SAH below them.
        const bool sah_level = p.mode == KDGB_BUILD_TUNED && level > p.upper_levels;
        const bool do_ess = p.split_empty_space && active != 0 && !sah_level;
        const int64_t nch = chunks_for(N);
        const unsigned ngrid = chunk_blocks(nch);
        KDGB_CHECK(grow_nodes(t, (int64_t)t.n_nodes + 14 * (int64_t)R, s));
        // Per-node arrays hold this level's R entries (written by the
        // previous level's k_children) and room for the next level's <= 2R.
        KDGB_CHECK(reserve_keep(w.pmin, 2 * (int64_t)R, R, s));
        KDGB_CHECK(reserve_keep(w.pmax, 2 * (int64_t)R, R, s));
        KDGB_CHECK(reserve_keep(w.keys, 12 * (int64_t)R, 6 * (int64_t)R, s));
        KDGB_CHECK(reserve_keep(w.cnt, 4 * (int64_t)R, 2 * (int64_t)R, s));
        KDGB_CHECK(grab(w.lanes, kLanes * (int64_t)R, s));
        KDGB_CHECK(grab(w.lbase, kLanes * ((int64_t)R + 1), s));
        KDGB_CHECK(grab(w.planes, R, s));
        KDGB_CHECK(grab(w.chunksum, 2 * nch, s));
        KDGB_CHECK(grab(w.chunkoff, 2 * (nch + 1), s));
        KDGB_CHECK(grab(w.nmin, 2 * N, s));
        KDGB_CHECK(grab(w.nmax, 2 * N, s));
        if (F + 2 * N > w.fmin.cap) {
            const int64_t want = (F + 2 * N) * 3 / 2 + 1024;
            KDGB_CHECK(ensure(w.fmin, want, s, F));
            KDGB_CHECK(ensure(w.fmax, want, s, F));
        }

        if (level == 1) {
            k_level_init<<<blocks_for(R), kBlock, 0, s>>>(R, active, t.bmin.p, t.bmax.p, w.pmin.p, w.pmax.p,
                                                          w.keys.p, w.cnt.p);
            KDGB_LAUNCH_CHECK();
        }
        if (N > 0) {
            k_reduce<<<ngrid, kBlock, 0, s>>>(N, w.cmin.p, w.cmax.p, w.keys.p);
            KDGB_LAUNCH_CHECK();
        }
        k_node_split<<<blocks_for(R), kBlock, 0, s>>>(R, active, do_ess, p.empty_space_threshold, w.pmin.p, w.pmax.p,
                                                      w.keys.p, t.bmin.p, t.bmax.p, t.split.p, t.info.p, w.planes.p,
                                                      w.lanes.p);
        KDGB_LAUNCH_CHECK();
        if (sah_level && N > 0) {
            const int B = p.sah_bins;
            KDGB_CHECK(grab(w.misc0, (int64_t)R * 6 * B, s));
            KDGB_CUDA(cudaMemsetAsync(w.misc0.p, 0, sizeof(int32_t) * (size_t)R * 6 * B, s));
            k_sah_bin<<<ngrid, kBlock, 0, s>>>(N, active, B, w.cmin.p, w.cmax.p, t.bmin.p, t.bmax.p, w.misc0.p);
            KDGB_LAUNCH_CHECK();
            k_sah_split<<<blocks_for((int64_t)R * 32), kBlock, 0, s>>>(R, active, B, t.bmin.p, t.bmax.p, t.bitmap.p,
                                                                      w.misc0.p, t.split.p, t.info.p);
            KDGB_LAUNCH_CHECK();
        }
        if (N > 0) {
            k_count<<<ngrid, kBlock, 0, s>>>(N, active, w.cmin.p, w.cmax.p, t.split.p, t.info.p, w.cnt.p,
                                             w.chunksum.p);
            KDGB_LAUNCH_CHECK();
        }
        KDGB_CHECK(scan_exclusive<2>(w.chunksum.p, w.chunkoff.p, nch, s, &w.scan));
        k_node_lanes<<<blocks_for(R), kBlock, 0, s>>>(R, LS, w.cnt.p, w.lanes.p);
        KDGB_LAUNCH_CHECK();
        KDGB_CHECK(scan_exclusive<kLanes>(w.lanes.p, w.lbase.p, R, s, &w.scan));
        if (N > 0) {
            k_scatter<<<ngrid, kBlock, 0, s>>>(N, R, active, LS, (int32_t)F, w.cmin.p, w.cmax.p, t.split.p, t.info.p,
                                               w.chunkoff.p, w.lbase.p, w.nmin.p, w.nmax.p, w.fmin.p, w.fmax.p);
            KDGB_LAUNCH_CHECK();
        }
        k_children<<<blocks_for(R), kBlock, 0, s>>>(R, active, t.n_nodes, do_ess, p.esc_zmax_as_x, LS, (int32_t)F,
                                                    p.split_empty_space, w.planes.p, w.lbase.p, NODE_ARGS, w.stats.p,
                                                    w.keys.p, w.cnt.p, w.pmin.p, w.pmax.p);
        KDGB_LAUNCH_CHECK();
        KDGB_CUDA(cudaMemcpyAsync(rec, w.stats.p, 16 * sizeof(int32_t), cudaMemcpyDeviceToHost, s));
        KDGB_CUDA(cudaStreamSynchronize(s));
        if (rec[15]) return fail(KDGB_ERR_NONFINITE, "non-finite vertex coordinate");

        const int32_t empty = rec[0];
        const int64_t total_l = rec[1], total_r = rec[2], leaf_l = rec[3], leaf_r = rec[4];
        const int32_t leaf_nodes = rec[5] + rec[6];
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
        std::swap(w.cmin, w.nmin);
        std::swap(w.cmax, w.nmax);
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
        if (2 * nr + nr > kHostRec) {
            // More leaf-producing levels than the pinned record holds: copy
            // from pageable memory (synchronous for the host).
            KDGB_CHECK(grab(w.ranges, nr, s));
            KDGB_CHECK(grab(w.roff, nr, s));
            KDGB_CUDA(cudaMemcpy(w.ranges.p, leaf_ranges.data(), sizeof(int2) * nr, cudaMemcpyHostToDevice));
            KDGB_CUDA(cudaMemcpy(w.roff.p, leaf_off.data(), sizeof(int32_t) * nr, cudaMemcpyHostToDevice));
        } else {
            KDGB_CHECK(grab(w.ranges, nr, s));
            KDGB_CHECK(grab(w.roff, nr, s));
            std::memcpy(rec, leaf_ranges.data(), sizeof(int2) * nr);
            std::memcpy(rec + 2 * nr, leaf_off.data(), sizeof(int32_t) * nr);
            KDGB_CUDA(cudaMemcpyAsync(w.ranges.p, rec, sizeof(int2) * nr, cudaMemcpyHostToDevice, s));
            KDGB_CUDA(cudaMemcpyAsync(w.roff.p, rec + 2 * nr, sizeof(int32_t) * nr, cudaMemcpyHostToDevice, s));
        }
        k_leaf_ids<<<blocks_for(n_leaf_ids), kBlock, 0, s>>>(w.ranges.p, nr, w.roff.p, n_leaf_ids, t.leaf_ids.p);
        KDGB_LAUNCH_CHECK();
    }
    if (F > 0) {
        k_extract_indices<<<blocks_for(F), kBlock, 0, s>>>((int32_t)F, w.fmin.p, t.prim_indices.p);
        KDGB_LAUNCH_CHECK();
    }
    if (!p.split_empty_space && p.propagate_aabbs && n_leaf_ids > 0) {
        k_propagate_parent<<<blocks_for(n_leaf_ids), kBlock, 0, s>>>(n_leaf_ids, t.leaf_ids.p, t.info.p, t.split.p,
                                                                     t.bmin.p, t.bmax.p, t.parent.p, t.children.p);
        KDGB_LAUNCH_CHECK();
    }

    t.stats.lower_levels = 0;
    if (p.lower == KDGB_LOWER_SAH) {
        // The SAH loop reuses the pinned record: wait until the range tables
        // above have been read from it.
        KDGB_CUDA(cudaStreamSynchronize(s));
        KDGB_CHECK(lower_sah(t, p, w.fmin.p, w.fmax.p, (int32_t)F, s));
    } else if (n_leaf_ids > 0) {
        k_bitmap_leaves<<<blocks_for(n_leaf_ids), kBlock, 0, s>>>(n_leaf_ids, t.leaf_ids.p, t.info.p, t.bitmap.p);
        KDGB_LAUNCH_CHECK();
    }
    return KDGB_OK;
}

}  // namespace kdgb
