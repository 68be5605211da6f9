// Traversal: kd-restart, short-stack, brute force and shadow rays.
//
// Each tracer restates its reference kernel with the shading left out and
// the first hit returned:
//   kd-restart  Raytracer.cu:57-106 (TraceNode) + :165-262 (KDRestart)
//   short-stack ShortStack.h:27-98 (ring buffer) + ShortStack.cu:58-194
//   brute force BruteTracer.cu:54-96 (cap of 4096 triangles lifted)
//   shadow      Raytracer.cu:108-163 (ShadowRay)
// with Moeller-Trumbore (IRayTracer.h:111-145) and the leaf-skipping slab test
// (IRayTracer.h:147-168).  Divisions are IEEE (__frcp_rn), products and sums
// separately rounded, so hit ids match the CPU restatement bit for bit.
//
// Memory layout read by the tracers (built by the pack kernels of kdgb_build.cu),
// in traversal order, where the two children of a node are adjacent:
//   tnode[j]  int2  interior: {split bits, (left << 2) | axis}, right = left + 1
//                   leaf:     {first record, (record count << 2) | 0}
//   ttri[3r..3r+2]  float4 x3 per leaf record, in leaf order:
//                   {v0.xyz, e1.x} {e1.yz, e2.xy} {e2.z, id bits, 0, 0}
//   box[2j], box[2j+1]  float4 min and max of leaf j (leaf skipping), one sector
// One 8-byte load per traversal step and three 16-byte loads per triangle
// test, with no index indirection; e1 = v1 - v0 and e2 = v2 - v0 are the
// same fp32 values the reference computes per test.
#include <cuda_runtime.h>

#include <algorithm>

#include "kdgb_internal.cuh"
#include "kdgb_photon.cuh"

namespace kdgb {

namespace {

constexpr int kMaxStack = 8;
// Hard cap on restarts/pops per ray when the caller passes 0, so that a
// pathological ray cannot keep a thread alive forever.
constexpr int kDefaultMaxIterations = 1 << 22;

inline unsigned blocks_for(int64_t n, int b) { return (unsigned)((n + b - 1) / b); }

struct Ctx {
    const int2 *__restrict__ node;
    const float4 *__restrict__ box;  // leaf boxes, min and max of node j at [2j], [2j + 1]
    const float4 *__restrict__ tri;
    const float4 *__restrict__ woop;  // per-triangle Woop values, or NULL for Moeller-Trumbore
    int root;  // root node of the ray's tree (forest of a batch: its mesh index)
};

// The box of leaf `node` (leaf skipping).
__device__ __forceinline__ float4 leaf_min(const Ctx &c, int node) { return __ldg(c.box + 2 * (int64_t)node); }
__device__ __forceinline__ float4 leaf_max(const Ctx &c, int node) { return __ldg(c.box + 2 * (int64_t)node + 1); }

// Fields of a tnode record.
__device__ __forceinline__ int node_axis(int2 nd) { return nd.y & 3; }
__device__ __forceinline__ int node_left(int2 nd) { return nd.y >> 2; }
__device__ __forceinline__ float node_split(int2 nd) { return __int_as_float(nd.x); }
__device__ __forceinline__ int32_t leaf_first(int2 nd) { return nd.x; }
__device__ __forceinline__ int32_t leaf_count(int2 nd) { return nd.y >> 2; }

// True when x = RN(RN(1/det) * n) is certainly negative and nonzero:
// det and n have opposite signs, and |det| <= 2^64, |n| >= 2^-64 (so n is
// not zero, nor NaN) so the product cannot round to -0 (a -0 would pass the
// `>= 0` tests).  det = +-0 gives +-inf, whose product with n is negative as
// well.
__device__ __forceinline__ bool surely_negative(float det, float n)
{
    return (signbit(det) != signbit(n)) && fabsf(det) <= 0x1p64f && fabsf(n) >= 0x1p-64f;
}

// Moeller-Trumbore on one packed record (IRayTracer.h:111-145).  Triangles
// whose u or v is certainly negative are rejected before the IEEE
// reciprocal, u first: most tests end there (on the 1M-triangle frame 86% of
// a primary ray's tests and 82% of a shadow ray's), so the v terms are only
// computed for triangles that pass it (primary trace of the frame 0.803 ->
// 0.785 ms).  Every accepted value is computed exactly as the reference does.
__device__ __forceinline__ void mt_test(float3 v0, float3 e1, float3 e2, int id, float3 o, float3 d, int tie,
                                        int &hit, float &tb, float &ub, float &vb)
{
    const float3 p = cross3(d, e2);
    const float3 t = sub3(o, v0);
    const float det = dot3(p, e1);
    const float pt = dot3(p, t);
    if (surely_negative(det, pt)) return;
    const float3 q = cross3(t, e1);
    const float qd = dot3(q, d);
    if (surely_negative(det, qd)) return;
    const float inv_det = __frcp_rn(det);
    const float ht = __fmul_rn(inv_det, dot3(q, e2));
    if (0.0f <= ht && ht <= tb) {
        const float hu = __fmul_rn(inv_det, pt);
        const float hv = __fmul_rn(inv_det, qd);
        if (hu >= 0.0f && hv >= 0.0f && __fadd_rn(hu, hv) <= 1.0f) {
            if (tie == KDGB_TIE_REF_LAST || hit == -1 || ht < tb || id < hit) {
                hit = id; tb = ht; ub = hu; vb = hv;
            }
        }
    }
}

__device__ __forceinline__ void mt_record(const float4 *__restrict__ tri, int32_t rec, float3 o, float3 d, int tie,
                                          int &hit, float &tb, float &ub, float &vb)
{
    const float4 a = __ldg(tri + 3 * (int64_t)rec);
    const float4 b = __ldg(tri + 3 * (int64_t)rec + 1);
    const float4 c = __ldg(tri + 3 * (int64_t)rec + 2);
    mt_test(make_float3(a.x, a.y, a.z), make_float3(a.w, b.x, b.y), make_float3(b.z, b.w, c.x), __float_as_int(c.y),
            o, d, tie, hit, tb, ub, vb);
}

// RayBoxIntersection<true> (IRayTracer.h:147-168), with the reference's
// min / max (fminf / fmaxf, one instruction each).  The values of n and f
// reach nothing but the comparison n <= f, which does not see the sign of a
// zero, so the order the tracers' other minima give -0 and +0 is not needed
// here.
__device__ __forceinline__ bool ray_box(float3 o, float3 inv, float4 bmin, float4 bmax)
{
    const float lx = __fmul_rn(__fsub_rn(bmin.x, o.x), inv.x), ly = __fmul_rn(__fsub_rn(bmin.y, o.y), inv.y),
                lz = __fmul_rn(__fsub_rn(bmin.z, o.z), inv.z);
    const float hx = __fmul_rn(__fsub_rn(bmax.x, o.x), inv.x), hy = __fmul_rn(__fsub_rn(bmax.y, o.y), inv.y),
                hz = __fmul_rn(__fsub_rn(bmax.z, o.z), inv.z);
    float n = fminf(lx, hx);
    n = fmaxf(n, fminf(ly, hy));
    n = fmaxf(n, fminf(lz, hz));
    float f = fmaxf(hx, lx);
    f = fminf(f, fmaxf(ly, hy));
    f = fminf(f, fmaxf(lz, hz));
    return n <= f;
}

// Woop's test (IRayTracer.h:78-109) against the triangle's transform rows
// m0, m1, m2 (GeometryList.cu:81-102): lambda = -(m2.o - m2.w) / (m2.d),
// u = lambda (m0.d) + m0.o - m0.w, v likewise with m1.
__device__ __forceinline__ float woop_lambda(float4 m2, float3 o, float3 d)
{
    const float3 n2 = make_float3(m2.x, m2.y, m2.z);
    return __fdiv_rn(-__fsub_rn(dot3(n2, o), m2.w), dot3(n2, d));
}

__device__ __forceinline__ void woop_accept(float lambda, float4 m0, float4 m1, int id, float3 o, float3 d, int tie,
                                            int &hit, float &tb, float &ub, float &vb)
{
    const float3 n0 = make_float3(m0.x, m0.y, m0.z), n1 = make_float3(m1.x, m1.y, m1.z);
    const float hu = __fsub_rn(__fadd_rn(__fmul_rn(lambda, dot3(n0, d)), dot3(n0, o)), m0.w);
    const float hv = __fsub_rn(__fadd_rn(__fmul_rn(lambda, dot3(n1, d)), dot3(n1, o)), m1.w);
    if (hu >= -0.0f && hv >= -0.0f && __fadd_rn(hu, hv) <= 1.0f) {
        if (tie == KDGB_TIE_REF_LAST || hit == -1 || lambda < tb || id < hit) {
            hit = id; tb = lambda; ub = hu; vb = hv;
        }
    }
}

// The rows in registers (brute-force tiles).
__device__ __forceinline__ void woop_test(float4 m0, float4 m1, float4 m2, int id, float3 o, float3 d, int tie,
                                          int &hit, float &tb, float &ub, float &vb)
{
    const float lambda = woop_lambda(m2, o, d);
    if (0.0f <= lambda && lambda <= tb) woop_accept(lambda, m0, m1, id, o, d, tie, hit, tb, ub, vb);
}

// The rows in global memory: m0 and m1 are loaded only when lambda passes.
__device__ __forceinline__ void woop_test(const float4 *__restrict__ w, int id, float3 o, float3 d, int tie, int &hit,
                                          float &tb, float &ub, float &vb)
{
    const float lambda = woop_lambda(__ldg(w + 2), o, d);
    if (0.0f <= lambda && lambda <= tb) woop_accept(lambda, __ldg(w), __ldg(w + 1), id, o, d, tie, hit, tb, ub, vb);
}

// The intersection test of a kernel: Moeller-Trumbore or Woop's test fixed
// at compile time (the frame's trace kernels), or chosen per launch by
// whether c.woop is set (kIsectAny).  A fixed choice takes the other test's
// branch out of the leaf loops.
constexpr int kIsectAny = 2;

template <int IS = kIsectAny>
__device__ __forceinline__ bool use_woop(const Ctx &c)
{
    return IS == KDGB_ISECT_WOOP || (IS == kIsectAny && c.woop != nullptr);
}

// Traversal steps of one thread, kept only by the counting launch
// (kdgb_trace_count_steps): node records read, leaves reached, leaf boxes
// read and triangle records tested.  Every other kernel is instantiated with
// CNT false, so the counting compiles out of it.
struct StepCount {
    unsigned node = 0, leaf = 0, box = 0, tri = 0;
};

template <int IS = kIsectAny, bool CNT = false>
__device__ __forceinline__ int leaf_test(const Ctx &c, int2 leaf, float3 o, float3 d, int tie, float &tb, float &ub,
                                         float &vb, StepCount *sc = nullptr)
{
    int hit = -1;
    if constexpr (CNT) sc->tri += leaf_count(leaf);
    if (use_woop<IS>(c)) {
        for (int32_t r = leaf_first(leaf), e = r + leaf_count(leaf); r < e; ++r) {
            const int id = __float_as_int(__ldg(c.tri + 3 * (int64_t)r + 2).y);
            woop_test(c.woop + 3 * (int64_t)id, id, o, d, tie, hit, tb, ub, vb);
        }
    } else {
        for (int32_t r = leaf_first(leaf), e = r + leaf_count(leaf); r < e; ++r) mt_record(c.tri, r, o, d, tie, hit, tb, ub, vb);
    }
    return hit;
}

// Whether any triangle of the leaf is hit within [0, tb] (the reference's
// shadow test, REF_LAST acceptance): the first accepted triangle settles it,
// so the loop stops there with the result testing all of them gives.
template <int IS = kIsectAny, bool CNT = false>
__device__ __forceinline__ bool leaf_any(const Ctx &c, int2 leaf, float3 o, float3 d, float tb, StepCount *sc = nullptr)
{
    int hit = -1;
    float ub = 0.0f, vb = 0.0f;
    if (use_woop<IS>(c)) {
        for (int32_t r = leaf_first(leaf), e = r + leaf_count(leaf); r < e; ++r) {
            if constexpr (CNT) ++sc->tri;
            const int id = __float_as_int(__ldg(c.tri + 3 * (int64_t)r + 2).y);
            woop_test(c.woop + 3 * (int64_t)id, id, o, d, KDGB_TIE_REF_LAST, hit, tb, ub, vb);
            if (hit != -1) return true;
        }
    } else {
        for (int32_t r = leaf_first(leaf), e = r + leaf_count(leaf); r < e; ++r) {
            if constexpr (CNT) ++sc->tri;
            mt_record(c.tri, r, o, d, KDGB_TIE_REF_LAST, hit, tb, ub, vb);
            if (hit != -1) return true;
        }
    }
    return false;
}

// Remembered descents for kd-restart.  A restart descends from the root
// with tmin' = tnext * 1.00001, larger than the tmin of the previous
// descent, so it repeats every decision of that descent (far ones stay far,
// near ones whose split distance exceeds tmin' stay near) down to the
// topmost near decision whose split distance is <= tmin', and turns to the
// far child there.  Keeping the near decisions of the current descent that
// lower the prefix minimum of the split distances from the root, as (far
// child, that minimum), lets the descent resume at that child with the
// previous entry's minimum as tnext: the leaves visited and their tnext
// values are exactly those of the full restart.  The deepest `cap` (a power
// of two) such decisions are kept (a ring in shared memory, entry slot s at
// e[s * stride]); when the turning node lies above them (`base`, the minimum
// over the dropped ones, is <= tmin') the descent starts again from the root.
//
// Capacity where the shared region is sized for it.  With only the lowering
// decisions kept, 8 entries leave almost no restart from the root, and the
// halved region leaves more of the SM to L1 (16 -> 8 entries: kd-restart
// photons 8.02 -> 6.98 ms, kd-restart frame rays 0.854 -> 0.794 ms, shadow
// rays alone 0.883 -> 0.836 ms, identical results).
constexpr int kMemo = 8;

struct Memo {
    int2 *e;
    int stride, cap, head, cnt;
    float base;
    __device__ __forceinline__ void reset()
    {
        head = 0;
        cnt = 0;
        base = KDGB_FINF;
    }
    __device__ __forceinline__ int2 &at(int i) const { return e[((head + i) & (cap - 1)) * stride]; }
    __device__ __forceinline__ void push(int far, float pm)
    {
        if (cnt == cap) {  // drop the shallowest; it is the deepest dropped so far
            base = __int_as_float(at(0).y);
            head = (head + 1) & (cap - 1);
            --cnt;
        }
        at(cnt) = make_int2(far, __float_as_int(pm));
        ++cnt;
    }
};

// The largest power of two <= n (n >= 1): the memo capacity of a region of
// n entries.
__device__ __forceinline__ int memo_cap(int n) { return 1 << (31 - __clz(n)); }

// Per-thread int2 entries of the tracers' shared-memory region: the short
// stack (ShortStack; its depth, so the region takes no L1 beyond it) or the
// remembered descents (kd-restart), then those of the shadow rays.
__host__ __device__ __forceinline__ int stack_entries(int tracer, int depth)
{
    return tracer == KDGB_TRACER_SHORTSTACK ? depth : kMemo;
}

// Descends from `node` (record nd) to a leaf, as the reference's kd-restart
// loop does (Raytracer.cu:73-86); the near decisions that lower tnext are
// remembered in m.
template <bool CNT = false>
__device__ __forceinline__ void restart_descend(const Ctx &c, float3 o, float3 inv, float tmin, int &node, int2 &nd,
                                                float &tnext, Memo &m, StepCount *sc = nullptr)
{
    while (node_axis(nd) != KDGB_LEAF) {
        const int ax = node_axis(nd), left = node_left(nd);
        const float ori = axis_of(o, ax), dir = axis_of(inv, ax);
        const float ts = __fmul_rn(__fsub_rn(node_split(nd), ori), dir);
        if (tmin < ts) {
            // Only near decisions that lower the prefix minimum are
            // remembered: a later restart turns at the topmost near decision
            // whose split distance is <= its tmin, and above a decision with
            // ts >= tnext lies one with a distance <= ts, so such a decision
            // is never the turning node.  Its entry would only take a ring
            // slot (frame shadow rays: 17 pushes instead of 40, and almost no
            // restarts from the root).  The entry names the far child, where a
            // restart that turns here continues.
            if (ts < tnext) m.push(0 < dir ? left + 1 : left, ts);
            // tnext reaches only comparisons and tmin, whose zero sign no
            // result sees: the reference's fminf is exact here.
            tnext = fminf(ts, tnext);
            node = 0 < dir ? left : left + 1;
        } else {
            node = 0 < dir ? left + 1 : left;
        }
        nd = __ldg(c.node + node);
        if constexpr (CNT) ++sc->node;
    }
}

// Where the next kd-restart descent starts: the far child of the topmost
// remembered near decision whose distance is <= tmin (prefix minima fall
// with depth, so it is the first entry whose minimum is <= tmin), or the
// root.
template <bool CNT = false>
__device__ __forceinline__ void restart_from(const Ctx &c, float tmin, int &node, int2 &nd, float &tnext, Memo &m,
                                             StepCount *sc = nullptr)
{
    if constexpr (CNT) ++sc->node;  // one node record on either path
    if (m.cnt > 0 && tmin < m.base) {
        // Usually the deepest entry: its minimum is the leaf's tnext, and the
        // one above it lies beyond tmin.  Otherwise the first entry whose
        // minimum is <= tmin, by binary search over the ones above.
        int lo = m.cnt - 1;
        float above = lo > 0 ? __int_as_float(m.at(lo - 1).y) : m.base;
        if (!(tmin < above)) {
            int hi = lo - 1;  // the entry at hi already qualifies
            lo = 0;
            while (lo < hi) {
                const int mid = (lo + hi) >> 1;
                if (__int_as_float(m.at(mid).y) <= tmin) hi = mid; else lo = mid + 1;
            }
            above = lo > 0 ? __int_as_float(m.at(lo - 1).y) : m.base;
        }
        const int2 e = m.at(lo);
        tnext = above;
        m.cnt = lo;
        node = e.x;  // the far child: one node load instead of two dependent ones
        nd = __ldg(c.node + node);
        return;
    }
    m.reset();
    node = c.root;
    nd = __ldg(c.node + c.root);
    tnext = KDGB_FINF;
}

// kd-restart, first hit (Raytracer.cu:57-106, 165-262), with the descents
// remembered in `cap` entries at mem[k * stride] (see Memo).
template <bool SKIP, int IS = kIsectAny>
__device__ int trace_restart(const Ctx &c, float3 o, float3 din, int tie, int maxit, float &t, float &u, float &v,
                             float3 *dused, int2 *mem, int stride, int cap = kMemo)
{
    const float3 d = adjust_dir(din);
    const float3 inv = inv3(d);
    if (dused) *dused = d;
    float tmin = 0.0f;
    int iters = 0;
    Memo memo;
    memo.e = mem;
    memo.stride = stride;
    memo.cap = cap;
    memo.reset();
    int node = c.root;
    int2 nd = __ldg(c.node + c.root);
    float tnext = KDGB_FINF;
    do {
        restart_descend(c, o, inv, tmin, node, nd, tnext, memo);
        tmin = __fmul_rn(tnext, 1.00001f);
        if (!SKIP || ray_box(o, inv, leaf_min(c, node), leaf_max(c, node))) {
            float tb = tmin, ub = 0.0f, vb = 0.0f;
            const int h = leaf_test<IS>(c, nd, o, d, tie, tb, ub, vb);
            if (h != -1) { t = tb; u = ub; v = vb; return h; }
        }
        if (++iters >= maxit) break;
        if (!(tmin < KDGB_FINF)) break;
        restart_from(c, tmin, node, nd, tnext, memo);
    } while (true);
    return -1;
}

// Short-stack loop (ShortStack.cu:58-194).  The stack of this thread lives
// in shared memory at st[i * stride]; entries are (node, tMax bits).  The
// reference inverts the direction in place before each descent and back
// after it (ShortStack.cu:134,148): with FIXED false, d is that direction
// and inv is unused.  With FIXED true that sequence is at its fixed point
// (see trace_shortstack): every descent and slab test uses inv and every
// triangle test d, neither changing, so the loop holds three registers and
// no selects fewer.
template <bool SKIP, bool FIXED, int IS, bool CNT, int DEPTH>
__device__ __forceinline__ int shortstack_loop(const Ctx &c, float3 o, float3 d, float3 inv, int tie, int depth,
                                               int maxit, int2 *st, int stride, float &t, float &u, float &v,
                                               float3 *dused, StepCount *sc)
{
    int nxt = 0, cnt = 0;
    float th = 0.0f;
    int iters = 0;
    do {
        int node;
        float tnext;
        if (cnt == 0) {
            node = c.root;
            tnext = KDGB_FINF;
        } else {
            // With a DEPTH fixed at compile time (a power of two) the ring
            // wraps by a mask; the same entries as the runtime form.
            nxt = DEPTH ? (nxt - 1) & (DEPTH - 1) : (nxt == 0 ? depth : nxt) - 1;
            --cnt;
            const int2 e = st[nxt * stride];
            node = e.x;
            tnext = __int_as_float(e.y);
        }
        int2 nd = __ldg(c.node + node);
        if constexpr (CNT) ++sc->node;
        if (!FIXED) d = inv3(d);
        const float3 dn = FIXED ? inv : d;  // the inverse direction of this descent
        while (node_axis(nd) != KDGB_LEAF) {
            const int ax = node_axis(nd), left = node_left(nd);
            const float ori = axis_of(o, ax), dir = axis_of(dn, ax);
            const float ts = __fmul_rn(__fsub_rn(node_split(nd), ori), dir);
            const int lower = 0 < dir ? left : left + 1;
            const int upper = 0 < dir ? left + 1 : left;
            // The near/far choice as selects, with only the push under a
            // branch (1.5% fewer cycles on the frame than branching on it).
            const bool go_near = th < ts;
            if (go_near && ts < tnext) {
                st[nxt * stride] = make_int2(upper, __float_as_int(tnext));
                nxt = DEPTH ? (nxt + 1) & (DEPTH - 1) : (nxt == depth - 1 ? 0 : nxt + 1);
                cnt = DEPTH ? min(cnt + 1, DEPTH) : (cnt == depth ? depth : cnt + 1);
            }
            tnext = go_near ? fminf(ts, tnext) : tnext;  // as in restart_descend
            node = go_near ? lower : upper;
            nd = __ldg(c.node + node);
            if constexpr (CNT) ++sc->node;
        }
        if (!FIXED) d = inv3(d);
        th = __fmul_rn(tnext, 1.00001f);
        if constexpr (CNT) {
            ++sc->leaf;
            if (SKIP) ++sc->box;
        }
        if (!SKIP || ray_box(o, FIXED ? inv : inv3(d), leaf_min(c, node), leaf_max(c, node))) {
            float tb = th, ub = 0.0f, vb = 0.0f;
            const int h = leaf_test<IS, CNT>(c, nd, o, d, tie, tb, ub, vb, sc);
            if (h != -1) {
                t = tb; u = ub; v = vb;
                if (dused) *dused = d;
                return h;
            }
        }
        if (++iters >= maxit) break;
    } while (th < KDGB_FINF);
    return -1;
}

// Short-stack, first hit (ShortStack.cu:58-194).  The reference inverts d
// before each descent and back after it, so d becomes rcp(rcp(d)) after the
// first iteration.  When rcp(rcp(rcp(d))) == rcp(d) the sequence is at its
// fixed point from then on: every descent and slab test uses inv1 = rcp(d)
// and every triangle test d1 = rcp(inv1).  That holds for all finite nonzero
// floats except six values next to FLT_MAX (checked exhaustively); it is
// tested per ray, and rays that miss it take the reference's loop.
template <bool SKIP, int IS = kIsectAny, bool CNT = false, int DEPTH = 0>
__device__ int trace_shortstack(const Ctx &c, float3 o, float3 din, int tie, int depth, int maxit, int2 *st,
                                int stride, float &t, float &u, float &v, float3 *dused = nullptr,
                                StepCount *sc = nullptr)
{
    const float3 d = adjust_dir(din);
    const float3 inv1 = inv3(d), d1 = inv3(inv1), inv2 = inv3(d1);
    const bool fixed = __float_as_uint(inv2.x) == __float_as_uint(inv1.x) &&
                       __float_as_uint(inv2.y) == __float_as_uint(inv1.y) &&
                       __float_as_uint(inv2.z) == __float_as_uint(inv1.z);
    if (fixed)
        return shortstack_loop<SKIP, true, IS, CNT, DEPTH>(c, o, d1, inv1, tie, depth, maxit, st, stride, t, u, v, dused,
                                                           sc);
    return shortstack_loop<SKIP, false, IS, CNT, DEPTH>(c, o, d, d, tie, depth, maxit, st, stride, t, u, v, dused, sc);
}

// ShadowRay (Raytracer.cu:108-163): from the light toward the point, the
// direction neither normalised nor clamped; leaves whose exit reaches 0.999
// are not tested; any hit occludes.
// The descents are remembered in `cap` entries at mem[k * stride] (see Memo).
template <int IS = kIsectAny, bool CNT = false>
__device__ int trace_shadow(const Ctx &c, float3 lp, float3 pt, int maxit, int2 *mem, int stride, int cap = kMemo,
                            StepCount *sc = nullptr)
{
    const float3 d = sub3(pt, lp);
    const float3 inv = inv3(d);
    float tmin = 0.0f;
    int iters = 0;
    Memo memo;
    memo.e = mem;
    memo.stride = stride;
    memo.cap = cap;
    memo.reset();
    int node = c.root;
    int2 nd = __ldg(c.node + c.root);
    if constexpr (CNT) ++sc->node;
    float tnext = KDGB_FINF;
    do {
        restart_descend<CNT>(c, lp, inv, tmin, node, nd, tnext, memo, sc);
        if constexpr (CNT) ++sc->leaf;
        tmin = __fmul_rn(tnext, 1.00001f);
        if (tmin >= 0.999f) return 0;
        if (leaf_any<IS, CNT>(c, nd, lp, d, tmin, sc)) return 1;
        if (++iters >= maxit) break;
        restart_from<CNT>(c, tmin, node, nd, tnext, memo, sc);
    } while (true);
    return 0;
}

// PacketIndex (IRayTracer.h:67-76): 4x8 pixel packets per warp.
constexpr int kPW = 4, kPH = 8;  // 4x8 pixels per warp (an 8x4 packet was 5% slower on the frame)
__device__ __forceinline__ int64_t ray_index(int64_t id, int tile_width)
{
    if (tile_width <= 0) return id;
    if (id < 0x7fffffff) {  // 32-bit arithmetic for image-sized launches
        const int32_t i = (int32_t)id, cell = i >> 5, cols = tile_width / kPW;
        const int32_t by = cell / cols, bx = cell - by * cols;
        return (int64_t)(bx * kPW + (i & (kPW - 1))) + (int64_t)(by * kPH + ((i & 31) / kPW)) * tile_width;
    }
    const int64_t cell = id / 32;
    const int64_t cols = tile_width / kPW;
    const int64_t bx = cell % cols, by = cell / cols;
    const int64_t x = id % kPW, y = (id % 32) / kPW;
    return bx * kPW + x + (by * kPH + y) * tile_width;
}

__device__ __forceinline__ float3 ld3(const float *__restrict__ p, int64_t i)
{
    return make_float3(__ldg(p + 3 * i), __ldg(p + 3 * i + 1), __ldg(p + 3 * i + 2));
}

struct TraceArgs {
    Ctx c;
    const float *o, *d;
    int64_t n;
    int32_t *hit;
    float *t, *u, *v;
    int32_t *occ;
    float3 light;
    int tie, depth, maxit, tile_width;
    // Batches: ray i belongs to mesh ray_mesh[i] (or i / rays_per_mesh when
    // ray_mesh is NULL); its tree's root is node m and hit ids are returned
    // relative to the mesh's first triangle mesh_off[m].
    const int32_t *mesh_off, *ray_mesh;
    int32_t rays_per_mesh, n_meshes;
    // Nonzero when the tree's last build failed (a graph rebuild that
    // outgrew its buffers): every ray then reports a miss without reading
    // the tree.
    const int32_t *build_err;
    // The counting launch's totals (primary rays' StepCount, then the shadow
    // rays'); unused by every other launch.
    unsigned long long *counts = nullptr;
};

// A shadow ray waiting in a block's queue: the hit point, the tree root and
// the ray it belongs to.
struct ShadowItem {
    float4 p;  // w = bits of the block thread whose primary ray hit there
};

// The mesh (forest root) of ray i of a batch (the tree's root otherwise).
__device__ __forceinline__ int ray_mesh_of(const TraceArgs &a, int64_t i)
{
    if (!a.mesh_off) return a.c.root;
    const int m = a.ray_mesh ? a.ray_mesh[i] : (int)(i / a.rays_per_mesh);
    return m < 0 ? 0 : (m >= a.n_meshes ? a.n_meshes - 1 : m);
}

// First hit of ray i with the tracer of TRACER (its tree: the ray's mesh for
// a batch), written to the outputs; the thread's stack or memo region is
// stk[k * stride].  Returns the hit id (relative to the whole tree) and the
// ray and t for a shadow ray.
template <int TRACER, bool SKIP, int IS = kIsectAny, bool CNT = false, int DEPTH = 0>
__device__ __forceinline__ int trace_ray(const TraceArgs &a, int64_t i, int2 *stk, int stride, float3 &o, float3 &d,
                                         float &t, StepCount *sc = nullptr)
{
    o = ld3(a.o, i);
    d = ld3(a.d, i);
    Ctx c = a.c;
    int32_t id_off = 0;
    if (a.mesh_off) {
        c.root = ray_mesh_of(a, i);
        id_off = a.mesh_off[c.root];
    }
    float u = 0.0f, v = 0.0f;
    int h;
    if (TRACER == KDGB_TRACER_SHORTSTACK)
        h = trace_shortstack<SKIP, IS, CNT, DEPTH>(c, o, d, a.tie, a.depth, a.maxit, stk, stride, t, u, v, nullptr, sc);
    else
        h = trace_restart<SKIP, IS>(c, o, d, a.tie, a.maxit, t, u, v, nullptr, stk, stride);
    if (h < 0) { t = INFINITY; u = 0.0f; v = 0.0f; }
    a.hit[i] = h >= 0 ? h - id_off : h;
    a.t[i] = t;
    a.u[i] = u;
    a.v[i] = v;
    return h;
}

// Dynamic shared memory: the per-thread regions of stack_entries() int2
// (short stack or remembered descents); with shadow rays, the queue of
// blockDim ShadowItem the primary rays fill for the shadow pass overlays
// them (at least two entries per thread).  Capped at 40 registers: the traversal is
// bound by latency and issue, and the extra resident warps (75% occupancy
// instead of 56%) gain more than the few spilled values cost (measured on
// the 1M-triangle frame: 1.61 ms against 1.72 ms uncapped, 1.67 ms at 48
// and 1.83 ms at 32 registers).
//
// BS, when nonzero, is the block size the instance is launched with
// (trace_launch picks it only for blocks of exactly BS threads): the stack
// regions' stride is then a constant, which the frame's launch (128 threads)
// traces 1.5% faster with.  BS = 0 reads the stride from blockDim.x.
template <int TRACER, bool SKIP, bool SHADOW, int IS, bool CNT = false, int BS = 0, int DEPTH = 0>
__global__ void __maxnreg__(40) k_trace(TraceArgs a)
{
    const int stride = BS ? BS : (int)blockDim.x;
    extern __shared__ __align__(16) unsigned char trace_smem[];
    int2 *stack_smem = (int2 *)trace_smem;
    const int64_t id = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const bool live = id < a.n;
    const int64_t i = live ? ray_index(id, a.tile_width) : 0;
    if (a.build_err && *a.build_err) {  // grid-uniform
        if (live) {
            a.hit[i] = -1;
            a.t[i] = INFINITY;
            a.u[i] = 0.0f;
            a.v[i] = 0.0f;
            if (SHADOW) a.occ[i] = 0;
        }
        return;
    }
    float3 o = make_float3(0.f, 0.f, 0.f), d = o;
    float t = 0.0f;
    int h = -1;
    StepCount cp, cs;  // counting launch only
    if (live) h = trace_ray<TRACER, SKIP, IS, CNT, DEPTH>(a, i, stack_smem + threadIdx.x, stride, o, d, t, &cp);
    if (SHADOW) {
        // The block's shadow rays (one per primary hit) are packed onto its
        // first threads, so warps stay full while they are traced.
        // The queue overlays the stack region, which no primary ray uses any
        // more once the block has passed this barrier.
        __shared__ int s_count;
        ShadowItem *queue = (ShadowItem *)trace_smem;
        if (threadIdx.x == 0) s_count = 0;
        __syncthreads();
        if (h >= 0) {
            const float3 p = make_float3(__fadd_rn(o.x, __fmul_rn(t, d.x)), __fadd_rn(o.y, __fmul_rn(t, d.y)),
                                         __fadd_rn(o.z, __fmul_rn(t, d.z)));
            const int slot = atomicAdd(&s_count, 1);
            queue[slot].p = make_float4(p.x, p.y, p.z, __int_as_float((int)threadIdx.x));
        } else if (live) {
            a.occ[i] = 0;
        }
        __syncthreads();
        const bool queued = (int)threadIdx.x < s_count;
        ShadowItem q;
        if (queued) q = queue[threadIdx.x];
        __syncthreads();  // every item is read before the shadow rays' descents reuse the region
        if (queued) {
            const int64_t ray = ray_index((int64_t)blockIdx.x * blockDim.x + __float_as_int(q.p.w), a.tile_width);
            Ctx cr = a.c;
            cr.root = ray_mesh_of(a, ray);
            a.occ[ray] = trace_shadow<IS, CNT>(cr, a.light, make_float3(q.p.x, q.p.y, q.p.z), a.maxit,
                                             stack_smem + threadIdx.x, stride,
                                             memo_cap(stack_entries(TRACER, DEPTH ? DEPTH : a.depth)), &cs);
        }
    }
    if constexpr (CNT) {  // every thread of the block is here: warp sums, one atomic per warp and counter
        const unsigned v[8] = {cp.node, cp.leaf, cp.box, cp.tri, cs.node, cs.leaf, cs.box, cs.tri};
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            const unsigned w = __reduce_add_sync(0xffffffffu, v[k]);
            if ((threadIdx.x & 31) == 0 && w) atomicAdd(a.counts + k, (unsigned long long)w);
        }
    }
}

// Queue schedule (KDGB_SCHEDULE_QUEUE): a persistent grid whose warps take
// 32-ray chunks from a device-side counter until the rays run out.  With a
// mesh order (a batch traced with rays_per_mesh), chunk c holds rays
// [k * 32, k * 32 + 32) of mesh order[c / chunks_per_mesh], k = c %
// chunks_per_mesh, so the rays of the largest meshes go first and the cheap
// ones fill the tail; otherwise chunks follow the ray order (4x8 pixel
// packets with a tile width).  No warp waits for another: the grid only has
// to start.  The last warp to finish resets the counters for the next
// launch.
struct TraceQueue {
    unsigned *ctr;          // [0] next chunk, [1] warps finished
    const int32_t *order;   // meshes, largest first, or NULL
    unsigned n_chunks;
    int32_t chunks_per_mesh;
    unsigned n_warps;
};

template <int TRACER, bool SKIP>
__global__ void __maxnreg__(40) k_trace_queue(TraceArgs a, TraceQueue q)
{
    extern __shared__ __align__(16) unsigned char trace_smem[];
    int2 *stk = (int2 *)trace_smem + threadIdx.x;
    const unsigned lane = threadIdx.x & 31;
    if (a.build_err && *a.build_err) {  // grid-uniform: every ray misses, the queue is not touched
        for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < a.n; i += (int64_t)gridDim.x * blockDim.x) {
            a.hit[i] = -1;
            a.t[i] = INFINITY;
            a.u[i] = 0.0f;
            a.v[i] = 0.0f;
        }
        return;
    }
    for (;;) {
        unsigned chunk = 0;
        if (lane == 0) chunk = atomicAdd(q.ctr, 1u);
        chunk = __shfl_sync(0xffffffffu, chunk, 0);
        if (chunk >= q.n_chunks) break;
        int64_t i;
        bool live;
        if (q.order) {
            const int32_t m = q.order[chunk / (unsigned)q.chunks_per_mesh];
            const int32_t k = (int32_t)(chunk % (unsigned)q.chunks_per_mesh) * 32 + (int32_t)lane;
            i = (int64_t)m * a.rays_per_mesh + k;
            live = k < a.rays_per_mesh && i < a.n;
        } else {
            const int64_t id = (int64_t)chunk * 32 + lane;
            live = id < a.n;
            i = live ? ray_index(id, a.tile_width) : 0;
        }
        if (live) {
            float3 o, d;
            float t = 0.0f;
            trace_ray<TRACER, SKIP>(a, i, stk, blockDim.x, o, d, t);
        }
    }
    if (lane == 0) {
        __threadfence();
        if (atomicAdd(q.ctr + 1, 1u) == q.n_warps - 1) {
            q.ctr[0] = 0;
            q.ctr[1] = 0;
            __threadfence();
        }
    }
}

template <int IS>
__global__ void k_shadow(TraceArgs a)
{
    extern __shared__ int2 memo_smem[];
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.n) return;
    if (a.build_err && *a.build_err) {
        a.occ[i] = 0;
        return;
    }
    a.occ[i] = trace_shadow<IS>(a.c, a.light, ld3(a.o, i), a.maxit, memo_smem + threadIdx.x, blockDim.x);
}

// Brute force (BruteTracer.cu:54-96): every ray tests every triangle in id
// order; triangles are staged through shared memory one tile at a time.
constexpr int kBruteBlock = 128;

// With `woop` set the tiles hold the Woop rows (m0, m1, m2) instead.
__global__ void __launch_bounds__(kBruteBlock) k_brute(const float4 *__restrict__ p0, const float4 *__restrict__ p1,
                                                      const float4 *__restrict__ p2, const float4 *__restrict__ woop,
                                                      int32_t T, int tie, const float *__restrict__ ro,
                                                      const float *__restrict__ rd, int64_t n, int32_t *hit,
                                                      float *ot, float *ou, float *ov)
{
    __shared__ float4 sa[kBruteBlock], sb[kBruteBlock], sc[kBruteBlock];
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const bool live = i < n;
    float3 o = make_float3(0.f, 0.f, 0.f), d = o;
    if (live) { o = ld3(ro, i); d = ld3(rd, i); }
    int h = -1;
    float tb = KDGB_FINF, ub = 0.0f, vb = 0.0f;
    for (int32_t base = 0; base < T; base += kBruteBlock) {
        const int32_t j = base + threadIdx.x;
        if (j < T && woop) {
            sa[threadIdx.x] = woop[3 * (int64_t)j];
            sb[threadIdx.x] = woop[3 * (int64_t)j + 1];
            sc[threadIdx.x] = woop[3 * (int64_t)j + 2];
        } else if (j < T) {
            const float4 a = p0[j], b = p1[j], c = p2[j];
            const float3 v0 = make_float3(a.x, a.y, a.z);
            const float3 e1 = sub3(make_float3(b.x, b.y, b.z), v0);
            const float3 e2 = sub3(make_float3(c.x, c.y, c.z), v0);
            sa[threadIdx.x] = make_float4(v0.x, v0.y, v0.z, e1.x);
            sb[threadIdx.x] = make_float4(e1.y, e1.z, e2.x, e2.y);
            sc[threadIdx.x] = make_float4(e2.z, __int_as_float(j), 0.0f, 0.0f);
        }
        __syncthreads();
        const int m = min(kBruteBlock, T - base);
        if (live && woop) {
            for (int k = 0; k < m; ++k) woop_test(sa[k], sb[k], sc[k], base + k, o, d, tie, h, tb, ub, vb);
        } else if (live) {
            for (int k = 0; k < m; ++k) {
                const float4 a = sa[k], b = sb[k], c = sc[k];
                mt_test(make_float3(a.x, a.y, a.z), make_float3(a.w, b.x, b.y), make_float3(b.z, b.w, c.x),
                        __float_as_int(c.y), o, d, tie, h, tb, ub, vb);
            }
        }
        __syncthreads();
    }
    if (!live) return;
    if (tb < KDGB_FINF) {
        hit[i] = h; ot[i] = tb; ou[i] = ub; ov[i] = vb;
    } else {
        hit[i] = -1; ot[i] = INFINITY; ou[i] = 0.0f; ov[i] = 0.0f;
    }
}

// Photon tracing (the incoherent workload): each photon leaves the light in
// a uniform direction drawn from Philox4x32-10 (key = seed, counter =
// (photon, 0)), and after every hit it survives Russian roulette with
// probability `survival` and continues in a cosine-weighted direction around
// the hit triangle's normal (counter = (photon, bounce)), from the hit point
// pushed 1e-4 along the normal.  Segment k of photon i is written to
// [i * (bounces + 1) + k]: the hit id (-1 = miss) and t, or -2 when the
// photon had already ended.
struct PhotonArgs {
    Ctx c;
    const float4 *p0, *p1, *p2;
    float3 light;
    uint2 key;
    int64_t n;
    int bounces;
    float survival;
    int tie, depth, maxit;
    int32_t *seg_hit;
    float *seg_t;
    const int32_t *build_err;  // as TraceArgs::build_err
};

// Capped at 40 registers like k_trace: 12 blocks of 128 per SM instead of 9
// (16M photons on the 262k-triangle scene: short-stack 7.54 -> 7.11 ms,
// kd-restart 11.17 -> 9.17 ms; 48 registers: 7.32 / 9.78 ms).
template <int TRACER, bool SKIP>
__global__ void __maxnreg__(40) k_photons(PhotonArgs a)
{
    extern __shared__ int2 stack_smem[];
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.n) return;
    const int S = a.bounces + 1;
    const int64_t base = i * S;
    if (a.build_err && *a.build_err) {
        for (int k = 0; k < S; ++k) {
            a.seg_hit[base + k] = -2;
            a.seg_t[base + k] = INFINITY;
        }
        return;
    }
    const unsigned lo = (unsigned)i, hi = (unsigned)(i >> 32);
    uint4 r = philox4x32_10(make_uint4(lo, hi, 0u, 0u), a.key);
    float3 o = a.light;
    float3 d = sample_sphere(u24(r.x), u24(r.y));
    int k = 0;
    while (k < S) {
        float t = 0.0f, u = 0.0f, v = 0.0f;
        int h;
        if (TRACER == KDGB_TRACER_SHORTSTACK)
            h = trace_shortstack<SKIP>(a.c, o, d, a.tie, a.depth, a.maxit, stack_smem + threadIdx.x, blockDim.x, t, u,
                                       v);
        else
            h = trace_restart<SKIP>(a.c, o, d, a.tie, a.maxit, t, u, v, nullptr, stack_smem + threadIdx.x, blockDim.x);
        a.seg_hit[base + k] = h;
        a.seg_t[base + k] = h >= 0 ? t : INFINITY;
        ++k;
        if (h < 0 || k == S) break;
        r = philox4x32_10(make_uint4(lo, hi, (unsigned)k, 0u), a.key);
        if (!(u24(r.z) < a.survival)) break;
        const float4 A = a.p0[h], B = a.p1[h], C = a.p2[h];
        const float3 v0 = make_float3(A.x, A.y, A.z);
        const float3 cr = cross3(sub3(make_float3(B.x, B.y, B.z), v0), sub3(make_float3(C.x, C.y, C.z), v0));
        const float inv = __frcp_rn(__fsqrt_rn(dot3(cr, cr)));
        float3 nrm = make_float3(__fmul_rn(cr.x, inv), __fmul_rn(cr.y, inv), __fmul_rn(cr.z, inv));
        if (dot3(nrm, d) > 0.0f) nrm = make_float3(-nrm.x, -nrm.y, -nrm.z);
        const float3 p = make_float3(__fadd_rn(o.x, __fmul_rn(t, d.x)), __fadd_rn(o.y, __fmul_rn(t, d.y)),
                                     __fadd_rn(o.z, __fmul_rn(t, d.z)));
        o = make_float3(__fadd_rn(p.x, __fmul_rn(1e-4f, nrm.x)), __fadd_rn(p.y, __fmul_rn(1e-4f, nrm.y)),
                        __fadd_rn(p.z, __fmul_rn(1e-4f, nrm.z)));
        d = sample_cosine(nrm, u24(r.x), u24(r.y));
    }
    for (; k < S; ++k) {
        a.seg_hit[base + k] = -2;
        a.seg_t[base + k] = INFINITY;
    }
}

// ---------------------------------------------------------------------------
// Shading (Raytracer.cu:165-262, ShortStack.cu:100-190, BruteTracer.cu:54-96
// with ColorKernels.h:15-85), into a headless RGBA8 buffer instead of the
// OpenGL canvas.  The un-vendored vector helpers are evaluated left to right
// with IEEE 1/sqrt in normalize (their host branch) and the specular power is
// this library's own series restatement, operation for operation the one of
// the CPU restatement, so the pixels match it bit for bit.
// ---------------------------------------------------------------------------

// x^y for x in [0, 1], y >= 0: 2^(y log2 x); log2 from the atanh series
// ln m = 2 s (1 + s^2/3 + ... + s^10/11), s = (m-1)/(m+1), m in
// [sqrt(1/2), sqrt(2)); 2^f from the Taylor series of e^(f ln 2) to the 8th
// power, f in [-1/2, 1/2]; within 2e-5 relative (the fp32 product y log2 x
// dominates at large y).
__device__ __forceinline__ float kpow(float x, float y)
{
    if (y == 0.0f) return 1.0f;
    if (!(x > 0.0f)) return 0.0f;
    if (x >= 1.0f) return 1.0f;
    int e = 0;
    if (x < 0x1p-126f) { x = __fmul_rn(x, 0x1p24f); e = -24; }
    const int b = __float_as_int(x);
    e += ((b >> 23) & 0xff) - 127;
    float m = __int_as_float((b & 0x007fffff) | 0x3f800000);
    if (m > 1.41421356f) { m = __fmul_rn(m, 0.5f); e += 1; }
    const float s = __fdiv_rn(__fsub_rn(m, 1.0f), __fadd_rn(m, 1.0f));
    const float s2 = __fmul_rn(s, s);
    float poly = 0.0909090909f;
    poly = __fadd_rn(0.111111111f, __fmul_rn(s2, poly));
    poly = __fadd_rn(0.142857143f, __fmul_rn(s2, poly));
    poly = __fadd_rn(0.2f, __fmul_rn(s2, poly));
    poly = __fadd_rn(0.333333333f, __fmul_rn(s2, poly));
    poly = __fadd_rn(1.0f, __fmul_rn(s2, poly));
    const float ln_m = __fmul_rn(__fmul_rn(2.0f, s), poly);
    const float z = __fmul_rn(y, __fadd_rn((float)e, __fmul_rn(ln_m, 1.44269504f)));
    if (z < -150.0f) return 0.0f;
    const float n = floorf(__fadd_rn(z, 0.5f));
    const float g = __fmul_rn(__fsub_rn(z, n), 0.693147181f);
    float q = 2.48015873e-5f;
    q = __fadd_rn(1.98412698e-4f, __fmul_rn(g, q));
    q = __fadd_rn(1.38888889e-3f, __fmul_rn(g, q));
    q = __fadd_rn(8.33333333e-3f, __fmul_rn(g, q));
    q = __fadd_rn(4.16666667e-2f, __fmul_rn(g, q));
    q = __fadd_rn(0.166666667f, __fmul_rn(g, q));
    q = __fadd_rn(0.5f, __fmul_rn(g, q));
    q = __fadd_rn(1.0f, __fmul_rn(g, q));
    q = __fadd_rn(1.0f, __fmul_rn(g, q));
    const int ni = (int)n, n1 = ni / 2, n2 = ni - n1;
    return __fmul_rn(__fmul_rn(q, __int_as_float((n1 + 127) << 23)), __int_as_float((n2 + 127) << 23));
}

__device__ __forceinline__ float3 nrm3(float3 v)
{
    const float inv = __fdiv_rn(1.0f, __fsqrt_rn(dot3(v, v)));
    return make_float3(__fmul_rn(v.x, inv), __fmul_rn(v.y, inv), __fmul_rn(v.z, inv));
}
__device__ __forceinline__ float sat(float x) { return x > 0.0f ? (x < 1.0f ? x : 1.0f) : 0.0f; }
__device__ __forceinline__ float clamp01(float x) { return fmaxf(0.0f, fminf(x, 1.0f)); }
__device__ __forceinline__ unsigned to_u8(float x)
{
    const float y = truncf(__fmul_rn(x, 255.0f));
    return (unsigned)(y > 0.0f ? (y < 255.0f ? y : 255.0f) : 0.0f);
}

struct Light {
    float3 pos, amb, dif, spec;
};

// PhongLighting (ColorKernels.h:15-41), shadow = 1.
__device__ __forceinline__ float4 phong(float4 c, float3 n, float3 pt, float3 origin, const Light &L)
{
    const float3 ld = nrm3(sub3(L.pos, pt));
    const float diffuse = sat(__fmul_rn(dot3(ld, n), 1.0f));
    const float k = __fmul_rn(2.0f, dot3(n, ld));
    const float3 refl = nrm3(make_float3(__fsub_rn(__fmul_rn(k, n.x), ld.x), __fsub_rn(__fmul_rn(k, n.y), ld.y),
                                         __fsub_rn(__fmul_rn(k, n.z), ld.z)));
    const float stemp = sat(dot3(nrm3(sub3(origin, pt)), refl));
    const float sp = __fsub_rn(1.0f, c.w);
    const float specular = __fmul_rn(sp, kpow(stemp, __fmul_rn(128.0f, sp)));
    const float lx = __fadd_rn(__fmul_rn(c.x, __fadd_rn(L.amb.x, __fmul_rn(L.dif.x, diffuse))),
                               __fmul_rn(__fmul_rn(__fmul_rn(L.spec.x, specular), 10.0f), 1.0f));
    const float ly = __fadd_rn(__fmul_rn(c.y, __fadd_rn(L.amb.y, __fmul_rn(L.dif.y, diffuse))),
                               __fmul_rn(__fmul_rn(__fmul_rn(L.spec.y, specular), 10.0f), 1.0f));
    const float lz = __fadd_rn(__fmul_rn(c.z, __fadd_rn(L.amb.z, __fmul_rn(L.dif.z, diffuse))),
                               __fmul_rn(__fmul_rn(__fmul_rn(L.spec.z, specular), 10.0f), 1.0f));
    return make_float4(clamp01(lx), clamp01(ly), clamp01(lz), c.w < specular ? specular : c.w);
}

struct ShadeArgs {
    Ctx c;
    const float4 *p0, *p1, *p2;   // geometry, for brute force
    int32_t T;
    const float4 *n0, *n1, *n2;   // vertex normals per triangle
    const uchar4 *c0;             // colour per triangle
    Light L;
    const float *o, *d;
    int64_t n;
    uchar4 *rgba;
    int tie, depth, maxit, max_bounces, tile_width;
    const int32_t *build_err;
};

// Exhaustive (BruteTracer.cu:54-96) from one thread: first hit over all
// triangles, no direction clamp.
__device__ __forceinline__ int brute_hit(const ShadeArgs &a, float3 o, float3 d, float &t, float &u, float &v)
{
    int hit = -1;
    float tb = KDGB_FINF, ub = 0.0f, vb = 0.0f;
    for (int32_t i = 0; i < a.T; ++i) {
        if (a.c.woop) {
            woop_test(a.c.woop + 3 * (int64_t)i, i, o, d, a.tie, hit, tb, ub, vb);
            continue;
        }
        const float4 A = __ldg(a.p0 + i), B = __ldg(a.p1 + i), C = __ldg(a.p2 + i);
        const float3 v0 = make_float3(A.x, A.y, A.z);
        mt_test(v0, sub3(make_float3(B.x, B.y, B.z), v0), sub3(make_float3(C.x, C.y, C.z), v0), i, o, d, a.tie, hit,
                tb, ub, vb);
    }
    if (!(tb < KDGB_FINF)) return -1;
    t = tb; u = ub; v = vb;
    return hit;
}

// Capped at 48 registers (53 uncapped): 1920x1080 shaded rays on the moving
// 1M-triangle surface 14.49 -> 13.93 ms (40 registers: 14.03 ms).
template <int TRACER, bool SKIP>
__global__ void __maxnreg__(48) k_shade(ShadeArgs a)
{
    extern __shared__ int2 stack_smem[];
    const int64_t id = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= a.n) return;
    const int64_t i = ray_index(id, a.tile_width);
    float4 col = make_float4(0.f, 0.f, 0.f, 0.f);
    if (!(a.build_err && *a.build_err)) {
        float3 o = ld3(a.o, i), d = ld3(a.d, i);
        if (TRACER != KDGB_TRACER_BRUTE) d = adjust_dir(d);
        for (int b = 0; b < a.max_bounces; ++b) {
            float t = 0.0f, u = 0.0f, v = 0.0f;
            float3 dh = d;
            int h;
            if (TRACER == KDGB_TRACER_SHORTSTACK)
                h = trace_shortstack<SKIP>(a.c, o, d, a.tie, a.depth, a.maxit, stack_smem + threadIdx.x, blockDim.x,
                                           t, u, v, &dh);
            else if (TRACER == KDGB_TRACER_RESTART)
                h = trace_restart<SKIP>(a.c, o, d, a.tie, a.maxit, t, u, v, &dh, stack_smem + threadIdx.x, blockDim.x);
            else
                h = brute_hit(a, o, d, t, u, v);
            if (h < 0) break;
            d = dh;
            // Lighting (ColorKernels.h:43-78).
            const float3 pt = make_float3(__fadd_rn(o.x, __fmul_rn(t, d.x)), __fadd_rn(o.y, __fmul_rn(t, d.y)),
                                          __fadd_rn(o.z, __fmul_rn(t, d.z)));
            const float w = __fsub_rn(__fsub_rn(1.0f, u), v);
            const float4 A = __ldg(a.n0 + h), B = __ldg(a.n1 + h), C = __ldg(a.n2 + h);
            const float3 nrm = nrm3(make_float3(
                __fadd_rn(__fadd_rn(__fmul_rn(w, A.x), __fmul_rn(u, B.x)), __fmul_rn(v, C.x)),
                __fadd_rn(__fadd_rn(__fmul_rn(w, A.y), __fmul_rn(u, B.y)), __fmul_rn(v, C.y)),
                __fadd_rn(__fadd_rn(__fmul_rn(w, A.z), __fmul_rn(u, B.z)), __fmul_rn(v, C.z))));
            const uchar4 cc = a.c0[h];
            float4 c = make_float4(__fdiv_rn((float)cc.x, 255.0f), __fdiv_rn((float)cc.y, 255.0f),
                                   __fdiv_rn((float)cc.z, 255.0f), __fdiv_rn((float)cc.w, 255.0f));
            const float k = __fmul_rn(2.0f, dot3(nrm, make_float3(-d.x, -d.y, -d.z)));
            const float3 nd = nrm3(make_float3(__fadd_rn(__fmul_rn(k, nrm.x), d.x), __fadd_rn(__fmul_rn(k, nrm.y), d.y),
                                               __fadd_rn(__fmul_rn(k, nrm.z), d.z)));
            c = phong(c, nrm, pt, o, a.L);
            o = make_float3(__fadd_rn(pt.x, __fmul_rn(0.00001f, nd.x)), __fadd_rn(pt.y, __fmul_rn(0.00001f, nd.y)),
                            __fadd_rn(pt.z, __fmul_rn(0.00001f, nd.z)));
            d = nd;
            // BlendColor (ColorKernels.h:80-85).
            const float kk = __fmul_rn(__fsub_rn(1.0f, col.w), c.w);
            col = make_float4(__fadd_rn(col.x, __fmul_rn(kk, c.x)), __fadd_rn(col.y, __fmul_rn(kk, c.y)),
                              __fadd_rn(col.z, __fmul_rn(kk, c.z)), __fadd_rn(col.w, __fmul_rn(kk, 1.0f)));
            if (TRACER != KDGB_TRACER_BRUTE) d = adjust_dir(d);
            if (!(col.w < 0.97f)) break;
        }
    }
    a.rgba[i] = make_uchar4((unsigned char)to_u8(col.x), (unsigned char)to_u8(col.y), (unsigned char)to_u8(col.z),
                            (unsigned char)to_u8(col.w));
}

// CreateWoopValues (GeometryList.cu:81-102): WoopTransformationMatrix
// (IntersectionTests.h:438-467) of (p1, p2, p0), the inverse of the matrix
// whose columns are a - c, b - c and (a - c) x (b - c) - c, rows scaled by
// 1/det, each row's w = row . c.
__global__ void k_woop_values(const float4 *__restrict__ p0, const float4 *__restrict__ p1,
                              const float4 *__restrict__ p2, int32_t T, float4 *__restrict__ out)
{
    const int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= T) return;
    const float4 A = p1[i], B = p2[i], C = p0[i];
    const float3 a = make_float3(A.x, A.y, A.z), b = make_float3(B.x, B.y, B.z), c = make_float3(C.x, C.y, C.z);
    const float3 m0 = sub3(a, c), m1 = sub3(b, c), m2 = sub3(cross3(m0, m1), c);
    const float det = __fadd_rn(
        __fadd_rn(__fmul_rn(m0.x, __fsub_rn(__fmul_rn(m1.y, m2.z), __fmul_rn(m1.z, m2.y))),
                  __fmul_rn(m1.x, __fsub_rn(__fmul_rn(m2.y, m0.z), __fmul_rn(m2.z, m0.y)))),
        __fmul_rn(m2.x, __fsub_rn(__fmul_rn(m0.y, m1.z), __fmul_rn(m0.z, m1.y))));
    const float inv = __fdiv_rn(1.0f, det);
    const float3 r0 = make_float3(__fmul_rn(__fsub_rn(__fmul_rn(m1.y, m2.z), __fmul_rn(m1.z, m2.y)), inv),
                                  __fmul_rn(__fsub_rn(__fmul_rn(m2.x, m1.z), __fmul_rn(m2.z, m1.x)), inv),
                                  __fmul_rn(__fsub_rn(__fmul_rn(m1.x, m2.y), __fmul_rn(m1.y, m2.x)), inv));
    const float3 r1 = make_float3(__fmul_rn(__fsub_rn(__fmul_rn(m2.y, m0.z), __fmul_rn(m2.z, m0.y)), inv),
                                  __fmul_rn(__fsub_rn(__fmul_rn(m0.x, m2.z), __fmul_rn(m0.z, m2.x)), inv),
                                  __fmul_rn(__fsub_rn(__fmul_rn(m2.x, m0.y), __fmul_rn(m2.y, m0.x)), inv));
    const float3 r2 = make_float3(__fmul_rn(__fsub_rn(__fmul_rn(m0.y, m1.z), __fmul_rn(m0.z, m1.y)), inv),
                                  __fmul_rn(__fsub_rn(__fmul_rn(m1.x, m0.z), __fmul_rn(m1.z, m0.x)), inv),
                                  __fmul_rn(__fsub_rn(__fmul_rn(m0.x, m1.y), __fmul_rn(m0.y, m1.x)), inv));
    out[3 * (int64_t)i + 0] = make_float4(r0.x, r0.y, r0.z, dot3(r0, c));
    out[3 * (int64_t)i + 1] = make_float4(r1.x, r1.y, r1.z, dot3(r1, c));
    out[3 * (int64_t)i + 2] = make_float4(r2.x, r2.y, r2.z, dot3(r2, c));
}

}  // namespace

int woop_values(const Tree &t, cudaStream_t s)
{
    if (t.woop_valid) return KDGB_OK;
    KDGB_CHECK(ensure(t.woop, 3 * (int64_t)std::max(t.n_tris, 1), s));
    if (t.n_tris > 0) {
        k_woop_values<<<blocks_for(t.n_tris, 256), 256, 0, s>>>(t.p0.p, t.p1.p, t.p2.p, t.n_tris, t.woop.p);
        KDGB_LAUNCH_CHECK();
    }
    t.woop_valid = true;
    return KDGB_OK;
}

// Sets c.woop to the Woop rows for the trace parameters (NULL for
// Moeller-Trumbore).
static int woop_for(const Tree &t, const kdgb_trace_params &p, cudaStream_t s, Ctx &c)
{
    c.woop = nullptr;
    if (p.intersection != KDGB_ISECT_WOOP) return KDGB_OK;
    KDGB_CHECK(woop_values(t, s));
    c.woop = t.woop.p;
    return KDGB_OK;
}


// The persistent queue-scheduled launch (k_trace_queue) for trace_launch.
static int trace_queue_launch(const Tree &t, const kdgb_trace_params &p, const TraceArgs &a, int bs, size_t smem,
                              cudaStream_t s)
{
    void (*kernel)(TraceArgs, TraceQueue);
    const bool skip = p.leaf_skipping != 0;
    if (p.tracer == KDGB_TRACER_SHORTSTACK)
        kernel = skip ? k_trace_queue<KDGB_TRACER_SHORTSTACK, true> : k_trace_queue<KDGB_TRACER_SHORTSTACK, false>;
    else
        kernel = skip ? k_trace_queue<KDGB_TRACER_RESTART, true> : k_trace_queue<KDGB_TRACER_RESTART, false>;
    if (smem > 48 * 1024) KDGB_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    Tree &tm = const_cast<Tree &>(t);
    if (!t.qctr.p) KDGB_CHECK(ensure(tm.qctr, 2, s, 0, true));
    int per_sm = 0, dev = 0, sms = 0;
    KDGB_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, bs, smem));
    KDGB_CUDA(cudaGetDevice(&dev));
    KDGB_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    TraceQueue q;
    q.ctr = t.qctr.p;
    q.order = nullptr;
    q.chunks_per_mesh = 1;
    int64_t chunks = (a.n + 31) / 32;
    if (a.mesh_off && !a.ray_mesh && t.mesh_order.p) {
        q.order = t.mesh_order.p;
        q.chunks_per_mesh = (a.rays_per_mesh + 31) / 32;
        chunks = (int64_t)q.chunks_per_mesh * a.n_meshes;
    }
    if (chunks >= (int64_t)0xffffffffll) return fail(KDGB_ERR_CAPACITY, "queue trace: too many ray chunks");
    q.n_chunks = (unsigned)chunks;
    const int64_t blocks = std::min<int64_t>((int64_t)std::max(per_sm, 1) * sms, std::max<int64_t>(1, (a.n + bs - 1) / bs));
    q.n_warps = (unsigned)(blocks * (bs / 32));
    kernel<<<(unsigned)blocks, bs, smem, s>>>(a, q);
    KDGB_LAUNCH_CHECK();
    return KDGB_OK;
}

// The k_trace instance of a launch: tracer, leaf skipping, fused shadow
// rays and intersection test are template parameters, and blocks of
// kFixedBlock threads get the instance with that constant stride and, for
// the short-stack tracer, a stack of exactly kFixedDepth entries (the other
// tracers keep kMemo entries whatever the depth): the ring's wrap-around is
// then a mask (fused frame trace 1.177 -> 1.155 ms, primary rays alone
// 0.659 -> 0.638 ms, bit-identical).
constexpr int kFixedBlock = 128;
constexpr int kFixedDepth = 8;
static_assert((kFixedDepth & (kFixedDepth - 1)) == 0, "the fixed depth's ring wraps by a mask: a power of two");

template <int TRACER, bool SKIP, bool SHADOW, int IS>
static void (*trace_kernel_bs(bool fixed_block))(TraceArgs)
{
    return fixed_block ? k_trace<TRACER, SKIP, SHADOW, IS, false, kFixedBlock, kFixedDepth> : k_trace<TRACER, SKIP, SHADOW, IS>;
}

template <int TRACER, bool SKIP, bool SHADOW>
static void (*trace_kernel_is(bool woop, bool fixed_block))(TraceArgs)
{
    return woop ? trace_kernel_bs<TRACER, SKIP, SHADOW, KDGB_ISECT_WOOP>(fixed_block)
                : trace_kernel_bs<TRACER, SKIP, SHADOW, KDGB_ISECT_MOELLER>(fixed_block);
}

template <int TRACER>
static void (*trace_kernel_tr(bool skip, bool shadow, bool woop, bool fb))(TraceArgs)
{
    return skip ? (shadow ? trace_kernel_is<TRACER, true, true>(woop, fb) : trace_kernel_is<TRACER, true, false>(woop, fb))
                : (shadow ? trace_kernel_is<TRACER, false, true>(woop, fb)
                          : trace_kernel_is<TRACER, false, false>(woop, fb));
}

static void (*trace_kernel(bool shortstack, bool skip, bool shadow, bool woop, bool fixed_block))(TraceArgs)
{
    return shortstack ? trace_kernel_tr<KDGB_TRACER_SHORTSTACK>(skip, shadow, woop, fixed_block)
                      : trace_kernel_tr<KDGB_TRACER_RESTART>(skip, shadow, woop, fixed_block);
}

int trace_launch(const Tree &t, const kdgb_trace_params &p, const float *o, const float *d, int64_t n,
                 int32_t *hit, float *tt, float *uu, float *vv, int32_t *occ, const float *light, cudaStream_t s,
                 const int32_t *ray_mesh, int32_t rays_per_mesh, unsigned long long *counts)
{
    TraceArgs a;
    a.c.node = t.tnode.p;
    a.c.box = t.tbox.p;
    a.c.tri = t.ttri.p;
    a.c.root = 0;
    KDGB_CHECK(woop_for(t, p, s, a.c));
    a.mesh_off = nullptr;
    a.ray_mesh = nullptr;
    a.rays_per_mesh = 1;
    a.n_meshes = 1;
    a.build_err = t.ws.state.p ? &t.ws.state.p->err : nullptr;
    if (t.n_meshes > 1) {
        a.mesh_off = t.mesh_off.p;
        a.ray_mesh = ray_mesh;
        a.rays_per_mesh = rays_per_mesh > 0 ? rays_per_mesh : 1;
        a.n_meshes = t.n_meshes;
    }
    a.o = o; a.d = d; a.n = n;
    a.hit = hit; a.t = tt; a.u = uu; a.v = vv; a.occ = occ;
    a.light = light ? make_float3(light[0], light[1], light[2]) : make_float3(0.f, 0.f, 0.f);
    a.tie = p.tie;
    a.depth = p.stack_depth;
    a.maxit = p.max_iterations > 0 ? p.max_iterations : kDefaultMaxIterations;
    a.tile_width = p.tile_width;
    const int bs = p.block_size > 0 ? p.block_size : 128;
    const unsigned grid = blocks_for(n, bs);
    const bool skip = p.leaf_skipping != 0;
    const bool shadow = occ != nullptr;
    // With shadow rays the block's queue (one ShadowItem, two int2, per
    // thread) overlays the stack region.
    const size_t smem = sizeof(int2) * (size_t)std::max(stack_entries(p.tracer, p.stack_depth), shadow ? 2 : 0) * bs;
    // The constant-stride instance only for blocks of exactly its size.
    void (*kernel)(TraceArgs) =
        trace_kernel(p.tracer == KDGB_TRACER_SHORTSTACK, skip, shadow, a.c.woop != nullptr,
                     bs == kFixedBlock && (p.tracer != KDGB_TRACER_SHORTSTACK || p.stack_depth == kFixedDepth));
    if (counts) {  // the counting launch: short-stack primary rays with fused shadow rays only
        if (p.tracer != KDGB_TRACER_SHORTSTACK || !shadow || t.n_meshes > 1)
            return fail(KDGB_ERR_UNSUPPORTED, "step counts are kept for short-stack primary + shadow traces only");
        a.counts = counts;
        kernel = skip ? (a.c.woop ? k_trace<KDGB_TRACER_SHORTSTACK, true, true, KDGB_ISECT_WOOP, true>
                                  : k_trace<KDGB_TRACER_SHORTSTACK, true, true, KDGB_ISECT_MOELLER, true>)
                      : (a.c.woop ? k_trace<KDGB_TRACER_SHORTSTACK, false, true, KDGB_ISECT_WOOP, true>
                                  : k_trace<KDGB_TRACER_SHORTSTACK, false, true, KDGB_ISECT_MOELLER, true>);
    }
    if (p.schedule == KDGB_SCHEDULE_QUEUE && !shadow) return trace_queue_launch(t, p, a, bs, smem, s);
    // Large blocks with deep stacks need more than the default 48 KB.
    if (smem > 48 * 1024) KDGB_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    kernel<<<grid, bs, smem, s>>>(a);
    KDGB_LAUNCH_CHECK();
    return KDGB_OK;
}

int shadow_launch(const Tree &t, const kdgb_trace_params &p, const float *pts, int64_t n, const float *light,
                  int32_t *occ, cudaStream_t s)
{
    TraceArgs a;
    a.c.node = t.tnode.p;
    a.c.box = t.tbox.p;
    a.c.tri = t.ttri.p;
    a.c.root = 0;
    KDGB_CHECK(woop_for(t, p, s, a.c));
    a.mesh_off = nullptr;
    a.ray_mesh = nullptr;
    a.rays_per_mesh = 1;
    a.n_meshes = 1;
    a.build_err = t.ws.state.p ? &t.ws.state.p->err : nullptr;
    a.o = pts; a.d = nullptr; a.n = n;
    a.hit = nullptr; a.t = a.u = a.v = nullptr; a.occ = occ;
    a.light = make_float3(light[0], light[1], light[2]);
    a.tie = p.tie; a.depth = p.stack_depth;
    a.maxit = p.max_iterations > 0 ? p.max_iterations : kDefaultMaxIterations;
    a.tile_width = 0;
    const int bs = p.block_size > 0 ? p.block_size : 128;
    const size_t smem = sizeof(int2) * (size_t)kMemo * bs;
    void (*kernel)(TraceArgs) = a.c.woop ? k_shadow<KDGB_ISECT_WOOP> : k_shadow<KDGB_ISECT_MOELLER>;
    if (smem > 48 * 1024)
        KDGB_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    kernel<<<blocks_for(n, bs), bs, smem, s>>>(a);
    KDGB_LAUNCH_CHECK();
    return KDGB_OK;
}

int brute_launch(const float4 *p0, const float4 *p1, const float4 *p2, const float4 *woop, int32_t T, int tie,
                 const float *o, const float *d, int64_t n, int32_t *hit, float *tt, float *uu, float *vv,
                 cudaStream_t s)
{
    k_brute<<<blocks_for(n, kBruteBlock), kBruteBlock, 0, s>>>(p0, p1, p2, woop, T, tie, o, d, n, hit, tt, uu, vv);
    KDGB_LAUNCH_CHECK();
    return KDGB_OK;
}

int photon_launch(const Tree &t, const kdgb_trace_params &p, const kdgb_photon_params &ph, int64_t n,
                  int32_t *seg_hit, float *seg_t, cudaStream_t s)
{
    PhotonArgs a;
    a.c.node = t.tnode.p;
    a.c.box = t.tbox.p;
    a.c.tri = t.ttri.p;
    a.c.root = 0;
    KDGB_CHECK(woop_for(t, p, s, a.c));
    a.p0 = t.p0.p; a.p1 = t.p1.p; a.p2 = t.p2.p;
    a.light = make_float3(ph.light[0], ph.light[1], ph.light[2]);
    a.key = make_uint2((unsigned)(ph.seed & 0xffffffffu), (unsigned)(ph.seed >> 32));
    a.n = n;
    a.bounces = ph.bounces;
    a.survival = ph.survival;
    a.tie = p.tie;
    a.depth = p.stack_depth;
    a.maxit = p.max_iterations > 0 ? p.max_iterations : kDefaultMaxIterations;
    a.seg_hit = seg_hit;
    a.seg_t = seg_t;
    a.build_err = t.ws.state.p ? &t.ws.state.p->err : nullptr;
    const int bs = p.block_size > 0 ? p.block_size : 128;
    const unsigned grid = blocks_for(n, bs);
    const bool skip = p.leaf_skipping != 0;
    {
        const size_t smem = sizeof(int2) * (size_t)stack_entries(p.tracer, p.stack_depth) * bs;
        void (*kernel)(PhotonArgs);
        if (p.tracer == KDGB_TRACER_SHORTSTACK)
            kernel = skip ? k_photons<KDGB_TRACER_SHORTSTACK, true> : k_photons<KDGB_TRACER_SHORTSTACK, false>;
        else
            kernel = skip ? k_photons<KDGB_TRACER_RESTART, true> : k_photons<KDGB_TRACER_RESTART, false>;
        if (smem > 48 * 1024)
            KDGB_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        kernel<<<grid, bs, smem, s>>>(a);
    }
    KDGB_LAUNCH_CHECK();
    return KDGB_OK;
}

int shade_launch(const Tree &t, const kdgb_trace_params &p, const float *n0, const float *n1, const float *n2,
                 const uint8_t *c0, const kdgb_light &light, int max_bounces, const float *o, const float *d, int64_t n,
                 uint8_t *rgba, cudaStream_t s)
{
    ShadeArgs a;
    a.c.node = t.tnode.p;
    a.c.box = t.tbox.p;
    a.c.tri = t.ttri.p;
    a.c.root = 0;
    KDGB_CHECK(woop_for(t, p, s, a.c));
    a.p0 = t.p0.p; a.p1 = t.p1.p; a.p2 = t.p2.p;
    a.T = t.n_tris;
    a.n0 = reinterpret_cast<const float4 *>(n0);
    a.n1 = reinterpret_cast<const float4 *>(n1);
    a.n2 = reinterpret_cast<const float4 *>(n2);
    a.c0 = reinterpret_cast<const uchar4 *>(c0);
    a.L.pos = make_float3(light.position[0], light.position[1], light.position[2]);
    a.L.amb = make_float3(light.ambient[0], light.ambient[1], light.ambient[2]);
    a.L.dif = make_float3(light.diffuse[0], light.diffuse[1], light.diffuse[2]);
    a.L.spec = make_float3(light.specular[0], light.specular[1], light.specular[2]);
    a.o = o; a.d = d; a.n = n;
    a.rgba = reinterpret_cast<uchar4 *>(rgba);
    a.tie = p.tie;
    a.depth = p.stack_depth;
    a.maxit = p.max_iterations > 0 ? p.max_iterations : kDefaultMaxIterations;
    a.max_bounces = max_bounces;
    a.tile_width = p.tile_width;
    a.build_err = t.ws.state.p ? &t.ws.state.p->err : nullptr;
    const int bs = p.block_size > 0 ? p.block_size : 128;
    const unsigned grid = blocks_for(n, bs);
    const bool skip = p.leaf_skipping != 0;
    if (p.tracer == KDGB_TRACER_SHORTSTACK || p.tracer == KDGB_TRACER_RESTART) {
        const size_t smem = sizeof(int2) * (size_t)stack_entries(p.tracer, p.stack_depth) * bs;
        void (*kernel)(ShadeArgs);
        if (p.tracer == KDGB_TRACER_SHORTSTACK)
            kernel = skip ? k_shade<KDGB_TRACER_SHORTSTACK, true> : k_shade<KDGB_TRACER_SHORTSTACK, false>;
        else
            kernel = skip ? k_shade<KDGB_TRACER_RESTART, true> : k_shade<KDGB_TRACER_RESTART, false>;
        if (smem > 48 * 1024)
            KDGB_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        kernel<<<grid, bs, smem, s>>>(a);
    } else {
        k_shade<KDGB_TRACER_BRUTE, false><<<grid, bs, 0, s>>>(a);
    }
    KDGB_LAUNCH_CHECK();
    return KDGB_OK;
}

}  // namespace kdgb
