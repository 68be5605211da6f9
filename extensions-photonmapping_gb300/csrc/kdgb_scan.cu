// Device-wide exclusive prefix sums of multi-lane int32 records.
//
// The reference scans with CUDPP (TriangleMapUpperCreator.cu:58-76, one plan
// of 262,144 elements, return codes ignored).  This replacement scans records
// of K independent lanes read through a loader (a plain array, or lanes
// computed on the fly from other arrays).  Up to kSingleMax records one
// block of 1024 threads scans everything in a single launch; above that a
// reduce-then-scan takes three launches (block totals, a single-block scan
// of the totals, a rescan of each block with its offset).  No block ever
// waits for another, so the scan cannot hang, and it has no size cap below
// 2^31 records.  The length may live in device memory (a build counter): the
// grids are then sized for an upper bound and blocks past the real length do
// nothing, so the scan can be captured once into a graph and replayed for
// any length up to the bound.
#include "kdgb_internal.cuh"

namespace kdgb {

namespace {

constexpr int kThreads = 256;
constexpr int kItems = 4;
constexpr int kTile = kThreads * kItems;
constexpr int kSingleThreads = 1024;
constexpr int kSingleTile = kSingleThreads * kItems;
constexpr int64_t kSingleMax = 16384;

// Exclusive block scan of one value per lane per thread.  Returns the block
// total of every lane in `total`.
template <int K, int THREADS>
__device__ __forceinline__ void block_scan(int32_t (&v)[K], int32_t (&total)[K])
{
    constexpr int W = THREADS / 32;
    __shared__ int32_t warp_sum[K][W];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int32_t incl[K];
#pragma unroll
    for (int k = 0; k < K; ++k) {
        int32_t x = v[k];
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int32_t y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        incl[k] = x;
        if (lane == 31) warp_sum[k][warp] = x;
    }
    __syncthreads();
    if (warp == 0) {
#pragma unroll
        for (int k = 0; k < K; ++k) {
            int32_t x = lane < W ? warp_sum[k][lane] : 0;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int32_t y = __shfl_up_sync(0xffffffffu, x, o);
                if (lane >= o) x += y;
            }
            if (lane < W) warp_sum[k][lane] = x;  // inclusive over warps
        }
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < K; ++k) {
        const int32_t before = warp > 0 ? warp_sum[k][warp - 1] : 0;
        total[k] = warp_sum[k][W - 1];
        v[k] = before + incl[k] - v[k];
    }
    __syncthreads();
}

// Loads kItems consecutive records starting at `base` (zeros past n) and
// returns their per-lane sums.
template <int K, class In>
__device__ __forceinline__ void load_items(const In &in, int64_t base, int64_t n, int32_t (&vals)[kItems][K],
                                           int32_t (&s)[K])
{
#pragma unroll
    for (int k = 0; k < K; ++k) s[k] = 0;
#pragma unroll
    for (int i = 0; i < kItems; ++i) {
        if (base + i < n) {
            in.load(base + i, vals[i]);
        } else {
#pragma unroll
            for (int k = 0; k < K; ++k) vals[i][k] = 0;
        }
#pragma unroll
        for (int k = 0; k < K; ++k) s[k] += vals[i][k];
    }
}

// One block, any n: segments of kSingleTile records with a running carry;
// writes the totals record out[n].
template <int K, class In>
__global__ void __launch_bounds__(kSingleThreads) scan_single_kernel(const In in, int32_t *__restrict__ out, int64_t n,
                                                                     const int32_t *__restrict__ n_dev)
{
    if (n_dev) n = *n_dev;
    int32_t carry[K];
#pragma unroll
    for (int k = 0; k < K; ++k) carry[k] = 0;
    for (int64_t start = 0; start < n; start += kSingleTile) {
        const int64_t base = start + (int64_t)threadIdx.x * kItems;
        int32_t vals[kItems][K], s[K], tot[K];
        load_items<K>(in, base, n, vals, s);
        block_scan<K, kSingleThreads>(s, tot);
#pragma unroll
        for (int i = 0; i < kItems; ++i) {
#pragma unroll
            for (int k = 0; k < K; ++k) {
                if (base + i < n) out[(base + i) * K + k] = carry[k] + s[k];
                s[k] += vals[i][k];
            }
        }
#pragma unroll
        for (int k = 0; k < K; ++k) carry[k] += tot[k];
    }
    if (threadIdx.x == 0) {
#pragma unroll
        for (int k = 0; k < K; ++k) out[n * K + k] = carry[k];
    }
}

template <int K, class In>
__global__ void __launch_bounds__(kThreads) scan_reduce_kernel(const In in, int64_t n,
                                                               const int32_t *__restrict__ n_dev,
                                                               int32_t *__restrict__ partial)
{
    if (n_dev) n = *n_dev;
    if ((int64_t)blockIdx.x * kTile >= n) return;  // block-uniform
    const int64_t base = (int64_t)blockIdx.x * kTile + (int64_t)threadIdx.x * kItems;
    int32_t vals[kItems][K], s[K], tot[K];
    load_items<K>(in, base, n, vals, s);
    block_scan<K, kThreads>(s, tot);
    if (threadIdx.x == 0) {
#pragma unroll
        for (int k = 0; k < K; ++k) partial[(int64_t)blockIdx.x * K + k] = tot[k];
    }
}

// Single block: exclusive scan of the block partials in place; writes the
// grand totals to out[n].
template <int K>
__global__ void __launch_bounds__(kSingleThreads) scan_partials_kernel(int32_t *__restrict__ partial, int64_t n,
                                                                       const int32_t *__restrict__ n_dev,
                                                                       int32_t *__restrict__ out)
{
    if (n_dev) n = *n_dev;
    const int64_t nb = (n + kTile - 1) / kTile;
    int32_t carry[K];
#pragma unroll
    for (int k = 0; k < K; ++k) carry[k] = 0;
    const ScanArray<K> in{partial};
    for (int64_t start = 0; start < nb; start += kSingleTile) {
        const int64_t b = start + (int64_t)threadIdx.x * kItems;
        int32_t vals[kItems][K], s[K], tot[K];
        load_items<K>(in, b, nb, vals, s);
        block_scan<K, kSingleThreads>(s, tot);
#pragma unroll
        for (int i = 0; i < kItems; ++i) {
#pragma unroll
            for (int k = 0; k < K; ++k) {
                if (b + i < nb) partial[(b + i) * K + k] = carry[k] + s[k];
                s[k] += vals[i][k];
            }
        }
#pragma unroll
        for (int k = 0; k < K; ++k) carry[k] += tot[k];
    }
    if (threadIdx.x == 0) {
#pragma unroll
        for (int k = 0; k < K; ++k) out[n * K + k] = carry[k];
    }
}

template <int K, class In>
__global__ void __launch_bounds__(kThreads) scan_down_kernel(const In in, int32_t *__restrict__ out, int64_t n,
                                                             const int32_t *__restrict__ n_dev,
                                                             const int32_t *__restrict__ partial)
{
    if (n_dev) n = *n_dev;
    if ((int64_t)blockIdx.x * kTile >= n) return;  // block-uniform
    const int64_t base = (int64_t)blockIdx.x * kTile + (int64_t)threadIdx.x * kItems;
    int32_t vals[kItems][K], s[K], tot[K];
    load_items<K>(in, base, n, vals, s);
    block_scan<K, kThreads>(s, tot);
#pragma unroll
    for (int k = 0; k < K; ++k) s[k] += partial[(int64_t)blockIdx.x * K + k];
#pragma unroll
    for (int i = 0; i < kItems; ++i) {
#pragma unroll
        for (int k = 0; k < K; ++k) {
            if (base + i < n) out[(base + i) * K + k] = s[k];
            s[k] += vals[i][k];
        }
    }
}

}  // namespace

int64_t scan_partials_needed(int K, int64_t n) { return n <= kSingleMax ? 0 : K * ((n + kTile - 1) / kTile); }

template <int K, class In>
int scan_exclusive_in(const In &in, int32_t *out, int64_t n, cudaStream_t s, DevArray<int32_t> *ws,
                      const int32_t *n_dev)
{
    if (n < 0) return fail(KDGB_ERR_INVALID_ARGUMENT, "scan: negative length");
    if (n == 0) {
        KDGB_CUDA(cudaMemsetAsync(out, 0, sizeof(int32_t) * K, s));
        return KDGB_OK;
    }
    if (n <= kSingleMax) {
        scan_single_kernel<K, In><<<1, kSingleThreads, 0, s>>>(in, out, n, n_dev);
        KDGB_LAUNCH_CHECK();
        return KDGB_OK;
    }
    const int64_t nb = (n + kTile - 1) / kTile;
    int32_t *partial = nullptr;
    if (ws) {
        KDGB_CHECK(grab(*ws, K * nb, s));
        partial = ws->p;
    } else {
        KDGB_CUDA(cudaMallocAsync(&partial, sizeof(int32_t) * K * (size_t)nb, s));
    }
    scan_reduce_kernel<K, In><<<(unsigned)nb, kThreads, 0, s>>>(in, n, n_dev, partial);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) {
        scan_partials_kernel<K><<<1, kSingleThreads, 0, s>>>(partial, n, n_dev, out);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) {
        scan_down_kernel<K, In><<<(unsigned)nb, kThreads, 0, s>>>(in, out, n, n_dev, partial);
        e = cudaGetLastError();
    }
    if (!ws) cudaFreeAsync(partial, s);
    if (e != cudaSuccess) return cuda_fail(e, "scan kernels");
    note_launch(3);
    return KDGB_OK;
}

template int scan_exclusive_in<1, ScanArray<1>>(const ScanArray<1> &, int32_t *, int64_t, cudaStream_t,
                                             DevArray<int32_t> *, const int32_t *);
template int scan_exclusive_in<2, ScanArray<2>>(const ScanArray<2> &, int32_t *, int64_t, cudaStream_t,
                                             DevArray<int32_t> *, const int32_t *);
template int scan_exclusive_in<7, ScanArray<7>>(const ScanArray<7> &, int32_t *, int64_t, cudaStream_t,
                                             DevArray<int32_t> *, const int32_t *);
template int scan_exclusive_in<7, NodeLanes>(const NodeLanes &, int32_t *, int64_t, cudaStream_t, DevArray<int32_t> *,
                                          const int32_t *);

}  // namespace kdgb
