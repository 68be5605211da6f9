// Device-wide exclusive prefix sums of multi-lane int32 records.
//
// The reference scans with CUDPP (TriangleMapUpperCreator.cu:58-76, one plan
// of 262,144 elements, return codes ignored).  This replacement scans records
// of K independent lanes read through a loader (a plain array, or lanes
// computed on the fly from other arrays) in ONE launch, whatever the length:
// a single-pass scan with decoupled look-back.  Each block takes a tile of
// kTile records in the order blocks start (a ticket counter), scans it,
// publishes the tile's totals at once and then the inclusive prefix once it
// knows its predecessors' prefix, which it assembles by looking back over
// the published tiles (32 at a time, one lane each).  A block only ever
// waits for tiles whose blocks started before it and publish without
// waiting, so every wait ends; each wait is still bounded and a scan that
// gives up records KDGB_ERR_TIMEOUT.  Status flags carry the invocation's
// epoch, so the status array is never cleared between scans; the last block
// of an invocation resets the ticket counter and advances the epoch.
//
// The length may live in device memory (a build counter): the grid is then
// sized for an upper bound and tiles past the real length do nothing, so the
// scan can be captured once into a graph and replayed for any length up to
// the bound.
#include "kdgb_internal.cuh"

#include <algorithm>
#include <vector>

namespace kdgb {

namespace {

constexpr int kThreads = 256;
constexpr int kItems = 4;
constexpr int kTile = kThreads * kItems;
constexpr unsigned kFull = 0xffffffffu;

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

// Scan state in the workspace array: kCtl control words, then kStatus ints
// per tile: the tile totals (K <= 7 lanes, written once), the inclusive
// prefix (8 + k) and a flag word (epoch << 2 | kind) at kFlag.  Totals and
// prefix live apart, so a reader that saw either kind reads values that no
// later store of the same epoch changes.
constexpr int kCtl = 4;  // ticket, finished blocks, epoch, spare
constexpr int kStatus = 16;
constexpr int kIncl = 8;
constexpr int kFlag = 15;
constexpr unsigned kAggregate = 1, kPrefix = 2;
constexpr int kSpinLimit = 1 << 22;

__device__ __forceinline__ unsigned load_flag(const int32_t *p)
{
    return *(const volatile unsigned *)p;
}

// One tile of a single-pass scan, run by a whole block: tile `tile` of the
// n records of `in`, with its status in `status` (tiles of this scan only).
template <int K, class In>
__device__ __forceinline__ void scan_tile(const In &in, int32_t *__restrict__ out, int64_t n, int64_t tile,
                                          int32_t *status, unsigned epoch, int32_t *err,
                                          int spin_limit = kSpinLimit)
{
    // The tile's records, then their exclusive prefixes: loaded and stored
    // striped (consecutive threads, consecutive records, so every access is
    // coalesced), scanned blocked (kItems consecutive records per thread).
    __shared__ int32_t s_rec[kTile * K];
    __shared__ int32_t s_excl[K];
    const int64_t ntiles = (n + kTile - 1) / kTile;
    if (tile >= ntiles) {  // block-uniform
        if (tile == 0 && threadIdx.x < K) out[threadIdx.x] = 0;  // n == 0: the totals record only
        return;
    }
    const int64_t tbase = tile * kTile;
#pragma unroll
    for (int i = 0; i < kItems; ++i) {
        const int j = i * kThreads + threadIdx.x;
        int32_t v[K];
        if (tbase + j < n) {
            in.load(tbase + j, v);
        } else {
#pragma unroll
            for (int k = 0; k < K; ++k) v[k] = 0;
        }
#pragma unroll
        for (int k = 0; k < K; ++k) s_rec[j * K + k] = v[k];
    }
    __syncthreads();
    int32_t vals[kItems][K], s[K], tot[K];
#pragma unroll
    for (int k = 0; k < K; ++k) s[k] = 0;
#pragma unroll
    for (int i = 0; i < kItems; ++i) {
#pragma unroll
        for (int k = 0; k < K; ++k) {
            vals[i][k] = s_rec[(threadIdx.x * kItems + i) * K + k];
            s[k] += vals[i][k];
        }
    }
    block_scan<K, kThreads>(s, tot);  // its barriers also end the reads of s_rec above
    int32_t *mine = status + kStatus * tile;
    if (threadIdx.x == 0) {
        // Publish the tile totals (for tile 0 they are the inclusive prefix).
        const int off = tile == 0 ? kIncl : 0;
#pragma unroll
        for (int k = 0; k < K; ++k) ((volatile int32_t *)mine)[off + k] = tot[k];
        __threadfence();
        ((volatile unsigned *)mine)[kFlag] = (epoch << 2) | (tile == 0 ? kPrefix : kAggregate);
    }
    if (threadIdx.x < 32) {
        const int lane = threadIdx.x;
        int32_t excl[K];
#pragma unroll
        for (int k = 0; k < K; ++k) excl[k] = 0;
        int64_t j = tile - 1;  // nearest unread predecessor
        while (j >= 0) {      // warp-uniform
            const int64_t t = j - lane;
            unsigned f = 0;
            bool dead = false;
            if (t >= 0) {
                int spins = 0;
                f = load_flag(status + kStatus * t + kFlag);
                while ((f >> 2) != epoch || (f & 3u) == 0) {
                    if (++spins > spin_limit) {
                        if (err) atomicCAS(err, 0, KDGB_ERR_TIMEOUT);
                        f = (epoch << 2) | kPrefix;  // give up: count it as a zero prefix
                        dead = true;
                        break;
                    }
                    __nanosleep(64);
                    f = load_flag(status + kStatus * t + kFlag);
                }
            }
            __threadfence();
            // Lanes up to the first prefix (nearest predecessor first) count.
            const unsigned pm = __ballot_sync(kFull, t >= 0 && (f & 3u) == kPrefix);
            const int stop = pm ? __ffs(pm) - 1 : 31;
            const bool use = t >= 0 && lane <= stop && !dead;
            const int off = (f & 3u) == kPrefix ? kIncl : 0;
#pragma unroll
            for (int k = 0; k < K; ++k) {
                int32_t v = use ? ((const volatile int32_t *)(status + kStatus * t))[off + k] : 0;
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(kFull, v, o);
                excl[k] += v;
            }
            if (pm) break;
            j -= 32;
        }
        if (lane == 0) {
#pragma unroll
            for (int k = 0; k < K; ++k) s_excl[k] = excl[k];
            if (tile > 0) {
#pragma unroll
                for (int k = 0; k < K; ++k) ((volatile int32_t *)mine)[kIncl + k] = excl[k] + tot[k];
                __threadfence();
                ((volatile unsigned *)mine)[kFlag] = (epoch << 2) | kPrefix;
            }
        }
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < K; ++k) s[k] += s_excl[k];
#pragma unroll
    for (int i = 0; i < kItems; ++i) {
#pragma unroll
        for (int k = 0; k < K; ++k) {
            s_rec[(threadIdx.x * kItems + i) * K + k] = s[k];
            s[k] += vals[i][k];
        }
    }
    __syncthreads();
    const int valid = (int)(n - tbase < kTile ? n - tbase : kTile);
    for (int f = threadIdx.x; f < valid * K; f += kThreads) out[tbase * K + f] = s_rec[f];
    if (tile == ntiles - 1 && threadIdx.x == 0) {
#pragma unroll
        for (int k = 0; k < K; ++k) out[n * K + k] = s_excl[k] + tot[k];
    }
}

// Takes a ticket (tiles in the order blocks start) and reads the epoch.
__device__ __forceinline__ int64_t scan_ticket(int32_t *ws, unsigned &epoch)
{
    __shared__ int64_t s_tile;
    unsigned *ctl = (unsigned *)ws;
    epoch = *(volatile unsigned *)(ctl + 2) & 0x3fffffffu;
    if (threadIdx.x == 0) s_tile = atomicAdd(ctl + 0, 1u);
    __syncthreads();
    return s_tile;
}

// The last block to finish resets the tickets and opens the next epoch.
__device__ __forceinline__ void scan_finish(int32_t *ws, unsigned epoch)
{
    if (threadIdx.x == 0) {
        unsigned *ctl = (unsigned *)ws;
        __threadfence();
        if (atomicAdd(ctl + 1, 1u) == gridDim.x - 1) {
            ctl[0] = 0;
            ctl[1] = 0;
            ctl[2] = (epoch + 1) & 0x3fffffffu;
            __threadfence();
        }
    }
}

template <int K, class In>
__global__ void __launch_bounds__(kThreads) scan_lookback_kernel(const In in, int32_t *__restrict__ out, int64_t n,
                                                                 const int32_t *__restrict__ n_dev, int32_t *ws,
                                                                 int32_t *err)
{
    if (n_dev) n = *n_dev;
    unsigned epoch;
    const int64_t tile = scan_ticket(ws, epoch);
    scan_tile<K>(in, out, n, tile, ws + kCtl, epoch, err);
    scan_finish(ws, epoch);
}

// Two independent scans in one launch: tickets below nb1 take tiles of the
// first, the rest tiles of the second (its status follows the first's).
template <int K1, class In1, int K2, class In2>
__global__ void __launch_bounds__(kThreads) scan_pair_kernel(const In1 in1, int32_t *__restrict__ out1, int64_t n1,
                                                             const int32_t *__restrict__ n1_dev, int64_t nb1,
                                                             const In2 in2, int32_t *__restrict__ out2, int64_t n2,
                                                             const int32_t *__restrict__ n2_dev, int32_t *ws,
                                                             int32_t *err)
{
    if (n1_dev) n1 = *n1_dev;
    if (n2_dev) n2 = *n2_dev;
    unsigned epoch;
    const int64_t ticket = scan_ticket(ws, epoch);
    if (ticket < nb1) scan_tile<K1>(in1, out1, n1, ticket, ws + kCtl, epoch, err);
    else scan_tile<K2>(in2, out2, n2, ticket - nb1, ws + kCtl + kStatus * nb1, epoch, err);
    scan_finish(ws, epoch);
}

// Give-up check of the look-back wait: one block scans tile 1 of a
// two-tile scan whose tile 0 never publishes (its status words are zero, so
// no flag ever matches).  The wait must stop after `spin_limit` polls, record
// KDGB_ERR_TIMEOUT in *err, count the missing tile as a zero prefix and
// finish the tile.  The status and output arrays are the caller's.
__global__ void __launch_bounds__(kThreads) k_scan_giveup(const int32_t *__restrict__ in, int32_t *out,
                                                           int32_t *status, int32_t *err, int spin_limit)
{
    ScanArray<1> a;
    a.in = in;
    scan_tile<1>(a, out, 2 * kTile, 1, status, 1u, err, spin_limit);
}

}  // namespace

int scan_giveup_check(int32_t spin_limit, int32_t *result, cudaStream_t s)
{
    if (spin_limit < 1) return fail(KDGB_ERR_INVALID_ARGUMENT, "scan give-up check: spin_limit must be >= 1");
    // in: 2 tiles of ones; out: 2 tiles + the totals record; status: 2 tiles;
    // err: one word.
    const int64_t n_in = 2 * kTile, n_out = 2 * kTile + 1, n_status = 2 * kStatus;
    int32_t *buf = nullptr;
    const int64_t words = n_in + n_out + n_status + 1;
    KDGB_CUDA(cudaMallocAsync((void **)&buf, sizeof(int32_t) * words, s));
    int32_t *in = buf, *out = in + n_in, *status = out + n_out, *err = status + n_status;
    std::vector<int32_t> ones(n_in, 1);
    cudaError_t e = cudaMemsetAsync(out, 0, sizeof(int32_t) * (n_out + n_status + 1), s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(in, ones.data(), sizeof(int32_t) * n_in, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) {
        k_scan_giveup<<<1, kThreads, 0, s>>>(in, out, status, err, spin_limit);
        note_launch();
        e = cudaGetLastError();
    }
    int32_t host[2] = {0, 0};
    if (e == cudaSuccess) e = cudaMemcpyAsync(&host[0], err, sizeof(int32_t), cudaMemcpyDeviceToHost, s);
    // The tile's first output: the exclusive prefix it assumed for tile 0.
    if (e == cudaSuccess) e = cudaMemcpyAsync(&host[1], out + kTile, sizeof(int32_t), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    cudaFreeAsync(buf, s);
    if (e != cudaSuccess) return cuda_fail(e, "scan give-up check");
    result[0] = host[0];
    result[1] = host[1];
    return KDGB_OK;
}

int64_t scan_partials_needed(int K, int64_t n)
{
    (void)K;
    return kCtl + kStatus * ((n + kTile - 1) / kTile);
}

template <int K, class In>
int scan_exclusive_in(const In &in, int32_t *out, int64_t n, cudaStream_t s, DevArray<int32_t> *ws,
                      const int32_t *n_dev, int32_t *err)
{
    static_assert(K <= 7, "a tile status holds K lanes twice and a flag");
    if (n < 0) return fail(KDGB_ERR_INVALID_ARGUMENT, "scan: negative length");
    if (!ws) return fail(KDGB_ERR_INVALID_ARGUMENT, "scan: no workspace");
    const int64_t need = scan_partials_needed(K, n);
    if (!ws->p || need > ws->cap) {
        // New state is zeroed (no flag matches any epoch); the control words
        // carry over.  Grows geometrically.
        const int64_t want = std::max<int64_t>(need, ws->cap + ws->cap / 2);
        KDGB_CHECK(ensure(*ws, want, s, ws->p ? kCtl : 0, true));
    }
    const int64_t nb = std::max<int64_t>(1, (n + kTile - 1) / kTile);
    KDGB_KERNEL((scan_lookback_kernel<K, In>), (unsigned)nb, kThreads, 0, s, in, out, n, n_dev, ws->p, err);
    return KDGB_OK;
}

template <int K1, class In1, int K2, class In2>
int scan_exclusive_pair(const In1 &in1, int32_t *out1, int64_t n1, const int32_t *n1_dev, const In2 &in2,
                        int32_t *out2, int64_t n2, const int32_t *n2_dev, cudaStream_t s, DevArray<int32_t> *ws,
                        int32_t *err)
{
    static_assert(K1 <= 7 && K2 <= 7, "a tile status holds K lanes twice and a flag");
    if (n1 < 0 || n2 < 0) return fail(KDGB_ERR_INVALID_ARGUMENT, "scan: negative length");
    if (!ws) return fail(KDGB_ERR_INVALID_ARGUMENT, "scan: no workspace");
    const int64_t nb1 = std::max<int64_t>(1, (n1 + kTile - 1) / kTile);
    const int64_t nb2 = std::max<int64_t>(1, (n2 + kTile - 1) / kTile);
    const int64_t need = kCtl + kStatus * (nb1 + nb2);
    if (!ws->p || need > ws->cap) {
        const int64_t want = std::max<int64_t>(need, ws->cap + ws->cap / 2);
        KDGB_CHECK(ensure(*ws, want, s, ws->p ? kCtl : 0, true));
    }
    KDGB_KERNEL((scan_pair_kernel<K1, In1, K2, In2>), (unsigned)(nb1 + nb2), kThreads, 0, s, in1, out1, n1, n1_dev, nb1, in2,
                                                                                 out2, n2, n2_dev, ws->p, err);
    return KDGB_OK;
}

int64_t scan_pair_needed(int64_t n1, int64_t n2)
{
    return kCtl + kStatus * (std::max<int64_t>(1, (n1 + kTile - 1) / kTile) +
                             std::max<int64_t>(1, (n2 + kTile - 1) / kTile));
}

template int scan_exclusive_pair<2, ScanArray<2>, 7, NodeLanes>(const ScanArray<2> &, int32_t *, int64_t,
                                                               const int32_t *, const NodeLanes &, int32_t *,
                                                               int64_t, const int32_t *, cudaStream_t,
                                                               DevArray<int32_t> *, int32_t *);

template int scan_exclusive_in<1, ScanArray<1>>(const ScanArray<1> &, int32_t *, int64_t, cudaStream_t,
                                             DevArray<int32_t> *, const int32_t *, int32_t *);
template int scan_exclusive_in<2, ScanArray<2>>(const ScanArray<2> &, int32_t *, int64_t, cudaStream_t,
                                             DevArray<int32_t> *, const int32_t *, int32_t *);
template int scan_exclusive_in<7, ScanArray<7>>(const ScanArray<7> &, int32_t *, int64_t, cudaStream_t,
                                             DevArray<int32_t> *, const int32_t *, int32_t *);
template int scan_exclusive_in<2, PackLanes>(const PackLanes &, int32_t *, int64_t, cudaStream_t, DevArray<int32_t> *,
                                          const int32_t *, int32_t *);
template int scan_exclusive_in<7, NodeLanes>(const NodeLanes &, int32_t *, int64_t, cudaStream_t, DevArray<int32_t> *,
                                          const int32_t *, int32_t *);

}  // namespace kdgb
