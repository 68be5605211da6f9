// SM partitions for pipelined frames: the device's SMs split into two green
// contexts, so that the rebuilds of the frames in flight run on one set of
// SMs and the traces on the other, instead of taking the whole device from
// each other kernel by kernel.
//
// A stream made by kdgb_sm_partition_stream runs its kernels on its
// partition's SMs only; kdgb_graph_create captures a rebuild graph in the
// context of the stream it is given, so that the graph's kernels keep to
// that partition wherever the graph is launched.  Memory, events and copies
// are shared with the primary context as usual.
//
// The driver functions are fetched through the runtime, so the library does
// not link the driver library itself.
#include <cuda.h>
#include <cuda_runtime.h>

#include <mutex>
#include <new>
#include <vector>

#include "kdgb_internal.cuh"

namespace kdgb {
namespace {

struct Driver {
    CUresult (*device_get)(CUdevice *, int) = nullptr;
    CUresult (*get_resource)(CUdevice, CUdevResource *, CUdevResourceType) = nullptr;
    CUresult (*split)(CUdevResource *, unsigned *, const CUdevResource *, CUdevResource *, unsigned, unsigned) = nullptr;
    CUresult (*gen_desc)(CUdevResourceDesc *, CUdevResource *, unsigned) = nullptr;
    CUresult (*green_create)(CUgreenCtx *, CUdevResourceDesc, CUdevice, unsigned) = nullptr;
    CUresult (*green_destroy)(CUgreenCtx) = nullptr;
    CUresult (*ctx_from_green)(CUcontext *, CUgreenCtx) = nullptr;
    CUresult (*ctx_push)(CUcontext) = nullptr;
    CUresult (*ctx_pop)(CUcontext *) = nullptr;
    CUresult (*ctx_current)(CUcontext *) = nullptr;
    CUresult (*ctx_resource)(CUcontext, CUdevResource *, CUdevResourceType) = nullptr;
    CUresult (*stream_ctx)(CUstream, CUcontext *) = nullptr;
    bool ok = false;
};

std::mutex g_driver_mu;
Driver g_driver;
bool g_driver_tried = false;

template <class F>
bool entry(const char *name, int version, F &fn)
{
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion(name, &p, version, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess || !p) {
        cudaGetLastError();
        return false;
    }
    fn = reinterpret_cast<F>(p);
    return true;
}

// The driver functions, or nullptr when this driver has no SM partitions.
const Driver *driver()
{
    std::lock_guard<std::mutex> lock(g_driver_mu);
    if (!g_driver_tried) {
        g_driver_tried = true;
        Driver d;
        d.ok = entry("cuDeviceGet", 12000, d.device_get) && entry("cuDeviceGetDevResource", 12040, d.get_resource) &&
               entry("cuDevSmResourceSplitByCount", 12040, d.split) &&
               entry("cuDevResourceGenerateDesc", 12040, d.gen_desc) &&
               entry("cuGreenCtxCreate", 12040, d.green_create) && entry("cuGreenCtxDestroy", 12040, d.green_destroy) &&
               entry("cuCtxFromGreenCtx", 12040, d.ctx_from_green) && entry("cuCtxPushCurrent", 12000, d.ctx_push) &&
               entry("cuCtxPopCurrent", 12000, d.ctx_pop) && entry("cuCtxGetCurrent", 12000, d.ctx_current) &&
               entry("cuCtxGetDevResource", 12040, d.ctx_resource) && entry("cuStreamGetCtx", 12000, d.stream_ctx);
        g_driver = d;
    }
    return g_driver.ok ? &g_driver : nullptr;
}

int drv_fail(CUresult r, const char *what)
{
    return fail(KDGB_ERR_CUDA, std::string(what) + " failed (CUresult " + std::to_string((int)r) + ")");
}

}  // namespace

int context_sm_count()
{
    const Driver *d = driver();
    if (!d) return 0;
    CUcontext ctx = nullptr;
    if (d->ctx_current(&ctx) != CUDA_SUCCESS || !ctx) return 0;
    CUdevResource r;
    if (d->ctx_resource(ctx, &r, CU_DEV_RESOURCE_TYPE_SM) != CUDA_SUCCESS) return 0;
    return (int)r.sm.smCount;
}

StreamContext::StreamContext(cudaStream_t s)
{
    const Driver *d = driver();
    if (!d) return;
    CUcontext want = nullptr, cur = nullptr;
    if (d->stream_ctx((CUstream)s, &want) != CUDA_SUCCESS || !want) return;
    if (d->ctx_current(&cur) != CUDA_SUCCESS || cur == want) return;
    pushed_ = d->ctx_push(want) == CUDA_SUCCESS;
}

StreamContext::~StreamContext()
{
    if (!pushed_) return;
    CUcontext popped = nullptr;
    driver()->ctx_pop(&popped);
}

}  // namespace kdgb

using namespace kdgb;

struct kdgb_sm_partition {
    CUgreenCtx green[2] = {nullptr, nullptr};
    CUcontext ctx[2] = {nullptr, nullptr};
    int32_t sms[2] = {0, 0};
    std::vector<cudaStream_t> streams;
};

extern "C" {

int kdgb_sm_partition_create(int32_t sms, kdgb_sm_partition **out)
{
    if (!out) return fail(KDGB_ERR_INVALID_ARGUMENT, "out is NULL");
    *out = nullptr;
    if (sms < 1) return fail(KDGB_ERR_INVALID_ARGUMENT, "an SM partition needs at least one SM");
    int ord = 0;
    KDGB_CUDA(cudaGetDevice(&ord));
    KDGB_CUDA(cudaFree(nullptr));  // the primary context exists
    const Driver *d = driver();
    if (!d) return fail(KDGB_ERR_UNSUPPORTED, "this driver has no SM partitions (green contexts)");
    CUdevice dev;
    CUresult r = d->device_get(&dev, ord);
    if (r != CUDA_SUCCESS) return drv_fail(r, "cuDeviceGet");
    CUdevResource all, first[1], rest;
    r = d->get_resource(dev, &all, CU_DEV_RESOURCE_TYPE_SM);
    if (r != CUDA_SUCCESS) return drv_fail(r, "cuDeviceGetDevResource");
    if ((unsigned)sms >= all.sm.smCount)
        return fail(KDGB_ERR_INVALID_ARGUMENT, "the first SM partition must leave SMs for the second");
    unsigned groups = 1;
    r = d->split(first, &groups, &all, &rest, 0, (unsigned)sms);
    if (r != CUDA_SUCCESS || groups != 1) return drv_fail(r, "cuDevSmResourceSplitByCount");
    if (rest.sm.smCount == 0) return fail(KDGB_ERR_INVALID_ARGUMENT, "no SMs left for the second partition");
    kdgb_sm_partition *p = new (std::nothrow) kdgb_sm_partition();
    if (!p) return fail(KDGB_ERR_OUT_OF_MEMORY, "host allocation");
    CUdevResource *res[2] = {&first[0], &rest};
    for (int i = 0; i < 2; ++i) {
        CUdevResourceDesc desc;
        r = d->gen_desc(&desc, res[i], 1);
        if (r == CUDA_SUCCESS) r = d->green_create(&p->green[i], desc, dev, CU_GREEN_CTX_DEFAULT_STREAM);
        if (r == CUDA_SUCCESS) r = d->ctx_from_green(&p->ctx[i], p->green[i]);
        if (r != CUDA_SUCCESS) {
            kdgb_sm_partition_destroy(p);
            return drv_fail(r, "green context creation");
        }
        p->sms[i] = (int32_t)res[i]->sm.smCount;
    }
    *out = p;
    return KDGB_OK;
}

int kdgb_sm_partition_sms(const kdgb_sm_partition *part, int32_t which, int32_t *sms)
{
    if (!part || !sms) return fail(KDGB_ERR_INVALID_ARGUMENT, "partition or sms is NULL");
    if (which != 0 && which != 1) return fail(KDGB_ERR_INVALID_ARGUMENT, "which must be 0 or 1");
    *sms = part->sms[which];
    return KDGB_OK;
}

int kdgb_sm_partition_stream(kdgb_sm_partition *part, int32_t which, int32_t priority, kdgb_stream_t *out)
{
    if (!part || !out) return fail(KDGB_ERR_INVALID_ARGUMENT, "partition or out is NULL");
    if (which != 0 && which != 1) return fail(KDGB_ERR_INVALID_ARGUMENT, "which must be 0 or 1");
    const Driver *d = driver();
    CUresult r = d->ctx_push(part->ctx[which]);
    if (r != CUDA_SUCCESS) return drv_fail(r, "cuCtxPushCurrent");
    cudaStream_t s = nullptr;
    const cudaError_t e = cudaStreamCreateWithPriority(&s, cudaStreamNonBlocking, priority);
    CUcontext popped = nullptr;
    d->ctx_pop(&popped);
    if (e != cudaSuccess) return cuda_fail(e, "partition stream");
    part->streams.push_back(s);
    *out = (kdgb_stream_t)s;
    return KDGB_OK;
}

int kdgb_sm_partition_destroy(kdgb_sm_partition *part)
{
    if (!part) return KDGB_OK;
    for (cudaStream_t s : part->streams) {
        cudaStreamSynchronize(s);
        cudaStreamDestroy(s);
    }
    const Driver *d = driver();
    for (int i = 0; i < 2; ++i)
        if (part->green[i] && d) d->green_destroy(part->green[i]);
    delete part;
    return KDGB_OK;
}

}  // extern "C"
