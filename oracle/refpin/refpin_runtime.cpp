// Host stand-in for the CUDA runtime under the tracer pin units, which are
// built with nvcc -cudart none.  TEST INFRASTRUCTURE ONLY.
//
// The reference's fetch helpers read through cudaMemcpy and
// cudaMemcpyFromSymbol on their host branch (Utils/CUDA/Utils.h:52-82); here
// those are plain host copies, so the traversal functions run on host arrays
// with no GPU and no driver.  The registration calls nvcc emits for each
// unit's kernels and __constant__ variables are accepted and ignored: no
// kernel is ever launched, and a launch would fail with
// cudaErrorNotSupported.  Signatures follow crt/host_runtime.h and
// crt/device_functions.h.
#include <cuda_runtime_api.h>

#include <cmath>
#include <cstring>

extern "C" {

cudaError_t CUDARTAPI cudaMemcpy(void *dst, const void *src, size_t count, enum cudaMemcpyKind)
{
    memmove(dst, src, count);
    return cudaSuccess;
}

cudaError_t CUDARTAPI cudaMemcpyToSymbol(const void *symbol, const void *src, size_t count, size_t offset,
                                         enum cudaMemcpyKind)
{
    memmove((char *)symbol + offset, src, count);
    return cudaSuccess;
}

cudaError_t CUDARTAPI cudaMemcpyFromSymbol(void *dst, const void *symbol, size_t count, size_t offset,
                                           enum cudaMemcpyKind)
{
    memmove(dst, (const char *)symbol + offset, count);
    return cudaSuccess;
}

cudaError_t CUDARTAPI cudaDeviceSynchronize(void) { return cudaSuccess; }

static void *kdgb_pin_module_handle = nullptr;

void **CUDARTAPI __cudaRegisterFatBinary(void *) { return &kdgb_pin_module_handle; }
void CUDARTAPI __cudaRegisterFatBinaryEnd(void **) {}
void CUDARTAPI __cudaUnregisterFatBinary(void **) {}
void CUDARTAPI __cudaRegisterVar(void **, char *, char *, const char *, int, size_t, int, int) {}
void CUDARTAPI __cudaRegisterFunction(void **, const char *, char *, const char *, int, uint3 *, uint3 *, dim3 *,
                                      dim3 *, int *)
{
}
char CUDARTAPI __cudaInitModule(void **) { return 0; }
unsigned CUDARTAPI __cudaPushCallConfiguration(dim3, dim3, size_t, struct CUstream_st *) { return 0; }
cudaError_t CUDARTAPI __cudaPopCallConfiguration(dim3 *, dim3 *, size_t *, void *) { return cudaErrorNotSupported; }
cudaError_t CUDARTAPI __cudaGetKernel(cudaKernel_t *, const void *) { return cudaErrorNotSupported; }
cudaError_t CUDARTAPI __cudaLaunchKernel(cudaKernel_t, dim3, dim3, void **, size_t, cudaStream_t)
{
    return cudaErrorNotSupported;
}

}  // extern "C"

// The specular power the tracer units' shading loop calls (declared in
// include_cu/Meta/CUDA.h): the C library's powf, or the function installed by
// ref_trace_set_pow.
namespace OpenEngine {
namespace Utils {
namespace CUDA {
static float (*kdgb_pin_pow)(float, float) = nullptr;
float powf(float x, float y) { return kdgb_pin_pow ? kdgb_pin_pow(x, y) : ::powf(x, y); }
}  // namespace CUDA
}  // namespace Utils
}  // namespace OpenEngine

extern "C" __attribute__((visibility("default"))) void ref_trace_set_pow(float (*fn)(float, float))
{
    OpenEngine::Utils::CUDA::kdgb_pin_pow = fn;
}
