// Test helper: the library's Philox4x32-10 block (csrc/kdgb_photon.cuh)
// next to cuRAND's, on the same counters and keys.
#include <curand_kernel.h>

#include "kdgb_photon.cuh"

__global__ void k_compare(uint4 *ours, uint4 *theirs, int n)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint4 c = make_uint4(2654435761u * (unsigned)i, (unsigned)i, (unsigned)i ^ 0xdeadbeefu, 7u);
    const uint2 k = make_uint2(0x12345678u + (unsigned)i, 0x9abcdef0u);
    ours[i] = kdgb::philox4x32_10(c, k);
    theirs[i] = curand_Philox4x32_10(c, k);
}

extern "C" int philox_compare(unsigned *h_ours, unsigned *h_theirs, int n)
{
    uint4 *a = nullptr, *b = nullptr;
    if (cudaMalloc(&a, sizeof(uint4) * n) != cudaSuccess) return 1;
    if (cudaMalloc(&b, sizeof(uint4) * n) != cudaSuccess) return 1;
    k_compare<<<(n + 127) / 128, 128>>>(a, b, n);
    if (cudaDeviceSynchronize() != cudaSuccess) return 2;
    cudaMemcpy(h_ours, a, sizeof(uint4) * n, cudaMemcpyDeviceToHost);
    cudaMemcpy(h_theirs, b, sizeof(uint4) * n, cudaMemcpyDeviceToHost);
    cudaFree(a);
    cudaFree(b);
    return 0;
}
