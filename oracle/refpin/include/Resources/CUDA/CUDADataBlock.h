// Stand-in for OpenEngine's CUDADataBlock (only declared by the pinned
// headers).  TEST INFRASTRUCTURE ONLY.
#pragma once
namespace OpenEngine {
namespace Resources {
namespace CUDA {
template <class T>
class CUDADataBlock {
public:
    T *GetDeviceData();
};
}  // namespace CUDA
}  // namespace Resources
}  // namespace OpenEngine
