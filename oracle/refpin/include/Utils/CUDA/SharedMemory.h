// Stand-in for extensions-CUDA's SharedMemory<T>() (dynamic shared memory):
// a static host buffer per type, large enough for one block of the pinned
// kernels.  TEST INFRASTRUCTURE ONLY.
#pragma once
template <class T>
inline T *SharedMemory()
{
    static T buf[1 << 14];
    return buf;
}
