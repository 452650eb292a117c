// The device a context is bound to (shared by the decompression and
// compression contexts).
#pragma once
#include <cuda_runtime.h>

namespace ozl {

// Makes `dev` the calling thread's current device for the scope and gives
// the caller's back after (a context keeps the device that was current when
// it was created; -1: the current one).
struct DeviceScope {
    int prev = -1;
    explicit DeviceScope(int dev)
    {
        int cur = 0;
        if (dev >= 0 && cudaGetDevice(&cur) == cudaSuccess && cur != dev && cudaSetDevice(dev) == cudaSuccess) prev = cur;
    }
    ~DeviceScope()
    {
        if (prev >= 0) cudaSetDevice(prev);
    }
    DeviceScope(const DeviceScope&) = delete;
    DeviceScope& operator=(const DeviceScope&) = delete;
};
inline int currentDevice()
{
    int d = -1;
    return cudaGetDevice(&d) == cudaSuccess ? d : -1;
}

} // namespace ozl
