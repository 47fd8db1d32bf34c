// device_guard.h -- keep the caller's current CUDA device across a C-ABI call.
//
// The engine works on the device a lattice, job or option names and makes it
// current for the kernels and copies it issues.  A caller (a PyTorch program
// working on another GPU, say) must find its own current device unchanged
// when the call returns: a DeviceGuard at the top of an entry point records
// the current device and restores it on every return path, if the call
// changed it.
#pragma once

#include <cuda_runtime.h>

namespace stg {

class DeviceGuard {
public:
    DeviceGuard()
    {
        if (cudaGetDevice(&prev_) != cudaSuccess) prev_ = -1;
    }
    ~DeviceGuard()
    {
        int cur = -1;
        if (prev_ >= 0 && cudaGetDevice(&cur) == cudaSuccess && cur != prev_)
            cudaSetDevice(prev_);
    }
    DeviceGuard(const DeviceGuard &) = delete;
    DeviceGuard &operator=(const DeviceGuard &) = delete;

private:
    int prev_ = -1;
};

}  // namespace stg
