// probe.cu -- measures this GPU's dense FP64 FMA throughput.
//
// The tracking kernel is bound by the FP64 pipe; the roofline it is reported
// against is this measured rate (not a datasheet number).  Each thread runs
// 8 independent FMA chains so the pipe, not latency, limits the rate; the
// grid covers every SM several times.
#include <cuda_runtime.h>

#include <cstdint>

#include "sixtracklib_gb300.h"
#include "device_guard.h"
#include "kernel_api.h"

namespace {

__global__ void fp64_fma_loop(double *out, int iters, double a, double b)
{
    double c0 = threadIdx.x * 1e-3, c1 = c0 + 1, c2 = c0 + 2, c3 = c0 + 3;
    double c4 = c0 + 4, c5 = c0 + 5, c6 = c0 + 6, c7 = c0 + 7;
    for (int i = 0; i < iters; ++i) {
        c0 = fma(c0, a, b);
        c1 = fma(c1, a, b);
        c2 = fma(c2, a, b);
        c3 = fma(c3, a, b);
        c4 = fma(c4, a, b);
        c5 = fma(c5, a, b);
        c6 = fma(c6, a, b);
        c7 = fma(c7, a, b);
    }
    double const s = ((c0 + c1) + (c2 + c3)) + ((c4 + c5) + (c6 + c7));
    if (s == 12345.678) out[blockIdx.x] = s;  // keeps the loop alive
}

}  // namespace

extern "C" double st_engine_measure_fp64_peak(int device)
{
    stg::DeviceGuard guard;  // the caller's current device is restored on return
    if (cudaSetDevice(device) != cudaSuccess) return -1.0;
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    double *d = nullptr;
    if (cudaMalloc(&d, 8 * 65536) != cudaSuccess) return -1.0;
    int const threads = 256, blocks = sms * 8, iters = 4096;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    fp64_fma_loop<<<blocks, threads>>>(d, iters, 0.999999, 1e-7);  // warm-up
    float best_ms = 1e30f;
    for (int rep = 0; rep < 5; ++rep) {
        cudaEventRecord(e0);
        fp64_fma_loop<<<blocks, threads>>>(d, iters, 0.999999, 1e-7);
        cudaEventRecord(e1);
        cudaEventSynchronize(e1);
        float ms = 0;
        cudaEventElapsedTime(&ms, e0, e1);
        if (ms < best_ms) best_ms = ms;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(d);
    if (cudaGetLastError() != cudaSuccess) return -1.0;
    double const flops = 2.0 * 8.0 * (double)iters * (double)threads * (double)blocks;
    return flops / (best_ms * 1e-3) / 1e12;  // TFLOP/s, FMA counted as 2
}

// The fast arithmetic policy's exponential on device arrays, for checking it
// against e^x.
extern "C" int32_t st_engine_exp_fast(const double *x, double *y, int64_t n, void *stream)
{
    return stg::launch_exp_fast(x, y, n, stream);
}

// The fast arithmetic policy's reciprocal on device arrays, for checking it
// against 1 / x.
extern "C" int32_t st_engine_rcp_fast(const double *x, double *y, int64_t n, void *stream)
{
    return stg::launch_rcp_fast(x, y, n, stream);
}
