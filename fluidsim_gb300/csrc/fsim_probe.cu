// fsim_probe.cu — measurement utility: the FP32 FMA throughput of the device,
// the denominator of the particle sweep's compute roofline (the sweep is a
// gather bound by FP32/ALU issue, not by HBM).  No counterpart in the
// reference.
#include "fsim_internal.h"

#include <cuda_runtime.h>

namespace {

constexpr int kChains = 8;   // independent FMA chains per thread (hides the FMA latency)
constexpr int kThreads = 256;

__global__ void __launch_bounds__(kThreads) k_fma_peak(float *__restrict__ out, float b, float c, int iters)
{
    float a[kChains];
#pragma unroll
    for (int k = 0; k < kChains; ++k) a[k] = (float)(threadIdx.x + k) * 1e-3f;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int u = 0; u < 16; ++u)
#pragma unroll
            for (int k = 0; k < kChains; ++k) a[k] = fmaf(a[k], b, c);
    }
    float s = 0.0f;
#pragma unroll
    for (int k = 0; k < kChains; ++k) s += a[k];
    out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

} // namespace

extern "C" fsim_status fsim_measure_fp32_peak(int device, double *tflops)
{
    if (!tflops) return FSIM_EINVAL;
    *tflops = 0.0;
    int prev = -1;
    cudaGetDevice(&prev);
    if (cudaSetDevice(device) != cudaSuccess) {
        cudaGetLastError();
        fsim_set_error("no CUDA device %d", device);
        return FSIM_ECUDA;
    }
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    const int blocks = sms * 8; // 8 x 256 threads = 64 warps per SM, the residency limit
    const int iters = 4096;
    float *out = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    cudaError_t e = cudaMalloc((void **)&out, sizeof(float) * blocks * kThreads);
    if (e == cudaSuccess) e = cudaEventCreate(&e0);
    if (e == cudaSuccess) e = cudaEventCreate(&e1);
    float best_ms = 0.0f;
    for (int rep = 0; rep < 4 && e == cudaSuccess; ++rep) { // first launch is a warm-up
        cudaEventRecord(e0);
        k_fma_peak<<<blocks, kThreads>>>(out, 0.999999f, 1e-7f, iters);
        cudaEventRecord(e1);
        e = cudaEventSynchronize(e1);
        float ms = 0.0f;
        if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
        if (rep > 0 && (best_ms == 0.0f || ms < best_ms)) best_ms = ms;
    }
    if (e == cudaSuccess) e = cudaGetLastError();
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (out) cudaFree(out);
    if (prev >= 0) cudaSetDevice(prev);
    if (e != cudaSuccess || best_ms <= 0.0f) {
        fsim_set_error("FP32 peak measurement failed: %s", cudaGetErrorString(e));
        return FSIM_ECUDA;
    }
    const double flops = 2.0 * 16.0 * kChains * (double)iters * blocks * kThreads;
    *tflops = flops / (best_ms * 1e-3) / 1e12;
    return FSIM_OK;
}
