// FP32 fused multiply-add throughput of the device, measured by a kernel of
// this library: the denominator of the FP32 SIMT roofline the benchmark
// reports for the FFT kernels (the measured peaks cover HBM and the
// bf16 tensor pipe only).  No counterpart in the reference.
#include <cuda_runtime.h>

#include "xcorr_gb300.h"
#include "xcorr_kernels.cuh"

namespace {

constexpr int kChains = 8;          // independent FMA chains per thread (covers the FMA latency)
constexpr int kThreads = 256;

// Every thread runs kChains dependent chains of x = x * a + b for iters
// steps; a and b are kernel arguments, so nothing folds at compile time, and
// the chains' sum is stored so nothing is dropped.
__global__ void __launch_bounds__(kThreads) k_fma_rate(float *out, int iters, float a, float b) {
    float x[kChains];
#pragma unroll
    for (int j = 0; j < kChains; j++) x[j] = (float)(threadIdx.x + j) * 1e-3f;
#pragma unroll 1
    for (int i = 0; i < iters; i++) {
#pragma unroll
        for (int u = 0; u < 16; u++)
#pragma unroll
            for (int j = 0; j < kChains; j++) x[j] = fmaf(x[j], a, b);
    }
    float s = 0.f;
#pragma unroll
    for (int j = 0; j < kChains; j++) s += x[j];
    out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

}  // namespace

extern "C" xcg_status xcg_fp32_fma_rate(int32_t device, double *tflops) {
    if (!tflops) return XCG_ERR_ARG;
    *tflops = 0.0;
    if (cudaSetDevice(device) != cudaSuccess) return XCG_ERR_NO_DEVICE;
    int sms = 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess || sms <= 0)
        return XCG_ERR_NO_DEVICE;
    const int blocks = sms * 8;           // 8 CTAs of 8 warps per SM: 16 warps per scheduler
    float *out = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    cudaStream_t s = nullptr;
    xcg_status st = XCG_OK;
    const int iters = 4096;               // 16 x 8 x 4096 FMAs per thread, tens of milliseconds
    float best = 1e30f;
    if (cudaMalloc(&out, (size_t)blocks * kThreads * sizeof(float)) != cudaSuccess) return XCG_ERR_NOMEM;
    if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess || cudaEventCreate(&e0) != cudaSuccess ||
        cudaEventCreate(&e1) != cudaSuccess) {
        st = XCG_ERR_CUDA;
    } else {
        for (int rep = 0; rep < 6 && st == XCG_OK; rep++) {      // first launch warms up; best of the rest
            cudaEventRecord(e0, s);
            k_fma_rate<<<blocks, kThreads, 0, s>>>(out, iters, 0.999f, 1e-4f);
            cudaEventRecord(e1, s);
            if (cudaEventSynchronize(e1) != cudaSuccess) { st = XCG_ERR_CUDA; break; }
            float ms = 0.f;
            cudaEventElapsedTime(&ms, e0, e1);
            if (rep > 0 && ms < best) best = ms;
        }
    }
    if (st == XCG_OK && cudaGetLastError() != cudaSuccess) st = XCG_ERR_CUDA;
    if (st == XCG_OK) {
        const double flops = 2.0 * 16.0 * kChains * (double)iters * (double)blocks * kThreads;
        *tflops = flops / (best * 1e-3) / 1e12;
    } else {
        xcg::set_last_error("FMA-rate probe: a CUDA call failed");
    }
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (s) cudaStreamDestroy(s);
    cudaFree(out);
    return st;
}
