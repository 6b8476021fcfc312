// Precision form of the correlation core on the tensor cores: split-FP16
// GEMM engine checks (tc_gemm.cuh) exposed through a diagnostic C entry.
#include <cuda_runtime.h>
#include <stdint.h>

#include "tc_gemm.cuh"
#include "xcorr_gb300.h"

namespace xcg {
void set_last_error(const char *msg);

namespace {

// A (M x K, row-major FP32) -> prepared chunks (hi tile, lo tile per K chunk)
template <int MT, int NT, int KC>
__global__ void k_tc_prepare(const float *__restrict__ A, int K, float scale, uint8_t *__restrict__ out) {
    using G = tc::GemmGeom<MT, NT, KC>;
    const int M = MT * 128;
    const size_t n = (size_t)M * K;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const int m = (int)(i / K), k = (int)(i % K);
        const int c = k / KC, kk = k % KC;
        __half h, l;
        tc::split_f16(A[i] * scale, h, l);
        __half *hi = reinterpret_cast<__half *>(out + (size_t)c * 2 * G::A_TILE);
        __half *lo = reinterpret_cast<__half *>(out + (size_t)c * 2 * G::A_TILE + G::A_TILE);
        const uint32_t off = tc::kmajor_off(m, kk, G::SBO) >> 1;
        hi[off] = h;
        lo[off] = l;
    }
}

template <int MT, int NT, int KC>
__global__ void __launch_bounds__(128) k_tc_gemm_check(const uint8_t *__restrict__ a_prep, int K,
                                                        const float *__restrict__ B, int Ntot, float bscale,
                                                        float cscale, float *__restrict__ C, int *err) {
    const int n0 = blockIdx.x * NT;
    auto loadB = [&](int k, int n) { return B[(size_t)k * Ntot + n0 + n] * bscale; };
    auto epi = [&](int m, int c0, const float *v) {
#pragma unroll
        for (int i = 0; i < 16; i++) C[(size_t)m * Ntot + n0 + c0 + i] = v[i] * cscale;
    };
    tc::gemm_block<MT, NT, KC>(a_prep, K, loadB, epi, err);
}

template <int MT, int NT, int KC>
xcg_status run_check(int K, int Ntot, const float *A, const float *B, float *C, cudaStream_t s) {
    using G = tc::GemmGeom<MT, NT, KC>;
    if (K % KC || Ntot % NT) return XCG_ERR_ARG;
    uint8_t *prep = nullptr;
    int *err = nullptr;
    cudaError_t e = cudaMalloc(&prep, tc::prepared_bytes<MT, NT, KC>(K));
    if (e == cudaSuccess) e = cudaMalloc(&err, sizeof(int));
    if (e == cudaSuccess) e = cudaMemsetAsync(err, 0, sizeof(int), s);
    if (e == cudaSuccess) {
        // operands scaled by powers of two into the FP16 range (exact)
        k_tc_prepare<MT, NT, KC><<<256, 256, 0, s>>>(A, K, 1.0f, prep);
        e = cudaFuncSetAttribute(k_tc_gemm_check<MT, NT, KC>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)G::SMEM);
    }
    if (e == cudaSuccess) {
        k_tc_gemm_check<MT, NT, KC><<<Ntot / NT, 128, G::SMEM, s>>>(prep, K, B, Ntot, 1.0f, 1.0f, C, err);
        e = cudaGetLastError();
    }
    int herr = 0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&herr, err, sizeof(int), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    cudaFree(prep);
    cudaFree(err);
    if (e != cudaSuccess) { set_last_error(cudaGetErrorString(e)); return XCG_ERR_CUDA; }
    if (herr) { set_last_error("tensor-core GEMM: a wait ran out"); return XCG_ERR_CUDA; }
    return XCG_OK;
}

}  // namespace
}  // namespace xcg

extern "C" xcg_status xcg_tc_gemm_check(int32_t m_tiles, int32_t n_tile, int32_t k, int32_t n_total,
                                        const float *d_a, const float *d_b, float *d_c, void *stream) {
    if (!d_a || !d_b || !d_c || k <= 0 || n_total <= 0) return XCG_ERR_ARG;
    cudaStream_t s = (cudaStream_t)stream;
    if (m_tiles == 4 && n_tile == 128) return xcg::run_check<4, 128, 32>(k, n_total, d_a, d_b, d_c, s);
    if (m_tiles == 2 && n_tile == 144) return xcg::run_check<2, 144, 32>(k, n_total, d_a, d_b, d_c, s);
    if (m_tiles == 1 && n_tile == 256) return xcg::run_check<1, 256, 32>(k, n_total, d_a, d_b, d_c, s);
    xcg::set_last_error("xcg_tc_gemm_check: shapes (4,128), (2,144), (1,256) only");
    return XCG_ERR_UNSUPPORTED;
}
