// Precision form of the correlation core on the tensor cores.  The 2-D
// correlation's forward row DFT, forward column DFT and the inverse column
// DFT of the conjugate product (do_freq_xcorr.cu:90-117: cufftExecC2C forward
// on both patches, d_mulaconjb, inverse) run as split-FP16 GEMMs on tcgen05
// (tc_gemm.cuh) against DFT matrices embedded as real 2x2 blocks:
//
//   k_tc_rows  zrow[w][r][x]  -> zrow[w][r][kx]    A = row DFT (2N x 2N),  B = packed rows
//   k_tc_cols  zrow[w][r][kx] -> zrow[w][ky][kx]   A = column DFT (2M x 2M), B = columns
//   k_tc_inv   product of the two patches' spectra (Hermitian split, mean
//              correction, (-1)^(kx+ky), as k_cols forms it) -> qspec rows of
//              the surface band            A = inverse DFT rows (2 nyc x 2M)
//
// Operands are scaled by powers of two into the FP16 range before the hi/lo
// split and scaled back in the epilogues (exact), so every buffer between the
// stages holds the same quantity as in the FP32 path.  The range
// interpolation (k_rows) and the inverse row transform with the peak search
// (k_peak) stay FP32.
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include <cmath>
#include <vector>

#include "tc_gemm.cuh"
#include "team_fft.cuh"
#include "xcorr_ctx.cuh"
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
__global__ void __launch_bounds__(256) k_tc_gemm_check(const uint8_t *__restrict__ a_prep, int K,
                                                        const float *__restrict__ B, int Ntot, float bscale,
                                                        float cscale, float *__restrict__ C, int *err) {
    const int n0 = blockIdx.x * NT;
    auto load = [&](int k, int n) {
        return make_float2(B[(size_t)k * Ntot + n0 + n], B[(size_t)(k + 1) * Ntot + n0 + n]);
    };
    auto cvt = [&](float2 v, int, int) { return make_float2(v.x * bscale, v.y * bscale); };
    auto epi = [&](int m, int c0, const float *v) {
#pragma unroll
        for (int i = 0; i < 16; i++) C[(size_t)m * Ntot + n0 + c0 + i] = v[i] * cscale;
    };
    tc::gemm_block_ws<MT, NT, 4, false>(a_prep, K, load, cvt, epi, err);
}

template <int MT, int NT, int KC>
xcg_status run_check(int K, int Ntot, const float *A, const float *B, float *C, cudaStream_t s) {
    using G = tc::WsGeom<MT, NT, 4>;
    static_assert(KC == G::KC, "chunk width");
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
        k_tc_gemm_check<MT, NT, KC><<<Ntot / NT, 256, G::SMEM, s>>>(prep, K, B, Ntot, 1.0f, 1.0f, C, err);
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

constexpr float S_ROW = 1.0f / 16.0f;      // packed amplitudes (< 2^17) into the FP16 range
constexpr float S_COL = 1.0f / 1024.0f;    // row spectra (< 2^8 * 2^17)

// per-window bound of the column spectra, kept in the (not yet written)
// first surface element of the window until k_peak runs
__device__ __forceinline__ unsigned *ymax_slot(const Plan &P, int w) {
    return reinterpret_cast<unsigned *>(P.surf + (size_t)w * P.nyc * P.nxc);
}

// warps per CTA of the precision-form stages: the MMA issuer, the A
// producer and the rest producing the data operand.  The forward stages
// convert plain loads (8 warps measured best); the inverse stage forms the
// conjugate product from two spectrum reads per element first, and more
// producer warps keep more of those loads in flight (16 warps: 0.48 -> 0.38
// ms per 1000 windows).
constexpr int TC_WARPS = 8;
constexpr int TC_THREADS = 32 * TC_WARPS;
constexpr int TC_WARPS_INV = 16;
constexpr int TC_THREADS_INV = 32 * TC_WARPS_INV;
// forward stages (512 accumulator columns): 16-wide K chunks, 4 stages (160 KB);
// the inverse (up to 288 columns, fewer MMAs per chunk): 32-wide chunks, 4 stages
constexpr int TC_STAGES = 4;
constexpr int TC_KC = 16;
constexpr int TC_STAGES_INV = 4;
constexpr int TC_KC_INV = 32;

// Epilogue transpose: the warp holds a 32 (lanes = rows m) x 16 (columns)
// block; rows m = 2j + c are the re/im parts of 16 complex outputs j.  It is
// passed through the (then idle) stage memory so that each store instruction
// writes one output j's 16 complex values: out(j, col) receives c = 0/1 for
// lane pairs, col = lane / 2.
template <class Out>
__device__ __forceinline__ void warp_store_t(const float *v, Out out) {
    extern __shared__ __align__(1024) uint8_t tc_smem[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    float *sc = reinterpret_cast<float *>(tc_smem) + warp * (32 * 17);
#pragma unroll
    for (int i = 0; i < 16; i++) sc[lane * 17 + i] = v[i];
    __syncwarp();
#pragma unroll 4
    for (int j = 0; j < 16; j++) out(j, lane >> 1, lane & 1, sc[(2 * j + (lane & 1)) * 17 + (lane >> 1)]);
    __syncwarp();
}

template <int N>
__global__ void __launch_bounds__(TC_THREADS, 1) k_tc_rows(Plan P) {
    const int w = blockIdx.y, r0 = blockIdx.x * 128;
    float2 *z = P.zrow + (size_t)w * P.npy * N;
    if (blockIdx.x == 0 && threadIdx.x == 0) *ymax_slot(P, w) = 0u;
    auto load = [&](int k, int n) { return z[(size_t)(r0 + n) * N + (k >> 1)]; };
    auto cvt = [&](float2 v, int, int) { return make_float2(v.x * S_ROW, v.y * S_ROW); };
    auto epi = [&](int m, int n0, const float *v) {
        float *base = reinterpret_cast<float *>(z) + (m & 1);
        const int kx = m >> 1;
#pragma unroll
        for (int i = 0; i < 16; i++) base[((size_t)(r0 + n0 + i) * N + kx) * 2] = v[i] * (1.0f / S_ROW);
    };
    tc::gemm_block_ws<2 * N / 128, 128, TC_STAGES, true, TC_KC, TC_WARPS>(P.tc_a_row, 2 * N, load, cvt, epi, P.tc_err);
}

template <int M>
__global__ void __launch_bounds__(TC_THREADS, 1) k_tc_cols(Plan P) {
    const int N = P.npx;
    const int w = blockIdx.y, kx0 = blockIdx.x * 128;
    float2 *z = P.zrow + (size_t)w * M * N;
    float ymax = 0.f;
    auto load = [&](int k, int n) { return z[(size_t)(k >> 1) * N + kx0 + n]; };
    auto cvt = [&](float2 v, int, int) { return make_float2(v.x * S_COL, v.y * S_COL); };
    auto epi = [&](int m, int n0, const float *v) {
        const int ky0 = (m & ~31) >> 1;          // the warp's 16 rows ky0 .. ky0+15
        float *zf = reinterpret_cast<float *>(z);
        warp_store_t(v, [&](int j, int col, int c, float x) {
            const float o = x * (1.0f / S_COL);
            zf[((size_t)(ky0 + j) * N + kx0 + n0 + col) * 2 + c] = o;
            ymax = fmaxf(ymax, fabsf(o));
        });
    };
    tc::gemm_block_ws<2 * M / 128, 128, TC_STAGES, false, TC_KC, TC_WARPS>(P.tc_a_col, 2 * M, load, cvt, epi, P.tc_err);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) ymax = fmaxf(ymax, __shfl_xor_sync(0xffffffffu, ymax, o));
    if ((threadIdx.x & 31) == 0) atomicMax(ymax_slot(P, w), __float_as_uint(ymax));
}

// shapes of the three stages for square n x n transforms (n = 128 or 256)
template <int n>
struct TcShapes {
    static constexpr int MT_FWD = 2 * n / 128;                   // 128-row tiles of the 2n real outputs
    static constexpr int MT_INV = n / 128;                       // 2 nyc = n real outputs of the band
    static constexpr int NT_INV = ((n / 2 + 1 + 15) / 16) * 16;  // kx in [0, n/2], padded to 16
};

template <int M>
__global__ void __launch_bounds__(TC_THREADS_INV, 1) k_tc_inv(Plan P) {
    const int N = P.npx;
    const int w = blockIdx.x;
    const float2 *z = P.zrow + (size_t)w * M * N;
    __shared__ double msh[2];
    __shared__ float ssh;
    if (threadIdx.x < 32) {      // patch means (:719-724), as k_cols forms them
        const int l32 = threadIdx.x;
        const float *pb = P.part + (size_t)w * 2 * P.nchunks;
        double s1 = 0.0, s2 = 0.0;
        for (int i = l32; i < P.nchunks; i += 32) { s1 += (double)pb[i]; s2 += (double)pb[P.nchunks + i]; }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            s1 += __shfl_xor_sync(0xffffffffu, s1, o);
            s2 += __shfl_xor_sync(0xffffffffu, s2, o);
        }
        if (l32 == 0) {
            // / (N M), a power of two: exact scaling instead of an FP64 division
            const double inv = __longlong_as_double((long long)(1023 - (31 - __clz(N * M))) << 52);
            s1 *= inv;
            s2 *= inv;
            msh[0] = s1; msh[1] = s2;
            P.means[2 * w] = s1; P.means[2 * w + 1] = s2;
            // |A1|, |A2| <= 2 |Y|max after the mean corrections: |product| < (2 sqrt2 ymax)^2
            const float yb = 2.0f * 1.41421356f * __uint_as_float(*ymax_slot(P, w));
            int e = 0;
            frexpf(yb, &e);                        // yb < 2^e
            ssh = ldexpf(1.0f, 13 - 2 * e);        // product * ssh < 2^13
        }
    }
    __syncthreads();
    const float dc1 = (float)(msh[0] * (double)N * (double)M);
    const float m2 = (float)msh[1];
    const float su = ssh;
    auto load = [&](int k, int n) {
        const int ky = k >> 1;
        float4 r = make_float4(0.f, 0.f, 0.f, 0.f);
        if (n <= N / 2) {
            const float2 z1 = z[(size_t)ky * N + n];
            const float2 z2 = z[(size_t)((M - ky) & (M - 1)) * N + ((N - n) & (N - 1))];
            r = make_float4(z1.x, z1.y, z2.x, z2.y);
        }
        return r;
    };
    auto cvt = [&](float4 r, int k, int n) {
        if (n > N / 2) return make_float2(0.f, 0.f);
        const int ky = k >> 1;
        const float2 z1 = make_float2(r.x, r.y), z2 = make_float2(r.z, r.w);
        // A1 = (z1 + conj z2)/2, A2 = (z1 - conj z2)/(2i)
        float2 A1 = make_float2(0.5f * (z1.x + z2.x), 0.5f * (z1.y - z2.y));
        float2 A2 = make_float2(0.5f * (z1.y + z2.y), -0.5f * (z1.x - z2.x));
        if (n == 0 && ky == 0) A1.x -= dc1;
        const float2 bm = cmulf(__ldg(P.box_x + n), __ldg(P.box_y + ky));
        A2.x -= m2 * bm.x;
        A2.y -= m2 * bm.y;
        float2 pr = cmulf_conj(A1, A2);
        if ((n + ky) & 1) { pr.x = -pr.x; pr.y = -pr.y; }
        return make_float2(pr.x * su, pr.y * su);
    };
    auto epi = [&](int m, int n0, const float *v) {
        const int yq0 = (m & ~31) >> 1;          // the warp's 16 surface rows
        float *q = reinterpret_cast<float *>(P.qspec + (size_t)w * P.nyc * P.qpitch);
        warp_store_t(v, [&](int j, int col, int c, float x) {
            if (n0 + col <= N / 2) q[((size_t)(yq0 + j) * P.qpitch + n0 + col) * 2 + c] = x / su;
        });
    };
    tc::gemm_block_ws<TcShapes<M>::MT_INV, TcShapes<M>::NT_INV, TC_STAGES_INV, false, TC_KC_INV, TC_WARPS_INV>(
        P.tc_a_inv, 2 * M, load, cvt, epi, P.tc_err);
}

// Real 2x2-block embedding of rows [row0, row0 + nrows) of an n-point DFT
// matrix (sign -1 forward, +1 inverse): out[2r + c][2k + c'] with
// (c, c') = (re, re) cos, (re, im) -sin*sign', (im, re) sin*sign', (im, im) cos.
std::vector<float> dft_blocks(int n, int row0, int nrows, int sign) {
    std::vector<float> a((size_t)2 * nrows * 2 * n);
    for (int r = 0; r < nrows; r++)
        for (int k = 0; k < n; k++) {
            const long long ph = ((long long)(row0 + r) * k) % n;
            const double th = 2.0 * M_PI * (double)ph / (double)n;
            const double c = std::cos(th), sn = sign * std::sin(th);   // w = c + i sn
            float *row_re = &a[(size_t)(2 * r) * 2 * n], *row_im = &a[(size_t)(2 * r + 1) * 2 * n];
            row_re[2 * k] = (float)c;   row_re[2 * k + 1] = (float)-sn;
            row_im[2 * k] = (float)sn;  row_im[2 * k + 1] = (float)c;
        }
    return a;
}

}  // namespace

// Prepares the three DFT operands for an n x n geometry (n = 128, 256) and
// switches the context's plan to the precision form.
template <int n>
static xcg_status tc_enable_t(xcg_ctx *c) {
    using S = TcShapes<n>;
    Plan &B = c->base;
    const std::vector<float> ar = dft_blocks(n, 0, n, -1), ai = dft_blocks(n, B.ysearch, B.nyc, +1);
    const size_t br = tc::ws_prepared_bytes<S::MT_FWD, 128, TC_STAGES>(2 * n),
                 bi = tc::ws_prepared_bytes<S::MT_INV, S::NT_INV, TC_STAGES_INV, TC_KC_INV>(2 * n);
    uint8_t *prep = nullptr;
    float *tmp = nullptr;
    int *err = nullptr;
    cudaError_t e = cudaMalloc(&prep, 2 * br + bi);
    if (e == cudaSuccess) e = cudaMalloc(&tmp, ar.size() * sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc(&err, sizeof(int));
    if (e == cudaSuccess) e = cudaMemset(err, 0, sizeof(int));
    // rows and columns use the same forward operand (square transforms)
    if (e == cudaSuccess) e = cudaMemcpy(tmp, ar.data(), ar.size() * sizeof(float), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) { k_tc_prepare<S::MT_FWD, 128, TC_KC><<<256, 256>>>(tmp, 2 * n, 1.0f, prep); e = cudaDeviceSynchronize(); }
    if (e == cudaSuccess) e = cudaMemcpy(prep + br, prep, br, cudaMemcpyDeviceToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(tmp, ai.data(), ai.size() * sizeof(float), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) {
        k_tc_prepare<S::MT_INV, S::NT_INV, TC_KC_INV><<<256, 256>>>(tmp, 2 * n, 1.0f, prep + 2 * br);
        e = cudaDeviceSynchronize();
    }
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_tc_rows<n>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)tc::WsGeom<S::MT_FWD, 128, TC_STAGES>::SMEM);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_tc_cols<n>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)tc::WsGeom<S::MT_FWD, 128, TC_STAGES>::SMEM);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_tc_inv<n>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)tc::WsGeom<S::MT_INV, S::NT_INV, TC_STAGES_INV, TC_KC_INV>::SMEM);
    cudaFree(tmp);
    if (e != cudaSuccess) {
        cudaFree(prep);
        cudaFree(err);
        set_last_error(cudaGetErrorString(e));
        return XCG_ERR_CUDA;
    }
    c->tc_prep = prep;
    c->tc_err = err;
    B.tc_a_row = prep;
    B.tc_a_col = prep + br;
    B.tc_a_inv = prep + 2 * br;
    B.tc_err = err;
    B.tc_form = 1;
    return XCG_OK;
}

xcg_status tc_reset_status(xcg_ctx *c, cudaStream_t s) {
    if (!c->base.tc_form || !c->tc_err) return XCG_OK;
    // 0xff bytes: a nonzero flag, as a stage whose wait ran out leaves it
    const int v = c->inject_tc_timeout ? 0xff : 0;
    c->inject_tc_timeout = 0;
    const cudaError_t e = cudaMemsetAsync(c->tc_err, v, sizeof(int), s);
    if (e != cudaSuccess) {
        set_last_error(cudaGetErrorString(e));
        return XCG_ERR_CUDA;
    }
    return XCG_OK;
}

xcg_status tc_enable(xcg_ctx *c) {
    Plan &B = c->base;
    if (B.npx != B.npy || (B.npx != 256 && B.npx != 128)) {
        set_last_error("the precision form needs square windows of 64 or 128 (128- or 256-point transforms)");
        return XCG_ERR_UNSUPPORTED;
    }
    if (B.corr_mode != 2) {
        set_last_error("the precision form applies to the frequency-domain mode");
        return XCG_ERR_UNSUPPORTED;
    }
    if (B.tc_a_row) { B.tc_form = 1; return XCG_OK; }
    return B.npx == 256 ? tc_enable_t<256>(c) : tc_enable_t<128>(c);
}

template <int n>
static void launch_tc_t(const Plan &P, int stage, cudaStream_t s) {
    using S = TcShapes<n>;
    if (stage == 0)
        k_tc_rows<n><<<dim3(n / 128, P.nwin), TC_THREADS, tc::WsGeom<S::MT_FWD, 128, TC_STAGES>::SMEM, s>>>(P);
    else if (stage == 1)
        k_tc_cols<n><<<dim3(n / 128, P.nwin), TC_THREADS, tc::WsGeom<S::MT_FWD, 128, TC_STAGES>::SMEM, s>>>(P);
    else
        k_tc_inv<n><<<P.nwin, TC_THREADS_INV, tc::WsGeom<S::MT_INV, S::NT_INV, TC_STAGES_INV, TC_KC_INV>::SMEM, s>>>(P);
}
void launch_tc_rows(const Plan &P, cudaStream_t s) { P.npx == 256 ? launch_tc_t<256>(P, 0, s) : launch_tc_t<128>(P, 0, s); }
void launch_tc_cols(const Plan &P, cudaStream_t s) { P.npx == 256 ? launch_tc_t<256>(P, 1, s) : launch_tc_t<128>(P, 1, s); }
void launch_tc_inv(const Plan &P, cudaStream_t s) { P.npx == 256 ? launch_tc_t<256>(P, 2, s) : launch_tc_t<128>(P, 2, s); }

}  // namespace xcg

extern "C" xcg_status xcg_set_dft_form(xcg_ctx *c, int32_t form) {
    if (!c || form < 0 || form > 1) return XCG_ERR_ARG;
    if (cudaSetDevice(c->device) != cudaSuccess) return XCG_ERR_CUDA;
    if (form == 0) { c->base.tc_form = 0; return XCG_OK; }
    return xcg::tc_enable(c);
}

extern "C" void xcg_debug_inject_stage_timeout(xcg_ctx *c) {
    if (c) c->inject_tc_timeout = 1;
}

extern "C" xcg_status xcg_tc_gemm_check(int32_t m_tiles, int32_t n_tile, int32_t k, int32_t n_total,
                                        const float *d_a, const float *d_b, float *d_c, void *stream) {
    if (!d_a || !d_b || !d_c || k <= 0 || n_total <= 0) return XCG_ERR_ARG;
    cudaStream_t s = (cudaStream_t)stream;
    if (m_tiles == 4 && n_tile == 128) return xcg::run_check<4, 128, 16>(k, n_total, d_a, d_b, d_c, s);
    if (m_tiles == 2 && n_tile == 144) return xcg::run_check<2, 144, 16>(k, n_total, d_a, d_b, d_c, s);
    if (m_tiles == 1 && n_tile == 256) return xcg::run_check<1, 256, 16>(k, n_total, d_a, d_b, d_c, s);
    xcg::set_last_error("xcg_tc_gemm_check: shapes (4,128), (2,144), (1,256) only");
    return XCG_ERR_UNSUPPORTED;
}
