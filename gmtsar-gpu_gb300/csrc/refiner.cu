// Subpixel refiner: a small CNN that reads the normalised 9x9 correlation
// surface around the integer peak and predicts the subpixel peak position
// (fx, fy, in surface pixels, the quantities highres_corr returns as
// xfrac/yfrac, highres_corr.cu:67-76) and the log variance s of that
// estimate.  No counterpart in the reference; it stands in for the FFT
// zero-pad interpolation where it is confident.
//
// Network (valid 3x3 convolutions, GELU): 9x9 -> 32@7x7 -> 32@5x5 -> 32@3x3
// -> dense 64 -> dense 3.  37,507 parameters, FP32 master copy.
//   training:  k_ref_fwd (FP32, keeps activations) -> k_ref_bwd (activation
//              gradients per sample) -> k_ref_wgrad (parameter gradients,
//              fixed-order reductions over the batch) -> k_ref_adam
//   inference: k_ref_infer, BF16 weights and activations on the tensor cores
//              (mma.sync m16n8k16, FP32 accumulation), conv+GELU fused with
//              the activations channel-last in shared memory, one CTA per
//              window at a time.
// Loss per sample: 0.5 r^2 + 0.5 stopgrad(r^2) exp(-s) + s.
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include "refiner.cuh"

namespace xcg {

__device__ __forceinline__ float gelu_f(float x) { return 0.5f * x * (1.0f + erff(x * 0.70710678118654752f)); }
__device__ __forceinline__ float gelu_g(float x) {
    return 0.5f * (1.0f + erff(x * 0.70710678118654752f)) + x * 0.39894228040143268f * expf(-0.5f * x * x);
}

// ---------------------------------------------------------------- training forward
// One warp per sample, lane = channel.  Activations (pre- and post-GELU) go to
// the per-sample record `act` for the backward pass.
__global__ void __launch_bounds__(128) k_ref_fwd(RefPlan R, const float *__restrict__ feat, int n) {
    extern __shared__ float sm[];
    float *W2t = sm;                 // [288][32]: (k*9+d, c)
    float *W3t = W2t + 9216;
    const int warp = threadIdx.x >> 5, c = threadIdx.x & 31;
    float *ws = W3t + 9216 + warp * 2816;
    float *x0 = ws, *a1 = x0 + 96, *a2 = a1 + 1568, *a3 = a2 + 800, *g1 = a3 + 288;
    for (int i = threadIdx.x; i < 9216; i += blockDim.x) { W2t[i] = R.w2t[i]; W3t[i] = R.w3t[i]; }
    __syncthreads();
    const float *P = R.theta;
    for (int s = blockIdx.x * 4 + warp; s < n; s += gridDim.x * 4) {
        float *act = R.act + (size_t)s * REF_ACT;
        for (int i = c; i < 81; i += 32) x0[i] = feat[(size_t)s * 81 + i];
        __syncwarp();
        for (int p = 0; p < 49; p++) {
            const int i = p / 7, j = p % 7;
            float y = P[RP_B1 + c];
#pragma unroll
            for (int d = 0; d < 9; d++) y = fmaf(P[RP_W1 + c * 9 + d], x0[(i + d / 3) * 9 + j + d % 3], y);
            act[ACT_Y1 + c * 49 + p] = y;
            const float a = gelu_f(y);
            a1[c * 49 + p] = a;
            act[ACT_A1 + c * 49 + p] = a;
        }
        __syncwarp();
        for (int p = 0; p < 25; p++) {
            const int i = p / 5, j = p % 5;
            float y = P[RP_B2 + c];
            for (int k = 0; k < 32; k++)
#pragma unroll
                for (int d = 0; d < 9; d++) y = fmaf(W2t[(k * 9 + d) * 32 + c], a1[k * 49 + (i + d / 3) * 7 + j + d % 3], y);
            act[ACT_Y2 + c * 25 + p] = y;
            const float a = gelu_f(y);
            a2[c * 25 + p] = a;
            act[ACT_A2 + c * 25 + p] = a;
        }
        __syncwarp();
        for (int p = 0; p < 9; p++) {
            const int i = p / 3, j = p % 3;
            float y = P[RP_B3 + c];
            for (int k = 0; k < 32; k++)
#pragma unroll
                for (int d = 0; d < 9; d++) y = fmaf(W3t[(k * 9 + d) * 32 + c], a2[k * 25 + (i + d / 3) * 5 + j + d % 3], y);
            act[ACT_Y3 + c * 9 + p] = y;
            const float a = gelu_f(y);
            a3[c * 9 + p] = a;
            act[ACT_A3 + c * 9 + p] = a;
        }
        __syncwarp();
#pragma unroll
        for (int h2 = 0; h2 < 2; h2++) {
            const int o = c + 32 * h2;
            float z = P[RP_C1 + o];
            for (int h = 0; h < 288; h++) z = fmaf(R.f1t[h * 64 + o], a3[h], z);
            act[ACT_Z1 + o] = z;
            const float g = gelu_f(z);
            g1[o] = g;
            act[ACT_G1 + o] = g;
        }
        __syncwarp();
        if (c < 3) {
            float o = P[RP_C2 + c];
            for (int k = 0; k < 64; k++) o = fmaf(P[RP_F2 + c * 64 + k], g1[k], o);
            act[ACT_OUT + c] = o;
            if (R.out) R.out[(size_t)s * 3 + c] = o;
        }
        __syncwarp();
    }
}

// ---------------------------------------------------------------- training backward
// One warp per sample: gradients of the loss w.r.t. every pre-activation.
__global__ void __launch_bounds__(128) k_ref_bwd(RefPlan R, const float *__restrict__ target, int n) {
    extern __shared__ float sm[];
    float *W2 = sm;                  // parameter layout [c][k][3][3]
    float *W3 = W2 + 9216;
    const int warp = threadIdx.x >> 5, c = threadIdx.x & 31;
    float *ws = W3 + 9216 + warp * 1184;
    float *dout = ws, *dz1 = dout + 4, *dy3 = dz1 + 64, *dy2 = dy3 + 288;
    for (int i = threadIdx.x; i < 9216; i += blockDim.x) { W2[i] = R.theta[RP_W2 + i]; W3[i] = R.theta[RP_W3 + i]; }
    __syncthreads();
    const float *P = R.theta;
    const float inv_n = 1.0f / (float)n;
    for (int s = blockIdx.x * 4 + warp; s < n; s += gridDim.x * 4) {
        const float *act = R.act + (size_t)s * REF_ACT;
        float *gr = R.grad_act + (size_t)s * REF_ACT;
        if (c == 0) {
            const float fx = act[ACT_OUT], fy = act[ACT_OUT + 1], lv = act[ACT_OUT + 2];
            const float rx = fx - target[2 * s], ry = fy - target[2 * s + 1];
            const float r2 = rx * rx + ry * ry;
            dout[0] = rx * inv_n;
            dout[1] = ry * inv_n;
            dout[2] = (1.0f - 0.5f * r2 * expf(-lv)) * inv_n;
            if (R.loss) R.loss[s] = 0.5f * r2 + 0.5f * r2 * expf(-lv) + lv;
            gr[ACT_OUT] = dout[0]; gr[ACT_OUT + 1] = dout[1]; gr[ACT_OUT + 2] = dout[2];
        }
        __syncwarp();
#pragma unroll
        for (int h2 = 0; h2 < 2; h2++) {
            const int k = c + 32 * h2;
            float g = 0.f;
#pragma unroll
            for (int o = 0; o < 3; o++) g = fmaf(P[RP_F2 + o * 64 + k], dout[o], g);
            const float dz = g * gelu_g(act[ACT_Z1 + k]);
            dz1[k] = dz;
            gr[ACT_Z1 + k] = dz;
        }
        __syncwarp();
        for (int q = 0; q < 9; q++) {
            const int h = c * 9 + q;
            float g = 0.f;
            for (int o = 0; o < 64; o++) g = fmaf(P[RP_F1 + o * 288 + h], dz1[o], g);
            const float dy = g * gelu_g(act[ACT_Y3 + h]);
            dy3[h] = dy;
            gr[ACT_Y3 + h] = dy;
        }
        __syncwarp();
        // conv3 input gradient: lane k, positions of the 5x5 input
        for (int p = 0; p < 25; p++) {
            const int pi = p / 5, pj = p % 5;
            float g = 0.f;
            for (int co = 0; co < 32; co++)
#pragma unroll
                for (int d = 0; d < 9; d++) {
                    const int oi = pi - d / 3, oj = pj - d % 3;
                    if (oi >= 0 && oi < 3 && oj >= 0 && oj < 3) g = fmaf(W3[co * 288 + c * 9 + d], dy3[co * 9 + oi * 3 + oj], g);
                }
            const float dy = g * gelu_g(act[ACT_Y2 + c * 25 + p]);
            dy2[c * 25 + p] = dy;
            gr[ACT_Y2 + c * 25 + p] = dy;
        }
        __syncwarp();
        for (int p = 0; p < 49; p++) {
            const int pi = p / 7, pj = p % 7;
            float g = 0.f;
            for (int co = 0; co < 32; co++)
#pragma unroll
                for (int d = 0; d < 9; d++) {
                    const int oi = pi - d / 3, oj = pj - d % 3;
                    if (oi >= 0 && oi < 5 && oj >= 0 && oj < 5) g = fmaf(W2[co * 288 + c * 9 + d], dy2[co * 25 + oi * 5 + oj], g);
                }
            gr[ACT_Y1 + c * 49 + p] = g * gelu_g(act[ACT_Y1 + c * 49 + p]);
        }
        __syncwarp();
    }
}

// ---------------------------------------------------------------- parameter gradients
// Fixed-order reductions over the batch (no atomics, reproducible).
// Blocks: [0,1024) W2 (c,k); [1024,2048) W3 (c,k); [2048,2080) W1 + biases of
// channel c; [2080,2144) F1 row o + c1[o]; 2144: F2 + c2.
__device__ __forceinline__ float block_sum(float v, float *red) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    const int w = threadIdx.x >> 5;
    __syncthreads();
    if ((threadIdx.x & 31) == 0) red[w] = v;
    __syncthreads();
    float t = 0.f;
    for (int i = 0; i < (int)(blockDim.x >> 5); i++) t += red[i];
    return t;
}

__global__ void __launch_bounds__(128) k_ref_wgrad(RefPlan R, const float *__restrict__ feat, int n) {
    __shared__ float red[8];
    const int b = blockIdx.x;
    const float *A = R.act, *G = R.grad_act;
    float *g = R.grad;
    if (b < 2048) {
        const bool l3 = b >= 1024;
        const int cc = (b & 1023) >> 5, k = b & 31;
        const int Ho = l3 ? 3 : 5, Hi = l3 ? 5 : 7;
        const int oG = l3 ? ACT_Y3 : ACT_Y2, oA = l3 ? ACT_A2 : ACT_A1;
        float acc[9];
#pragma unroll
        for (int d = 0; d < 9; d++) acc[d] = 0.f;
        for (int s = threadIdx.x; s < n; s += blockDim.x) {
            const float *dy = G + (size_t)s * REF_ACT + oG + cc * Ho * Ho;
            const float *a = A + (size_t)s * REF_ACT + oA + k * Hi * Hi;
            for (int p = 0; p < Ho * Ho; p++) {
                const float v = dy[p];
                const int i = p / Ho, j = p % Ho;
#pragma unroll
                for (int d = 0; d < 9; d++) acc[d] = fmaf(v, a[(i + d / 3) * Hi + j + d % 3], acc[d]);
            }
        }
        for (int d = 0; d < 9; d++) {
            const float t = block_sum(acc[d], red);
            if (threadIdx.x == 0) g[(l3 ? RP_W3 : RP_W2) + cc * 288 + k * 9 + d] = t;
        }
    } else if (b < 2080) {
        const int cc = b - 2048;
        float acc[9], sb1 = 0.f, sb2 = 0.f, sb3 = 0.f;
#pragma unroll
        for (int d = 0; d < 9; d++) acc[d] = 0.f;
        for (int s = threadIdx.x; s < n; s += blockDim.x) {
            const float *dy = G + (size_t)s * REF_ACT + ACT_Y1 + cc * 49;
            const float *x = feat + (size_t)s * 81;
            for (int p = 0; p < 49; p++) {
                const float v = dy[p];
                sb1 += v;
                const int i = p / 7, j = p % 7;
#pragma unroll
                for (int d = 0; d < 9; d++) acc[d] = fmaf(v, x[(i + d / 3) * 9 + j + d % 3], acc[d]);
            }
            for (int p = 0; p < 25; p++) sb2 += G[(size_t)s * REF_ACT + ACT_Y2 + cc * 25 + p];
            for (int p = 0; p < 9; p++) sb3 += G[(size_t)s * REF_ACT + ACT_Y3 + cc * 9 + p];
        }
        for (int d = 0; d < 9; d++) {
            const float t = block_sum(acc[d], red);
            if (threadIdx.x == 0) g[RP_W1 + cc * 9 + d] = t;
        }
        float t = block_sum(sb1, red); if (threadIdx.x == 0) g[RP_B1 + cc] = t;
        t = block_sum(sb2, red); if (threadIdx.x == 0) g[RP_B2 + cc] = t;
        t = block_sum(sb3, red); if (threadIdx.x == 0) g[RP_B3 + cc] = t;
    } else if (b < 2144) {
        const int o = b - 2080;
        // thread h accumulates F1[o][h] over the batch (h = tid, tid+128, tid+256)
        for (int h = threadIdx.x; h < 288; h += blockDim.x) {
            float acc = 0.f;
            for (int s = 0; s < n; s++) acc = fmaf(G[(size_t)s * REF_ACT + ACT_Z1 + o], A[(size_t)s * REF_ACT + ACT_A3 + h], acc);
            g[RP_F1 + o * 288 + h] = acc;
        }
        float sb = 0.f;
        for (int s = threadIdx.x; s < n; s += blockDim.x) sb += G[(size_t)s * REF_ACT + ACT_Z1 + o];
        const float t = block_sum(sb, red);
        if (threadIdx.x == 0) g[RP_C1 + o] = t;
    } else {
        for (int e = threadIdx.x; e < 192 + 3; e += blockDim.x) {
            float acc = 0.f;
            if (e < 192) {
                const int o = e / 64, k = e % 64;
                for (int s = 0; s < n; s++) acc = fmaf(G[(size_t)s * REF_ACT + ACT_OUT + o], A[(size_t)s * REF_ACT + ACT_G1 + k], acc);
                g[RP_F2 + e] = acc;
            } else {
                for (int s = 0; s < n; s++) acc += G[(size_t)s * REF_ACT + ACT_OUT + (e - 192)];
                g[RP_C2 + e - 192] = acc;
            }
        }
    }
}

// ---------------------------------------------------------------- Adam + derived copies
__global__ void k_ref_adam(RefPlan R, float lr, float b1, float b2, float eps, float c1, float c2) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < RP_N; i += gridDim.x * blockDim.x) {
        const float gi = R.grad[i];
        const float m = b1 * R.m[i] + (1.f - b1) * gi;
        const float v = b2 * R.v[i] + (1.f - b2) * gi * gi;
        R.m[i] = m;
        R.v[i] = v;
        R.theta[i] = R.theta[i] - lr * (m / c1) / (sqrtf(v / c2) + eps);
    }
}

// transposed FP32 copies for the training forward and BF16 copies for inference
__global__ void k_ref_derive(RefPlan R) {
    __nv_bfloat16 *wb = reinterpret_cast<__nv_bfloat16 *>(R.wpack);
    float *ws = reinterpret_cast<float *>(R.wpack + INF_ROWS * INF_KS * 2);
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < INF_ROWS * INF_KS; e += gridDim.x * blockDim.x) {
        const int n = e / INF_KS, kk = e % INF_KS;
        float v = 0.f;
        if (kk < 288) {
            const int hi = kk >> 5, lo = kk & 31;        // tap (or dense input position), input channel
            const int base = (n < 32) ? RP_W2 + n * 288 : (n < 64) ? RP_W3 + (n - 32) * 288 : RP_F1 + (n - 64) * 288;
            v = R.theta[base + lo * 9 + hi];
        }
        wb[e] = __float2bfloat16_rn(v);
    }
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < INF_SMALL; e += gridDim.x * blockDim.x) {
        float v = 0.f;
        if (e < 288) v = R.theta[RP_W1 + e];
        else if (e < 320) v = R.theta[RP_B1 + e - 288];
        else if (e < 352) v = R.theta[RP_B2 + e - 320];
        else if (e < 384) v = R.theta[RP_B3 + e - 352];
        else if (e < 448) v = R.theta[RP_C1 + e - 384];
        else if (e < 643) v = R.theta[RP_F2 + e - 448];       // F2 (192) then c2 (3)
        ws[e] = v;
    }
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < RP_N; i += gridDim.x * blockDim.x) {
        const float t = R.theta[i];
        if (i >= RP_W2 && i < RP_W2 + 9216) { const int e = i - RP_W2, c = e / 288, kk = e % 288; R.w2t[kk * 32 + c] = t; }
        if (i >= RP_W3 && i < RP_W3 + 9216) { const int e = i - RP_W3, c = e / 288, kk = e % 288; R.w3t[kk * 32 + c] = t; }
        if (i >= RP_F1 && i < RP_F1 + 18432) { const int e = i - RP_F1, o = e / 288, h = e % 288; R.f1t[h * 64 + o] = t; }
    }
}

// ---------------------------------------------------------------- inference, BF16 tensor cores
// mma.sync m16n8k16 row.col bf16 -> f32.  Fragment layout (PTX ISA): with
// g = lane/4, t = lane%4, A regs {a0: (g, 2t..2t+1), a1: (g+8, 2t..), a2: (g, 2t+8..),
// a3: (g+8, 2t+8..)}, B regs {b0: (k=2t..2t+1, n=g), b1: (k=2t+8.., n=g)},
// C {c0,c1: (g, 2t..2t+1), c2,c3: (g+8, 2t..2t+1)}.
__device__ __forceinline__ void mma_bf16(float (&d)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1) {
    asm volatile("mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};\n"
                 : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
                 : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// Per-CTA shared memory of the inference kernel after the parameter pack:
// the window's input (81 f32, padded to 84) and its activations, channel-last
// with a padded channel stride INF_CS (conv1 out 7x7, conv2 out 5x5, conv3
// out 3x3, BF16), then the dense layer's 64 outputs (f32).
constexpr int INF_CS = 40;
constexpr int INF_ACT_BYTES = 84 * 4 + (49 + 25 + 9) * INF_CS * 2 + 64 * 4;
constexpr int INF_GROUPS = 2;      // windows per CTA at a time (four warps each)

// One warp's share of a convolution or dense layer as m16n8k16 tiles: rows are
// output positions (mt: 16-row tile), columns output channels (n-tiles nt0,
// nt0 + 1), K = 288 walked tap by tap (k' = 32 tap + c_in).  a_row(m) is the
// BF16 activation row of output position m's tap-0 input (nullptr: padding
// row), step(tap) the offset of tap's input row from it; B rows are INF_KS apart.
template <class ARow, class Step>
__device__ __forceinline__ void warp_gemm_288(float (&acc)[2][4], ARow a_row, Step step, const __nv_bfloat16 *B,
                                              int mt, int nt0, int lane) {
    const int g = lane >> 2, t = lane & 3;
    const __nv_bfloat16 *r0 = a_row(mt * 16 + g), *r1 = a_row(mt * 16 + g + 8);
    const __nv_bfloat16 *b0p = B + (size_t)(nt0 * 8 + g) * INF_KS + 2 * t;
    const __nv_bfloat16 *b1p = b0p + 8 * INF_KS;
#pragma unroll 3
    for (int ks = 0; ks < 18; ks++) {
        const int off = step(ks >> 1) + (ks & 1) * 16 + 2 * t;
        uint32_t a[4];
        a[0] = r0 ? *reinterpret_cast<const uint32_t *>(r0 + off) : 0u;
        a[1] = r1 ? *reinterpret_cast<const uint32_t *>(r1 + off) : 0u;
        a[2] = r0 ? *reinterpret_cast<const uint32_t *>(r0 + off + 8) : 0u;
        a[3] = r1 ? *reinterpret_cast<const uint32_t *>(r1 + off + 8) : 0u;
        const int k0 = ks * 16;
        mma_bf16(acc[0], a, *reinterpret_cast<const uint32_t *>(b0p + k0), *reinterpret_cast<const uint32_t *>(b0p + k0 + 8));
        mma_bf16(acc[1], a, *reinterpret_cast<const uint32_t *>(b1p + k0), *reinterpret_cast<const uint32_t *>(b1p + k0 + 8));
    }
}

__device__ __forceinline__ void cp_async16(void *smem, const void *gmem) {
    const unsigned d = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(d), "l"(gmem) : "memory");
}

// A CTA of four warps per window at a time (grid-stride over the windows):
// conv1 on the SIMT pipes in FP32 (K = 9), conv2, conv3 and the dense
// 288 -> 64 layer as tensor-core tiles with bias + GELU applied to the
// accumulators, the 64 -> 3 layer as warp dot products.  With the
// activations channel-last, each A-fragment element pair is one 32-bit load.
// the decision of RefDecide for window w: r3 = (fx, fy, s), f its 9x9 neighbourhood
__device__ static void ref_decide(const RefDecide &D, int w, const float *r3, const float *f) {
    const float fx = r3[0], fy = r3[1], sg = expf(0.5f * r3[2]);
    auto vertex = [](float a, float b, float c) {
        const float den = a - 2.f * b + c;
        return (den < 0.f) ? 0.5f * (a - c) / den : 0.f;
    };
    const float px = vertex(f[4 * 9 + 3], f[4 * 9 + 4], f[4 * 9 + 5]);
    const float py = vertex(f[3 * 9 + 4], f[4 * 9 + 4], f[5 * 9 + 4]);
    const bool ok = (sg < D.max_sigma) && fabsf(fx - px) < D.max_dis && fabsf(fy - py) < D.max_dis &&
                    isfinite(fx) && isfinite(fy) && f[4 * 9 + 4] > 0.f;
    D.skip[w] = ok ? 1 : 0;
    if (ok) {
        xcg_result &o = D.res[w];
        o.xfrac = fx;
        o.yfrac = fy;
        o.fip = -1;
        o.fjp = -1;
        o.flags |= XCG_FLAG_REFINED;
    }
}

__global__ void __launch_bounds__(128 * INF_GROUPS) k_ref_infer(RefPlan R, const float *__restrict__ feat,
                                                                 float *__restrict__ out, int n, RefDecide D) {
    extern __shared__ __align__(16) unsigned char smc[];
    const __nv_bfloat16 *B2 = reinterpret_cast<const __nv_bfloat16 *>(smc);    // [32][INF_KS]
    const __nv_bfloat16 *B3 = B2 + 32 * INF_KS;
    const __nv_bfloat16 *BF = B3 + 32 * INF_KS;                                 // [64][INF_KS]
    const float *small = reinterpret_cast<const float *>(smc + INF_ROWS * INF_KS * 2);
    // one group of four warps per window; each group has its own activations
    const int grp = threadIdx.x >> 7, gt = threadIdx.x & 127;
    float *x0 = reinterpret_cast<float *>(smc + INF_PACK_BYTES + (size_t)grp * INF_ACT_BYTES);   // [84]
    __nv_bfloat16 *a1 = reinterpret_cast<__nv_bfloat16 *>(x0 + 84);             // [49][INF_CS]
    __nv_bfloat16 *a2 = a1 + 49 * INF_CS;                                       // [25][INF_CS]
    __nv_bfloat16 *a3 = a2 + 25 * INF_CS;                                       // [9][INF_CS]
    float *g1 = reinterpret_cast<float *>(a3 + 9 * INF_CS);                     // [64]
    const float *W1 = small, *b1 = small + 288, *b2 = small + 320, *b3 = small + 352, *c1 = small + 384;
    const float *F2 = small + 448, *c2 = small + 448 + 192;

    // the parameter pack, 16 bytes per copy (no waits on flags: cp.async groups)
    for (int i = threadIdx.x; i < INF_PACK_BYTES / 16; i += blockDim.x) cp_async16(smc + 16 * i, R.wpack + 16 * i);
    asm volatile("cp.async.commit_group;\ncp.async.wait_group 0;\n" ::: "memory");
    __syncthreads();

    const int warp = gt >> 5, lane = threadIdx.x & 31;      // warp within the group
    const int g = lane >> 2, t = lane & 3;
    // the groups of a CTA take windows base + grp; barriers stay CTA-wide, so
    // a group without a window in the last round still takes part in them
    for (int base = blockIdx.x * INF_GROUPS; base < n; base += gridDim.x * INF_GROUPS) {
        const int w = base + grp;
        const bool have = w < n;
        if (gt < 81) x0[gt] = have ? feat[(size_t)w * 81 + gt] : 0.f;
        __syncthreads();
        // conv1 (FP32): lane = output channel, warps take positions in turn
        for (int p = warp; p < 49; p += 4) {
            const int i = p / 7, j = p % 7;
            float y = b1[lane];
#pragma unroll
            for (int d = 0; d < 9; d++) y = fmaf(W1[lane * 9 + d], x0[(i + d / 3) * 9 + j + d % 3], y);
            a1[p * INF_CS + lane] = __float2bfloat16_rn(gelu_f(y));
        }
        __syncthreads();
        // conv2: 25 positions (2 row tiles) x 32 channels (4 n-tiles); warp: tile mt = warp/2, n-tiles 2 (warp%2) +0/1
        {
            float acc[2][4] = {};
            auto row = [&](int m) -> const __nv_bfloat16 * {
                return (m < 25) ? a1 + ((m / 5) * 7 + m % 5) * INF_CS : nullptr;
            };
            auto step = [&](int tap) { return ((tap / 3) * 7 + tap % 3) * INF_CS; };
            const int mt = warp >> 1, nt0 = 2 * (warp & 1);
            warp_gemm_288(acc, row, step, B2, mt, nt0, lane);
#pragma unroll
            for (int q = 0; q < 2; q++)
#pragma unroll
                for (int h = 0; h < 4; h++) {
                    const int m = mt * 16 + g + (h >> 1) * 8, ch = (nt0 + q) * 8 + 2 * t + (h & 1);
                    if (m < 25) a2[m * INF_CS + ch] = __float2bfloat16_rn(gelu_f(acc[q][h] + b2[ch]));
                }
        }
        __syncthreads();
        // conv3: 9 positions (1 row tile) x 32 channels; warps 0, 1 take two n-tiles each
        if (warp < 2) {
            float acc[2][4] = {};
            auto row = [&](int m) -> const __nv_bfloat16 * {
                return (m < 9) ? a2 + ((m / 3) * 5 + m % 3) * INF_CS : nullptr;
            };
            auto step = [&](int tap) { return ((tap / 3) * 5 + tap % 3) * INF_CS; };
            const int nt0 = 2 * warp;
            warp_gemm_288(acc, row, step, B3, 0, nt0, lane);
#pragma unroll
            for (int q = 0; q < 2; q++)
#pragma unroll
                for (int h = 0; h < 4; h++) {
                    const int m = g + (h >> 1) * 8, ch = (nt0 + q) * 8 + 2 * t + (h & 1);
                    if (m < 9) a3[m * INF_CS + ch] = __float2bfloat16_rn(gelu_f(acc[q][h] + b3[ch]));
                }
        }
        __syncthreads();
        // dense 288 -> 64: one row (this window), k' = 32 position + channel; warp: n-tiles 2 warp +0/1
        {
            float acc[2][4] = {};
            auto row = [&](int m) -> const __nv_bfloat16 * { return (m == 0) ? a3 : nullptr; };
            auto step = [&](int pos) { return pos * INF_CS; };
            const int nt0 = 2 * warp;
            warp_gemm_288(acc, row, step, BF, 0, nt0, lane);
            if (g == 0)
#pragma unroll
                for (int q = 0; q < 2; q++)
#pragma unroll
                    for (int h = 0; h < 2; h++) {
                        const int o = (nt0 + q) * 8 + 2 * t + h;
                        g1[o] = gelu_f(acc[q][h] + c1[o]);
                    }
        }
        __syncthreads();
        // 64 -> 3, then the decision (x0 still holds the neighbourhood)
        if (warp == 0 && have) {
            float r3[3];
#pragma unroll
            for (int o = 0; o < 3; o++) {
                float v = fmaf(F2[o * 64 + lane], g1[lane], F2[o * 64 + 32 + lane] * g1[32 + lane]);
#pragma unroll
                for (int s = 16; s > 0; s >>= 1) v += __shfl_xor_sync(0xffffffffu, v, s);
                r3[o] = v + c2[o];
                if (lane == 0) out[(size_t)w * 3 + o] = r3[o];
            }
            if (D.skip && lane == 0) ref_decide(D, w, r3, x0);
        }
        __syncthreads();                           // x0 .. g1 are reused by the next window
    }
}

size_t ref_fwd_smem() { return (size_t)(2 * 9216 + 4 * 2816) * sizeof(float); }
size_t ref_bwd_smem() { return (size_t)(2 * 9216 + 4 * 1184) * sizeof(float); }
size_t ref_infer_smem() { return (size_t)INF_PACK_BYTES + (size_t)INF_GROUPS * INF_ACT_BYTES; }

cudaError_t ref_setup() {
    cudaError_t e = cudaFuncSetAttribute(k_ref_fwd, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ref_fwd_smem());
    if (!e) e = cudaFuncSetAttribute(k_ref_bwd, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ref_bwd_smem());
    if (!e) e = cudaFuncSetAttribute(k_ref_infer, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ref_infer_smem());
    return e;
}

void ref_launch_fwd(const RefPlan &R, const float *feat, int n, cudaStream_t s) {
    const int blocks = (n + 3) / 4 < 608 ? (n + 3) / 4 : 608;
    k_ref_fwd<<<blocks, 128, ref_fwd_smem(), s>>>(R, feat, n);
}
void ref_launch_bwd(const RefPlan &R, const float *target, int n, cudaStream_t s) {
    const int blocks = (n + 3) / 4 < 608 ? (n + 3) / 4 : 608;
    k_ref_bwd<<<blocks, 128, ref_bwd_smem(), s>>>(R, target, n);
}
void ref_launch_wgrad(const RefPlan &R, const float *feat, int n, cudaStream_t s) {
    k_ref_wgrad<<<2145, 128, 0, s>>>(R, feat, n);
}
void ref_launch_adam(const RefPlan &R, float lr, int step, cudaStream_t s) {
    const float b1 = 0.9f, b2 = 0.999f;
    const float c1 = 1.f - powf(b1, (float)step), c2 = 1.f - powf(b2, (float)step);
    k_ref_adam<<<(RP_N + 255) / 256, 256, 0, s>>>(R, lr, b1, b2, 1e-8f, c1, c2);
}
void ref_launch_derive(const RefPlan &R, cudaStream_t s) { k_ref_derive<<<(RP_N + 255) / 256, 256, 0, s>>>(R); }
void ref_launch_infer(const RefPlan &R, const float *feat, float *out, int n, cudaStream_t s, const RefDecide *D) {
    // INF_GROUPS windows per CTA at a time, two CTAs per SM (91 KB of shared memory each)
    const int need = (n + INF_GROUPS - 1) / INF_GROUPS;
    const int blocks = need < 2 * 152 ? need : 2 * 152;
    const RefDecide none{nullptr, nullptr, 0.f, 0.f};
    k_ref_infer<<<blocks > 0 ? blocks : 1, 128 * INF_GROUPS, ref_infer_smem(), s>>>(R, feat, out, n, D ? *D : none);
}

}  // namespace xcg
