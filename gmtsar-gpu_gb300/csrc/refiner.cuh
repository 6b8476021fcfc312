// Subpixel refiner internals: parameter and activation layouts, plan, launchers.
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "xcorr_gb300.h"

namespace xcg {

// flat parameter vector (FP32): conv weights [c_out][c_in][3][3], dense [out][in]
constexpr int RP_W1 = 0, RP_B1 = 288, RP_W2 = 320, RP_B2 = 9536, RP_W3 = 9568, RP_B3 = 18784, RP_F1 = 18816,
              RP_C1 = 37248, RP_F2 = 37312, RP_C2 = 37504, RP_N = 37507;
// per-sample activation record (and the same layout for its gradients)
constexpr int ACT_Y1 = 0, ACT_A1 = 1568, ACT_Y2 = 3136, ACT_A2 = 3936, ACT_Y3 = 4736, ACT_A3 = 5024, ACT_Z1 = 5312,
              ACT_G1 = 5376, ACT_OUT = 5440, REF_ACT = 5444;
// Inference parameter pack (built by k_ref_derive, copied whole into each
// inference CTA's shared memory): 128 BF16 weight rows -- conv2 (32), conv3
// (32), dense 288->64 (64) -- with K reordered tap- (or position-) major,
// k' = 32 * tap + c_in, and padded to INF_KS so the B-fragment loads of
// eight rows hit distinct banks; then INF_SMALL floats: conv1 weights (288),
// biases b1 b2 b3 (3 x 32), dense bias c1 (64), the 64->3 layer (192 + 3).
constexpr int INF_KS = 296;
constexpr int INF_ROWS = 128;
constexpr int INF_SMALL = 648;
constexpr int INF_PACK_BYTES = INF_ROWS * INF_KS * 2 + INF_SMALL * 4;     // 78,368

struct RefPlan {
    float *theta, *m, *v, *grad;        // RP_N each
    float *w2t, *w3t, *f1t;             // transposed FP32 copies (training forward)
    unsigned char *wpack;               // INF_PACK_BYTES, the inference parameter pack
    float *act, *grad_act;              // [batch][REF_ACT]
    float *loss;                        // [batch] per-sample loss (nullable)
    float *out;                         // [batch][3] training-forward outputs (nullable)
};

cudaError_t ref_setup();
void ref_launch_fwd(const RefPlan &R, const float *feat, int n, cudaStream_t s);
void ref_launch_bwd(const RefPlan &R, const float *target, int n, cudaStream_t s);
void ref_launch_wgrad(const RefPlan &R, const float *feat, int n, cudaStream_t s);
void ref_launch_adam(const RefPlan &R, float lr, int step, cudaStream_t s);
void ref_launch_derive(const RefPlan &R, cudaStream_t s);
// The refined path's decision, taken by the inference kernel for each window
// it evaluates: the refiner's (fx, fy) replace the FFT interpolation where
// the predicted standard deviation exp(s/2) is below max_sigma and both
// coordinates lie within max_dis of a three-point parabola fit through the
// centre row and column of the 9x9 neighbourhood.
struct RefDecide {
    xcg_result *res;              // [n] the windows' result records
    unsigned char *skip;          // [n] 1: refined, the subpixel stage leaves the window alone
    float max_sigma, max_dis;
};
// Inference of n windows' (fx, fy, s); with D, also the decision above.
void ref_launch_infer(const RefPlan &R, const float *feat, float *out, int n, cudaStream_t s,
                      const RefDecide *D = nullptr);

}  // namespace xcg
