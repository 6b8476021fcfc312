// Subpixel refiner internals: parameter and activation layouts, plan, launchers.
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>

namespace xcg {

// flat parameter vector (FP32): conv weights [c_out][c_in][3][3], dense [out][in]
constexpr int RP_W1 = 0, RP_B1 = 288, RP_W2 = 320, RP_B2 = 9536, RP_W3 = 9568, RP_B3 = 18784, RP_F1 = 18816,
              RP_C1 = 37248, RP_F2 = 37312, RP_C2 = 37504, RP_N = 37507;
// per-sample activation record (and the same layout for its gradients)
constexpr int ACT_Y1 = 0, ACT_A1 = 1568, ACT_Y2 = 3136, ACT_A2 = 3936, ACT_Y3 = 4736, ACT_A3 = 5024, ACT_Z1 = 5312,
              ACT_G1 = 5376, ACT_OUT = 5440, REF_ACT = 5444;
// shared bytes per warp in the inference kernel: x0 4x84 f32, a1 4x32x49 bf16,
// a2 4x32x25 bf16, a3 4x288 bf16, g1 4x64 f32
constexpr int WARP_INFER_BYTES = 4 * 84 * 4 + 4 * 32 * 49 * 2 + 4 * 32 * 25 * 2 + 4 * 288 * 2 + 4 * 64 * 4;

struct RefPlan {
    float *theta, *m, *v, *grad;        // RP_N each
    float *w2t, *w3t, *f1t;             // transposed FP32 copies (training forward)
    __nv_bfloat16 *wbf;                 // BF16 copy (inference)
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
void ref_launch_infer(const RefPlan &R, const float *feat, float *out, int n, cudaStream_t s);

}  // namespace xcg
