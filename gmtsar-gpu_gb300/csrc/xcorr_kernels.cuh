// Launch entry points of the xcorr kernels (xcorr_kernels.cu).
#pragma once
#include <cuda_runtime.h>

#include "xcorr_plan.cuh"

namespace xcg {
cudaError_t kernels_setup(const Plan &P);
void launch_rows(const Plan &P, cudaStream_t s);
void launch_cols(const Plan &P, cudaStream_t s);
void launch_peak(const Plan &P, cudaStream_t s);
void launch_subpix(const Plan &P, cudaStream_t s);
void launch_decide(const Plan &P, const float *pred, unsigned char *skip, float max_sigma, float max_dis,
                   cudaStream_t s);
void set_last_error(const char *msg);
}  // namespace xcg
