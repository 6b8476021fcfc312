// Launch entry points of the -time / -time4 kernels (time_corr.cu).
#pragma once
#include <cuda_runtime.h>

#include "xcorr_plan.cuh"

namespace xcg {
cudaError_t time_setup(const Plan &P);
size_t time_smem_needed(int nx_corr, int mode);
void launch_tcorr(const Plan &P, cudaStream_t s);
void launch_tpeak(const Plan &P, cudaStream_t s);
}  // namespace xcg
