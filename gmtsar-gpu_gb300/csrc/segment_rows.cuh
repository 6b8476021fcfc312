// Launch entry points of the shared-row-segment path (segment_rows.cu).
#pragma once
#include <cuda_runtime.h>

#include "xcorr_plan.cuh"

namespace xcg {
// windows per batch the planner takes (two patch entries each)
constexpr int RC_MAX_WINDOWS = 2048;
cudaError_t segrows_setup(const Plan &P);
// chunks of 1024 samples the chunk arrays must hold for nwin windows
size_t rc_max_chunks(int npx, int npy, int nwin);
void launch_rc_plan(const Plan &P, cudaStream_t s);
void launch_segrows(const Plan &P, cudaStream_t s);
void launch_cols_rc(const Plan &P, cudaStream_t s);
}  // namespace xcg
