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
void set_last_error(const char *msg);
// Range-interpolation table of the row kernel for n-point rows and factor ri
// (Plan::phase), written to dst; returns the entries written, (ri-1)*n (1
// for ri = 1).  For ri = 2 and n <= 512 it holds the half-shift twiddles of
// team_ifft_half_shift, else the phase factors exp(2 pi i f' p/(ri n))/n.
int put_row_phase(float2 *dst, int n, int ri);
}  // namespace xcg
