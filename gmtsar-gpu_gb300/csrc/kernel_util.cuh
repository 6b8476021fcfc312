// Device helpers shared by the kernels of the frequency-domain path
// (xcorr_kernels.cu, segment_rows.cu): amplitude, exact power-of-two
// reciprocals, the slave row shift, warp sums, cp.async wrappers and the
// column stage's launch geometry.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "team_fft.cuh"
#include "xcorr_plan.cuh"

namespace xcg {

__device__ __forceinline__ double warp_sum_f64(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// |v| of an interpolated sample.  The reference's amplitudes (hypotf of its
// cuFFT outputs) and these (of this library's own FFT outputs) already differ
// by transform rounding, so the hardware square root approximation
// (sqrt.approx.f32) stands in for the correctly rounded sqrtf, whose
// special-case branch cost k_rows 7% of its instructions.  Measured on GB300
// against sqrtf: at most one unit in the last place (exhaustively over
// [1, 4), so over every binade), equal on 83% of inputs, exact at zero.  The
// flush-to-zero form drops the subnormal fix-up: a sum of squares below
// 1.2e-38 (never negative) gives 0 instead of a value below 1.1e-19.
__device__ __forceinline__ float amp_of(float2 v) {
    const float s = fmaf(v.x, v.x, v.y * v.y);
    float r;
    asm("sqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(s));
    return r;
}

// 1 / n for n a power of two, exactly (built from the exponent bits)
__device__ __forceinline__ double pow2_inv(int n) {
    const int lg = 31 - __clz(n);
    return __longlong_as_double((long long)(1023 - lg) << 52);
}

__device__ __forceinline__ int slave_row_shift(const PairDev &pd, int y) {
    return (int)((double)y * pd.astretcha);    // ishft, read_xcorr_data.c:65
}

// ---------------------------------------------------------------- cp.async
__device__ __forceinline__ void cp_async8(void *smem, const void *gmem) {
    const unsigned d = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(d), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async4(void *smem, const void *gmem) {
    const unsigned d = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(d), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async16(void *smem, const void *gmem) {   // 16-byte aligned both
    const unsigned d = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(d), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int NPEND>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(NPEND) : "memory"); }

// Launch shapes a plan selects (Plan::cols_cfg, Plan::peak_cfg; the stack's
// autotuner times them per window geometry):
//   k_cols  0: 128 threads, staging in two cp.async groups (partner columns
//              first), 5 CTAs/SM (the default); 1: 256 threads (twice the
//              column pairs per CTA), two groups; 2: 128 threads, one group
//   k_peak  0: 4 resident CTAs/SM (64 registers, a few spills; beats 3 for
//              transforms up to 256 points), 3 for 512 points; 1: one fewer
#define XCG_COLS_BLOCKS 5

template <int M, int THR = 128>
struct ColsGeom {
    static constexpr int T = fft_lanes(M);
    static constexpr int PADM = fft_padded_len(M);
    static constexpr int THREADS = THR;
    static constexpr int CP = THREADS / T;        // column pairs per CTA = teams
    // slot stride in float2: a multiple of 16 plus 16 / CP, so that the
    // (slot, row) pairs a half-warp stages or copies out (CP slots x 16 / CP
    // rows) fall in distinct bank pairs
    static constexpr int CS = PADM + ((CP >= 16) ? 1 : 16 / CP);
    static constexpr int TWL = fft_twiddle_len(M);
    static constexpr int BLOCKS = (M >= 1024) ? (THREADS >= 256 ? 1 : 2)
                                : (M >= 512 ? (THREADS >= 256 ? 1 : 3) : XCG_COLS_BLOCKS * 128 / THREADS);
};

}  // namespace xcg
