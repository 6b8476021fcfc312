// Context internals shared by the C ABI translation units.
#pragma once
#include <cuda_runtime.h>

#include <vector>

#include "xcorr_gb300.h"
#include "xcorr_plan.cuh"

struct xcg_ctx {
    xcg_params prm;
    int device;
    xcg::Plan base;           // sizes and tables; per-batch fields filled at launch
    // tables
    float2 *d_tables = nullptr;
    // scratch
    void *d_scratch = nullptr;
    size_t scratch_bytes = 0;
    int max_batch = 0;
    size_t off_zrow, off_amp1, off_amp2c, off_part, off_oob, off_minmax, off_means, off_qspec, off_surf, off_md,
        off_mdnext, off_corr0n;
    // host-entry buffers
    void *d_img[2] = {nullptr, nullptr};
    size_t img_bytes[2] = {0, 0};
    xcg_loc *d_locs = nullptr;
    xcg_result *d_res = nullptr;
    int io_cap = 0;
    cudaStream_t stream = nullptr;
    // profiling
    int profiling = 0;
    std::vector<cudaEvent_t> events;
    xcg_stats stats;
};

namespace xcg {
// The context's plan with its tables and scratch filled in; the caller sets
// the pair fields, the window arrays and launches with ctx_launch.
Plan ctx_plan(const xcg_ctx *c);
// Launch the four kernels for windows [starts[b], starts[b+1]) of the
// window arrays in P (locs, winref), b < nbatch; updates the context stats.
xcg_status ctx_launch(xcg_ctx *c, Plan P, const int *starts, int nbatch, cudaStream_t s);
void set_last_error(const char *msg);
}  // namespace xcg
