// Context internals shared by the C ABI translation units.
#pragma once
#include <cuda_runtime.h>

#include <functional>
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
    size_t scratch_bytes = 0;     // all slots
    int max_batch = 0;            // windows per batch (per slot)
    // consecutive batches alternate between slots on their own streams, so
    // one batch's column/peak stages overlap the next batch's row stage; a
    // call whose batches fit in half a slot runs them in 2 nslots lanes, each
    // half of a slot, so that four batches are in flight
    int nslots = 2;
    static constexpr int MAX_LANES = 4;
    cudaStream_t slot_stream[MAX_LANES] = {};
    cudaEvent_t ev_fork = nullptr, ev_join[MAX_LANES] = {};
    int batches_cfg = 0;          // xcg_set_batches: batches per call (0: automatic)
    // host entry: the two images are copied on one stream in row bands, and
    // each row-stage sub-launch waits only for its band
    cudaStream_t copy_stream = nullptr;
    std::vector<cudaEvent_t> band_ready;      // one per band of a call
    // scratch arrays of one slot (offsets from its start) for a batch capacity
    struct Layout {
        size_t zrow, amp1, amp2c, part, oob, minmax, means, qspec, surf, md, mdnext, corr0n;
        // shared row segments (segment_rows.cu): chunk arrays
        size_t rc_desc, rc_wch, rc_count, rc_amp, rc_spec, rc_part, rc_minmax, rc_oob, rc_order, rc_band_start,
            rc_tile_next;
        size_t slot_bytes;
        int windows;
    };
    // lay[0]: nslots slots of max_batch windows; lay[1]: 2 nslots lanes of
    // max_batch / 2 windows in the same memory (windows 0: none)
    Layout lay[2] = {};
    // host-entry buffers
    void *d_img[2] = {nullptr, nullptr};
    size_t img_bytes[2] = {0, 0};
    xcg_loc *d_locs = nullptr;
    xcg_result *d_res = nullptr;
    void *h_io = nullptr;         // pinned: io_cap locations, then io_cap results
    int io_cap = 0;
    cudaStream_t stream = nullptr;
    // optional per-window 9x9 neighbourhoods written by xcg_correlate_device
    float *features = nullptr;
    // buffers of the refined path (xcg_correlate_device_refined)
    float *ref_feat = nullptr, *ref_pred = nullptr;
    unsigned char *ref_skip = nullptr;
    int ref_cap = 0;
    // precision form: prepared DFT operands and the tensor-core error flag
    uint8_t *tc_prep = nullptr;
    int *tc_err = nullptr;
    int inject_tc_timeout = 0;    // xcg_debug_inject_stage_timeout: the next call sets the flag instead of clearing it
    // profiling: 1 events around each launch, 2 timeline marks
    int profiling = 0;
    std::vector<cudaEvent_t> events;
    std::vector<cudaEvent_t> tl_events;
    std::vector<int> tl_tags;             // marks of the current call, in order of recording
    xcg_stats stats;
};

namespace xcg {
// The context's plan with its tables and scratch filled in; the caller sets
// the pair fields, the window arrays and launches with ctx_launch.
Plan ctx_plan(const xcg_ctx *c);
// P with its scratch pointers in lane `lane` of layout `mode` (0: slots of
// max_batch windows, 1: half slots).
Plan in_lane(const xcg_ctx *c, Plan P, int mode, int lane);
// Launches the row stage of one batch (plan Q) on stream ss in place of the
// single row launch; the host entry copies image bands between sub-launches.
using RowsHook = std::function<xcg_status(const Plan &Q, cudaStream_t ss)>;
// Launch the four kernels for windows [starts[b], starts[b+1]) of the
// window arrays in P (locs, winref), b < nbatch; updates the context stats.
// `tail`, when given, stands in for the subpixel launch of each batch (the
// refined path: refiner inference, decision, subpixel stage for the rest).
xcg_status ctx_launch(xcg_ctx *c, Plan P, const int *starts, int nbatch, cudaStream_t s,
                      const RowsHook &rows = {}, const RowsHook &tail = {});
// Timeline mode: record mark `tag` on stream ss; tl_finish (after the call's
// work was enqueued) waits for the device and fills the stats' timeline.
xcg_status tl_mark(xcg_ctx *c, cudaStream_t ss, int tag);
xcg_status tl_finish(xcg_ctx *c, cudaStream_t s);
// Windows per batch xcg_correlate_device uses for nlocs windows.
int ctx_batch_windows(const xcg_ctx *c, int nlocs, int strip_len);
// Windows [off, off + n) of batch plan P, for a row-stage sub-launch.
Plan rows_subrange(Plan P, int off, int n);
void set_last_error(const char *msg);
// precision form (tc_dft.cu)
xcg_status tc_enable(xcg_ctx *c);
// Queues the reset of the tensor-core error flag on s at the start of a call
// in the precision form (or its setting, when a timeout was injected).
xcg_status tc_reset_status(xcg_ctx *c, cudaStream_t s);
void launch_tc_rows(const Plan &P, cudaStream_t s);
void launch_tc_cols(const Plan &P, cudaStream_t s);
void launch_tc_inv(const Plan &P, cudaStream_t s);
}  // namespace xcg
