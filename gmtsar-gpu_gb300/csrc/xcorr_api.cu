// C ABI of the GB300 xcorr library (include/xcorr_gb300.h): context,
// transform tables, scratch, batching and launches.
//
// The context replaces the reference's device plan and allocations
// (d_allocate_arrays xcorr.cu:65-119, estimate_istep :161-230) and its strip
// loop (do_correlation :299-378).  Windows run in batches sized to the
// scratch, consecutive batches on two slots with their own streams; a batch
// is the row stage (with shared row segments: the planner, then the rows),
// the column stage, the peak stage and the subpixel stage.
#include <cuda_runtime.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <stdint.h>

#include <algorithm>
#include <chrono>
#include <complex>
#include <functional>
#include <string>
#include <vector>

#include "team_fft.cuh"
#include "xcorr_gb300.h"
#include "time_corr.cuh"
#include "xcorr_kernels.cuh"
#include "segment_rows.cuh"
#include "xcorr_ctx.cuh"

using cd = std::complex<double>;

// windows per row-stage sub-launch of the host-buffer entry
#ifndef XCG_ROW_SUB
#define XCG_ROW_SUB 192
#endif

namespace {

thread_local std::string g_last_error;

xcg_status cuda_fail(cudaError_t e, const char *what) {
    char buf[256];
    snprintf(buf, sizeof buf, "%s: %s", what, cudaGetErrorString(e));
    g_last_error = buf;
    return (e == cudaErrorMemoryAllocation) ? XCG_ERR_NOMEM : XCG_ERR_CUDA;
}

#define XCG_CK(call, what)                                   \
    do {                                                     \
        cudaError_t e_ = (call);                             \
        if (e_ != cudaSuccess) return cuda_fail(e_, what);   \
    } while (0)

#define XCG_TRY_ST(expr)                       \
    do {                                       \
        const xcg_status st_ = (expr);         \
        if (st_ != XCG_OK) return st_;         \
    } while (0)

bool pow2(int v) { return v > 0 && (v & (v - 1)) == 0; }
int ilog2(int v) { int l = 0; while ((1 << l) < v) l++; return l; }
size_t align256(size_t v) { return (v + 255) & ~(size_t)255; }

// Stockham pass twiddles of an n-point FFT, [pass >= 1][r-1][k], forward sign.
std::vector<float2> stockham_twiddles(int n) {
    std::vector<float2> t;
    int ns = 1;
    for (int p = 0; p < xcg::fft_npasses(n); p++) {
        const int r = xcg::fft_radix(n, p);
        if (p > 0)
            for (int rr = 1; rr < r; rr++)
                for (int k = 0; k < ns; k++) {
                    const double a = -2.0 * M_PI * (double)k * rr / ((double)ns * r);
                    t.push_back(make_float2((float)cos(a), (float)sin(a)));
                }
        ns *= r;
    }
    return t;
}

// Operator of d_fft_interpolate_1d_strip (fft_interpolate_routines.cu:76-113)
// from n samples to m = ifc*n: FFT, bins [0,n/2) kept, bins [n/2,n) moved to
// the top (frequency f-n), inverse FFT of m, scale 1/n.  op[X][c].
std::vector<float2> interp_operator(int n, int m) {
    std::vector<float2> op((size_t)m * n);
    for (int X = 0; X < m; X++)
        for (int c = 0; c < n; c++) {
            cd s = 0;
            for (int f = 0; f < n; f++) {
                const int fp = (f < n / 2) ? f : f - n;
                s += std::polar(1.0, -2.0 * M_PI * f * c / n) * std::polar(1.0, 2.0 * M_PI * fp * X / m);
            }
            s /= (double)n;
            op[(size_t)X * n + c] = make_float2((float)s.real(), (float)s.imag());
        }
    return op;
}

// DFT of the 0/1 mask along one axis (make_mask, xcorr.cu:385-401): ones on [lo, n-lo).
std::vector<float2> box_spectrum(int n, int lo) {
    std::vector<float2> b(n);
    for (int k = 0; k < n; k++) {
        cd s = 0;
        for (int c = lo; c < n - lo; c++) s += std::polar(1.0, -2.0 * M_PI * (double)k * c / n);
        b[k] = make_float2((float)s.real(), (float)s.imag());
    }
    return b;
}

}  // namespace

namespace xcg {
// lets other translation units of the library report through xcg_last_error
void set_last_error(const char *msg) { g_last_error = msg ? msg : ""; }
}  // namespace xcg



extern "C" {

const char *xcg_status_string(xcg_status s) {
    switch (s) {
        case XCG_OK: return "ok";
        case XCG_ERR_ARG: return "invalid argument";
        case XCG_ERR_UNSUPPORTED: return "unsupported parameter combination";
        case XCG_ERR_CUDA: return "CUDA error";
        case XCG_ERR_NOMEM: return "out of memory";
        case XCG_ERR_NO_DEVICE: return "no usable CUDA device";
        case XCG_ERR_TOO_LARGE: return "size exceeds a fixed limit";
    }
    return "unknown status";
}

const char *xcg_last_error(void) { return g_last_error.c_str(); }

void xcg_default_params(xcg_params *p) {
    if (!p) return;
    p->xsearch = 64; p->ysearch = 64;
    p->nx_corr = 128; p->ny_corr = 128;
    p->ri = 2;
    p->interp_flag = 1;
    p->interp_factor = 16;
    p->n2x = 8; p->n2y = 8;
    p->format = 0;
    p->corr_mode = 2;
}

static size_t per_window_bytes(const xcg::Plan &B) {
    // the arrays every form uses
    size_t common = align256(2 * sizeof(double));
    common += align256((size_t)B.nyc * B.qpitch * sizeof(float2));
    common += align256((size_t)B.nyc * B.nxc * sizeof(float));
    common += align256(64 * sizeof(float)) + align256(64) + align256(sizeof(double));
    // one row stage per window
    size_t pw = align256((size_t)B.npy * B.npx * sizeof(float2));
    pw += align256((size_t)B.npy * B.npx * sizeof(float));
    pw += align256((size_t)B.ny_corr * B.nx_corr * sizeof(float));
    pw += align256((size_t)2 * B.nchunks * sizeof(float));
    pw += align256((size_t)B.nchunks);
    pw += align256((size_t)4 * B.nchunks * sizeof(float));
    // shared row segments: at most 2 * nchunks chunks per window
    const size_t ch = (size_t)2 * B.nchunks;
    const size_t rc = align256(ch * sizeof(int4)) + align256(sizeof(int2)) + align256(sizeof(int)) +
                      align256(ch * 1024 * sizeof(float)) + align256(ch * 512 * sizeof(float2)) +
                      align256(ch * sizeof(float)) + align256(ch * sizeof(float2)) + align256(ch) +
                      align256(ch * sizeof(int)) + align256(sizeof(int)) + align256(sizeof(int));
    return common + (pw > rc ? pw : rc);      // a batch uses one of the two row-stage layouts
}

xcg_status xcg_create(const xcg_params *p, int32_t device, int32_t max_batch, xcg_ctx **out) {
    if (!p || !out) return XCG_ERR_ARG;
    *out = nullptr;
    const int xs = p->xsearch, ys = p->ysearch;
    if (!pow2(xs) || !pow2(ys) || xs < 16 || ys < 16 || xs > 256 || ys > 256) {
        g_last_error = "xsearch/ysearch must be powers of two in 16..256";
        return XCG_ERR_ARG;
    }
    if (p->nx_corr != 2 * xs || p->ny_corr != 2 * ys) {
        g_last_error = "nx_corr/ny_corr must be 2*xsearch/2*ysearch (parse_xcorr_input.c:143,153)";
        return XCG_ERR_UNSUPPORTED;
    }
    if (!(p->ri == 1 || p->ri == 2 || p->ri == 4 || p->ri == 8)) { g_last_error = "ri must be 1, 2, 4 or 8"; return XCG_ERR_ARG; }
    if (p->interp_flag && !(p->interp_factor == 8 || p->interp_factor == 16 || p->interp_factor == 32 || p->interp_factor == 64)) {
        g_last_error = "interp_factor must be 8, 16, 32 or 64";
        return XCG_ERR_ARG;
    }
    if (p->n2x != 8 || p->n2y != 8) { g_last_error = "n2x = n2y = 8 only"; return XCG_ERR_UNSUPPORTED; }
    if (p->format != 0 && p->format != 1) { g_last_error = "format must be 0 or 1"; return XCG_ERR_ARG; }
    if (p->corr_mode < 0 || p->corr_mode > 2) { g_last_error = "corr_mode must be 0 (-time), 1 (-time4) or 2"; return XCG_ERR_ARG; }
    if (p->corr_mode < 2 && (xs < 32 || ys < 32)) {
        g_last_error = "-time/-time4 need xsearch/ysearch of 32 or more (lag tiles of 32 x 64)";
        return XCG_ERR_UNSUPPORTED;
    }

    int ndev = 0;
    cudaError_t e = cudaGetDeviceCount(&ndev);
    if (e != cudaSuccess || ndev <= device || device < 0) {
        g_last_error = (e != cudaSuccess) ? cudaGetErrorString(e) : "device index out of range";
        return XCG_ERR_NO_DEVICE;
    }
    XCG_CK(cudaSetDevice(device), "cudaSetDevice");

    xcg_ctx *c = new xcg_ctx();
    c->prm = *p;
    c->device = device;
    memset(&c->stats, 0, sizeof c->stats);
    xcg::Plan &B = c->base;
    memset(&B, 0, sizeof B);
    B.xsearch = xs; B.ysearch = ys;
    B.npx = 4 * xs; B.npy = 4 * ys;
    B.nxc = 2 * xs; B.nyc = 2 * ys;
    B.nx_corr = 2 * xs; B.ny_corr = 2 * ys;
    B.ri = p->ri; B.log2ri = ilog2(p->ri);
    B.interp_flag = p->interp_flag;
    B.ifc = p->interp_flag ? p->interp_factor : 16;
    B.n2x = p->n2x; B.n2y = p->n2y;
    B.nx2 = B.n2x * B.ifc; B.ny2 = B.n2y * B.ifc;
    B.format = p->format;
    B.corr_mode = p->corr_mode;
    B.nchunks = B.npx * B.npy / 1024;
    B.qpitch = B.npx / 2 + 16;
    B.rpc = B.npx >= 1024 ? 1 : 1024 / B.npx;
    B.rc = (B.corr_mode == 2) ? 1 : 0;      // the frequency-domain mode shares row segments by default

    // tables
    std::vector<float2> tw_row = stockham_twiddles(B.npx), tw_col = stockham_twiddles(B.npy);
    std::vector<float2> phase((size_t)(B.ri > 1 ? B.ri - 1 : 1) * B.npx);
    xcg::put_row_phase(phase.data(), B.npx, B.ri);
    std::vector<float2> bx = box_spectrum(B.npx, xs), by = box_spectrum(B.npy, ys);
    std::vector<float2> kxo = interp_operator(B.n2x, B.nx2), kyo = interp_operator(B.n2y, B.ny2);
    std::vector<float2> all;
    size_t o_twr = all.size(); all.insert(all.end(), tw_row.begin(), tw_row.end()); all.resize(align256(all.size() * 8) / 8);
    size_t o_twc = all.size(); all.insert(all.end(), tw_col.begin(), tw_col.end()); all.resize(align256(all.size() * 8) / 8);
    size_t o_ph = all.size(); all.insert(all.end(), phase.begin(), phase.end()); all.resize(align256(all.size() * 8) / 8);
    size_t o_bx = all.size(); all.insert(all.end(), bx.begin(), bx.end()); all.resize(align256(all.size() * 8) / 8);
    size_t o_by = all.size(); all.insert(all.end(), by.begin(), by.end()); all.resize(align256(all.size() * 8) / 8);
    size_t o_kx = all.size(); all.insert(all.end(), kxo.begin(), kxo.end()); all.resize(align256(all.size() * 8) / 8);
    size_t o_ky = all.size(); all.insert(all.end(), kyo.begin(), kyo.end()); all.resize(align256(all.size() * 8) / 8);
    xcg_status st = XCG_OK;
#define XCG_CK_C(call, what)                                              \
    do {                                                                  \
        cudaError_t e_ = (call);                                          \
        if (e_ != cudaSuccess) { st = cuda_fail(e_, what); goto fail; }   \
    } while (0)
    {
        XCG_CK_C(cudaMalloc(&c->d_tables, all.size() * sizeof(float2)), "cudaMalloc tables");
        XCG_CK_C(cudaMemcpy(c->d_tables, all.data(), all.size() * sizeof(float2), cudaMemcpyHostToDevice), "upload tables");
        B.tw_row = c->d_tables + o_twr;
        B.tw_col = c->d_tables + o_twc;
        B.phase = c->d_tables + o_ph;
        B.box_x = c->d_tables + o_bx;
        B.box_y = c->d_tables + o_by;
        B.kx = c->d_tables + o_kx;
        B.ky = c->d_tables + o_ky;
        XCG_CK_C(xcg::kernels_setup(B), "kernel attributes");
        XCG_CK_C(xcg::segrows_setup(B), "kernel attributes");
        if (B.corr_mode < 2) XCG_CK_C(xcg::time_setup(B), "kernel attributes");

        // scratch: up to max_batch windows, at most 32 GiB or 40% of free
        // memory (shared row segments share more rows in larger batches: the
        // full frame's 512-row patches need x1.6 fewer row chunks in
        // 2000-window batches than in 500-window ones)
        const size_t pw = per_window_bytes(B);
        size_t freeb = 0, totb = 0;
        XCG_CK_C(cudaMemGetInfo(&freeb, &totb), "cudaMemGetInfo");
        size_t budget = (size_t)32 << 30;
        if (budget > freeb * 2 / 5) budget = freeb * 2 / 5;
        // at most RC_MAX_WINDOWS windows per batch: the row-segment planner's capacity
        int mb = max_batch > 0 ? std::min(max_batch, xcg::RC_MAX_WINDOWS) : xcg::RC_MAX_WINDOWS;
        if ((size_t)mb * pw * c->nslots > budget) mb = (int)(budget / (pw * c->nslots));
        if (mb < 1) { st = XCG_ERR_NOMEM; g_last_error = "not enough device memory for one window"; goto fail; }
        c->max_batch = mb;
        // one slot's arrays for mbw windows
        auto layout = [&](int mbw) {
            xcg_ctx::Layout L{};
            L.windows = mbw;
            size_t off = 0;
            auto take = [&](size_t bytes) { size_t o = off; off += align256(bytes * (size_t)mbw); return o; };
            L.means = take(2 * sizeof(double));
            L.qspec = take((size_t)B.nyc * B.qpitch * sizeof(float2));
            L.surf = take((size_t)B.nyc * B.nxc * sizeof(float));
            L.md = take(64 * sizeof(float));
            L.mdnext = take(64);
            L.corr0n = take(sizeof(double));
            // the two row-stage layouts share one region: one row stage per
            // window (per-window arrays), or shared row segments (chunk arrays);
            // a batch uses one of them, and a slot's next batch starts after it
            const size_t region = off;
            L.zrow = take((size_t)B.npy * B.npx * sizeof(float2));
            L.amp1 = take((size_t)B.npy * B.npx * sizeof(float));
            L.amp2c = take((size_t)B.ny_corr * B.nx_corr * sizeof(float));
            L.part = take((size_t)2 * B.nchunks * sizeof(float));
            L.oob = take((size_t)B.nchunks);
            L.minmax = take((size_t)4 * B.nchunks * sizeof(float));
            const size_t end_pw = off;
            off = region;
            const size_t ch = (size_t)2 * B.nchunks;        // chunks per window at most
            L.rc_desc = take(ch * sizeof(int4));
            L.rc_wch = take(sizeof(int2));
            L.rc_count = take(sizeof(int));
            L.rc_amp = take(ch * 1024 * sizeof(float));
            L.rc_spec = take(ch * 512 * sizeof(float2));
            L.rc_part = take(ch * sizeof(float));
            L.rc_minmax = take(ch * sizeof(float2));
            L.rc_oob = take(ch);
            L.rc_order = take(ch * sizeof(int));
            L.rc_band_start = take(sizeof(int));       // 9 ints: one 256-byte block at least
            L.rc_tile_next = take(sizeof(int));
            if (off < end_pw) off = end_pw;
            L.slot_bytes = align256(off);
            return L;
        };
        c->lay[0] = layout(mb);
        c->scratch_bytes = c->lay[0].slot_bytes * (size_t)c->nslots;
        if (mb >= 2) {                 // half slots: the same memory, give or take the alignment
            c->lay[1] = layout(mb / 2);
            c->scratch_bytes = std::max(c->scratch_bytes, c->lay[1].slot_bytes * (size_t)(2 * c->nslots));
        }
        XCG_CK_C(cudaMalloc(&c->d_scratch, c->scratch_bytes), "cudaMalloc scratch");
        XCG_CK_C(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking), "cudaStreamCreate");
        for (int k = 0; k < xcg_ctx::MAX_LANES; k++) {
            XCG_CK_C(cudaStreamCreateWithFlags(&c->slot_stream[k], cudaStreamNonBlocking), "cudaStreamCreate");
            XCG_CK_C(cudaEventCreateWithFlags(&c->ev_join[k], cudaEventDisableTiming), "cudaEventCreate");
        }
        XCG_CK_C(cudaEventCreateWithFlags(&c->ev_fork, cudaEventDisableTiming), "cudaEventCreate");
        XCG_CK_C(cudaStreamCreateWithFlags(&c->copy_stream, cudaStreamNonBlocking), "cudaStreamCreate");
    }
#undef XCG_CK_C
    c->stats.scratch_bytes = c->scratch_bytes;
    *out = c;
    return XCG_OK;
fail:
    xcg_destroy(c);
    return st;
}

void xcg_destroy(xcg_ctx *c) {
    if (!c) return;
    cudaSetDevice(c->device);
    if (c->stream) cudaStreamSynchronize(c->stream);
    cudaFree(c->d_tables);
    cudaFree(c->d_scratch);
    cudaFree(c->d_img[0]);
    cudaFree(c->d_img[1]);
    cudaFree(c->d_locs);
    cudaFree(c->d_res);
    if (c->h_io) cudaFreeHost(c->h_io);
    cudaFree(c->ref_feat);
    cudaFree(c->ref_pred);
    cudaFree(c->ref_skip);
    cudaFree(c->tc_prep);
    cudaFree(c->tc_err);
    for (cudaEvent_t ev : c->events) cudaEventDestroy(ev);
    for (int k = 0; k < xcg_ctx::MAX_LANES; k++) {
        if (c->slot_stream[k]) { cudaStreamSynchronize(c->slot_stream[k]); cudaStreamDestroy(c->slot_stream[k]); }
        if (c->ev_join[k]) cudaEventDestroy(c->ev_join[k]);
    }
    if (c->ev_fork) cudaEventDestroy(c->ev_fork);
    if (c->copy_stream) { cudaStreamSynchronize(c->copy_stream); cudaStreamDestroy(c->copy_stream); }
    for (cudaEvent_t ev : c->band_ready) cudaEventDestroy(ev);
    for (cudaEvent_t ev : c->tl_events) cudaEventDestroy(ev);
    if (c->stream) cudaStreamDestroy(c->stream);
    delete c;
}

xcg_status xcg_set_batches(xcg_ctx *c, int32_t batches) {
    if (!c || batches < 0) return XCG_ERR_ARG;
    c->batches_cfg = batches;
    return XCG_OK;
}

xcg_status xcg_set_row_sharing(xcg_ctx *c, int32_t enable) {
    if (!c) return XCG_ERR_ARG;
    c->base.rc = (enable && c->base.corr_mode == 2) ? 1 : 0;
    return XCG_OK;
}

xcg_status xcg_set_launch_shapes(xcg_ctx *c, int32_t cols_cfg, int32_t peak_cfg) {
    if (!c || cols_cfg < 0 || cols_cfg > 2 || peak_cfg < 0 || peak_cfg > 2) return XCG_ERR_ARG;
    c->base.cols_cfg = cols_cfg;
    c->base.peak_cfg = peak_cfg;
    return XCG_OK;
}

void xcg_set_features(xcg_ctx *c, float *d_features) {
    if (c) c->features = d_features;
}

void xcg_set_profiling(xcg_ctx *c, int32_t enable) {
    if (c) c->profiling = (enable == 2) ? 2 : (enable ? 1 : 0);
}

void xcg_get_stats(const xcg_ctx *c, xcg_stats *out) {
    if (c && out) *out = c->stats;
}

xcg_status xcg_correlate_device(xcg_ctx *c, const void *d_master, int32_t m_nx, int32_t m_ny,
                                const void *d_slave, int32_t s_nx, int32_t s_ny,
                                int32_t x_offset, int32_t y_offset, double astretcha,
                                const xcg_loc *d_locs, int32_t nlocs, int32_t strip_len,
                                xcg_result *d_results, void *stream) {
    if (!c || nlocs < 0 || (nlocs > 0 && (!d_master || !d_slave || !d_locs || !d_results))) return XCG_ERR_ARG;
    if (m_nx <= 0 || m_ny <= 0 || s_nx <= 0 || s_ny <= 0 || strip_len < 0) return XCG_ERR_ARG;
    XCG_CK(cudaSetDevice(c->device), "cudaSetDevice");
    memset(&c->stats, 0, sizeof c->stats);
    c->stats.scratch_bytes = c->scratch_bytes;
    if (nlocs == 0) return XCG_OK;
    const int bw = xcg::ctx_batch_windows(c, nlocs, strip_len);
    xcg::Plan P = xcg::ctx_plan(c);
    P.single.master = d_master; P.single.m_nx = m_nx; P.single.m_ny = m_ny;
    P.single.slave = d_slave; P.single.s_nx = s_nx; P.single.s_ny = s_ny;
    P.single.x_offset = x_offset; P.single.y_offset = y_offset; P.single.astretcha = astretcha;
    P.single.strip_len = strip_len;
    P.single.nlocs = nlocs;
    P.single.out = d_results;
    P.single.feat = c->features;
    P.pairs = nullptr;
    P.winref = nullptr;
    P.locs = d_locs;
    std::vector<int> starts;
    for (int w = 0; w < nlocs; w += bw) starts.push_back(w);
    starts.push_back(nlocs);
    c->tl_tags.clear();
    if (c->profiling == 2) XCG_TRY_ST(xcg::tl_mark(c, (cudaStream_t)stream, 1));
    XCG_TRY_ST(xcg::ctx_launch(c, P, starts.data(), (int)starts.size() - 1, (cudaStream_t)stream));
    if (c->profiling == 2) return xcg::tl_finish(c, (cudaStream_t)stream);
    return XCG_OK;
}

}  // extern "C"

namespace xcg {

Plan in_lane(const xcg_ctx *c, Plan P, int mode, int lane) {
    const xcg_ctx::Layout &L = c->lay[mode];
    char *sc = (char *)c->d_scratch + (size_t)lane * L.slot_bytes;
    P.zrow = (float2 *)(sc + L.zrow);
    P.amp1 = (float *)(sc + L.amp1);
    P.amp2c = (float *)(sc + L.amp2c);
    P.part = (float *)(sc + L.part);
    P.oobmap = (unsigned char *)(sc + L.oob);
    P.minmax = (float *)(sc + L.minmax);
    P.means = (double *)(sc + L.means);
    P.qspec = (float2 *)(sc + L.qspec);
    P.surf = (float *)(sc + L.surf);
    P.md = (float *)(sc + L.md);
    P.mdnext = (unsigned char *)(sc + L.mdnext);
    P.corr0n = (double *)(sc + L.corr0n);
    P.rc_desc = (int4 *)(sc + L.rc_desc);
    P.rc_wch = (int2 *)(sc + L.rc_wch);
    P.rc_count = (int *)(sc + L.rc_count);
    P.rc_amp = (float *)(sc + L.rc_amp);
    P.rc_spec = (float2 *)(sc + L.rc_spec);
    P.rc_part = (float *)(sc + L.rc_part);
    P.rc_minmax = (float2 *)(sc + L.rc_minmax);
    P.rc_oob = (unsigned char *)(sc + L.rc_oob);
    P.rc_order = (int *)(sc + L.rc_order);
    P.rc_band_start = (int *)(sc + L.rc_band_start);
    P.rc_tile_next = (int *)(sc + L.rc_tile_next);
    return P;
}

Plan ctx_plan(const xcg_ctx *c) { return in_lane(c, c->base, 0, 0); }

// Windows [off, off + n) of batch plan P as a plan of their own, for the row
// stage, whose kernel writes only the per-window arrays below.
Plan rows_subrange(Plan P, int off, int n) {
    const size_t o = (size_t)off;
    P.locs += off;
    if (P.winref) P.winref += off;
    P.win0 += off;
    P.nwin = n;
    P.zrow += o * P.npy * P.npx;
    P.amp1 += o * P.npy * P.npx;
    P.amp2c += o * P.ny_corr * P.nx_corr;
    P.part += o * 2 * P.nchunks;
    P.oobmap += o * P.nchunks;
    P.minmax += o * 4 * P.nchunks;
    return P;
}

int ctx_batch_windows(const xcg_ctx *c, int nlocs, int strip_len) {
    // With one row stage per window, as many windows per batch as the scratch
    // holds: one 1000-window launch per stage fills the GPU better than two
    // overlapped 500-window batches (0.758 against 0.792 ms on the 128x128
    // case); jobs larger than the scratch alternate between the two slots.
    // Two batches for jobs of 512 windows or more on the precision form (its
    // one-CTA-per-SM tensor stages: 626 K against 601 K windows/s) and on
    // shared row segments (the second batch's row stage overlaps the first's
    // column stage: 0.548 against 0.563 ms per 1000 windows of 128x128, and
    // in the host entry its image copy too: 0.732 against 0.791 ms).  On the
    // host entry a first batch of a quarter of the windows measured the same
    // as two halves (0.702 against 0.703 ms per call): the call's timeline
    // shows the device busy from the end of the first batch's row stage on.
    int bw = c->max_batch;
    if ((c->base.tc_form || c->base.rc) && nlocs >= 512 && (nlocs + 1) / 2 < bw) bw = (nlocs + 1) / 2;
    if (c->batches_cfg > 0) bw = std::min(c->max_batch, (nlocs + c->batches_cfg - 1) / c->batches_cfg);
    if (strip_len > 0 && strip_len <= bw) bw = ((bw + strip_len - 1) / strip_len) * strip_len;   // whole strips
    if (bw > c->max_batch) bw = (c->max_batch / (strip_len > 0 ? strip_len : 1)) * (strip_len > 0 ? strip_len : 1);
    if (bw < 1) bw = c->max_batch;
    return bw;
}

xcg_status ctx_launch(xcg_ctx *c, Plan P, const int *starts, int nb, cudaStream_t s, const RowsHook &rows,
                      const RowsHook &tail) {
    // launch slots: rows, columns, peak, subpixel; the precision form splits
    // the column stage into three tensor-core DFT stages
    const bool tcf = P.tc_form != 0;
    // shared row segments: frequency-domain FP32 path only (the precision
    // form and the time modes read the per-window arrays)
    if (tcf || P.corr_mode < 2) P.rc = 0;
    const bool rc = P.rc != 0;
    const int nk = (tcf ? 6 : 4) - (P.interp_flag ? 0 : 1);
    if (c->profiling == 1) {
        const size_t need = (size_t)nb * nk * 2 + (size_t)nb * 2;   // + the planners' own pair
        while (c->events.size() < need) {
            cudaEvent_t ev;
            XCG_CK(cudaEventCreate(&ev), "cudaEventCreate");
            c->events.push_back(ev);
        }
    }
    const xcg_loc *locs0 = P.locs;
    const int2 *ref0 = P.winref;
    int ei = 0, maxw = 0;
    int pe = nb * nk * 2;                  // profiling: the planner launches' events follow the slots'
    // batches alternate between the scratch slots on the slot streams (forked
    // from and joined back into s); profiling runs them in order on s so each
    // kernel's events time that kernel alone
    int widest = 0;
    for (int b = 0; b < nb; b++) {         // before anything is enqueued
        if (starts[b + 1] - starts[b] > c->max_batch) {
            set_last_error("batch larger than the context's scratch");
            return XCG_ERR_TOO_LARGE;
        }
        widest = std::max(widest, starts[b + 1] - starts[b]);
    }
    // more batches than slots, each fitting in half a slot: they run in the
    // half-slot lanes, four in flight instead of two
    const int mode = (nb > c->nslots && c->lay[1].windows > 0 && widest <= c->lay[1].windows) ? 1 : 0;
    const int lanes = mode ? 2 * c->nslots : c->nslots;
    const bool fork = nb > 1 && lanes > 1 && c->profiling != 1;
    const bool tl = c->profiling == 2;
    if (tcf) {             // a timeout of an earlier call must not be reported by this one
        const xcg_status rs = tc_reset_status(c, s);
        if (rs != XCG_OK) return rs;
    }
    if (fork) {
        XCG_CK(cudaEventRecord(c->ev_fork, s), "cudaEventRecord");
        for (int k = 0; k < lanes; k++) XCG_CK(cudaStreamWaitEvent(c->slot_stream[k], c->ev_fork, 0), "cudaStreamWaitEvent");
    }
    // shared row segments through the device entry: the first batches'
    // planners (one CTA each, reading only the locations) go first on their
    // slot streams, so a later batch's plan is ready when its rows start
    // instead of waiting for an SM behind the earlier batch's row stage
    const int npre = (rc && fork && !rows) ? std::min(nb, lanes) : 0;
    for (int b = 0; b < npre; b++) {
        Plan Q = in_lane(c, P, mode, b);
        Q.win0 = starts[b];
        Q.nwin = starts[b + 1] - starts[b];
        Q.locs = locs0 + Q.win0;
        Q.winref = ref0 ? ref0 + Q.win0 : nullptr;
        launch_rc_plan(Q, c->slot_stream[b]);
    }
    for (int b = 0; b < nb; b++) {
        const int lane = fork ? b % lanes : 0;
        cudaStream_t ss = fork ? c->slot_stream[lane] : s;
        Plan Q = in_lane(c, P, mode, lane);
        Q.win0 = starts[b];
        Q.nwin = starts[b + 1] - starts[b];
        if (Q.nwin > c->max_batch) { set_last_error("batch larger than the context's scratch"); return XCG_ERR_TOO_LARGE; }
        if (Q.nwin > maxw) maxw = Q.nwin;
        Q.locs = locs0 + Q.win0;
        Q.winref = ref0 ? ref0 + Q.win0 : nullptr;
        for (int k = 0; k < nk; k++) {
            if (c->profiling == 1) cudaEventRecord(c->events[ei++], ss);
            const bool tm = Q.corr_mode < 2;     // -time / -time4: full-search surface
            if (k == 0 && rows) {
                const xcg_status rs = rows(Q, ss);
                if (rs != XCG_OK) return rs;
            } else if (tcf) {
                switch (k) {
                    case 0: launch_rows(Q, ss); break;
                    case 1: launch_tc_rows(Q, ss); break;
                    case 2: launch_tc_cols(Q, ss); break;
                    case 3: launch_tc_inv(Q, ss); break;
                    case 4: launch_peak(Q, ss); break;
                    case 5:
                        if (tail) { const xcg_status ts = tail(Q, ss); if (ts != XCG_OK) return ts; }
                        else launch_subpix(Q, ss);
                        break;
                }
            } else {
                switch (k) {
                    case 0:
                        if (rc) {
                            if (b >= npre) {
                                if (c->profiling == 1) cudaEventRecord(c->events[pe], ss);
                                launch_rc_plan(Q, ss);
                                if (c->profiling == 1) cudaEventRecord(c->events[pe + 1], ss);
                                pe += 2;
                            }
                            launch_segrows(Q, ss);
                            c->stats.launches++;
                        } else {
                            launch_rows(Q, ss);
                        }
                        break;
                    case 1:
                        if (tm) launch_tcorr(Q, ss);
                        else if (rc) launch_cols_rc(Q, ss);
                        else launch_cols(Q, ss);
                        break;
                    case 2: if (tm) launch_tpeak(Q, ss); else launch_peak(Q, ss); break;
                    case 3:
                        if (tail) { const xcg_status ts = tail(Q, ss); if (ts != XCG_OK) return ts; }
                        else launch_subpix(Q, ss);
                        break;
                }
            }
            if (c->profiling == 1) cudaEventRecord(c->events[ei++], ss);
            if (tl) XCG_TRY_ST(tl_mark(c, ss, 1000 + 10 * b + k));
            c->stats.launches++;
        }
        if (c->profiling == 1 && rc) {     // the chunks this batch's row stage computed (profiling synchronises anyway)
            int n[2] = {0, 0};
            XCG_CK(cudaMemcpyAsync(n, Q.rc_count, 2 * sizeof(int), cudaMemcpyDeviceToHost, ss), "read chunk count");
            XCG_CK(cudaStreamSynchronize(ss), "cudaStreamSynchronize");
            c->stats.row_chunks += n[0] + n[1];
        }
    }
    if (fork) {
        for (int k = 0; k < lanes; k++) {
            XCG_CK(cudaEventRecord(c->ev_join[k], c->slot_stream[k]), "cudaEventRecord");
            XCG_CK(cudaStreamWaitEvent(s, c->ev_join[k], 0), "cudaStreamWaitEvent");
        }
    }
    if (tl) XCG_TRY_ST(tl_mark(c, s, 2));
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(e, "kernel launch");
    c->stats.batches += nb;
    c->stats.batch_windows = maxw;
    c->stats.nkernels = nk;
    if (c->profiling == 1) {
        XCG_CK(cudaStreamSynchronize(s), "cudaStreamSynchronize");
        ei = 0;
        for (int b = 0; b < nb; b++)
            for (int k = 0; k < nk; k++) {
                float ms = 0.f;
                XCG_CK(cudaEventElapsedTime(&ms, c->events[ei], c->events[ei + 1]), "cudaEventElapsedTime");
                c->stats.kernel_ms[k] += ms;
                ei += 2;
            }
        for (; ei < pe; ei += 2) {         // the planners, a part of slot 0, also on their own
            float ms = 0.f;
            XCG_CK(cudaEventElapsedTime(&ms, c->events[ei], c->events[ei + 1]), "cudaEventElapsedTime");
            c->stats.kernel_ms[7] += ms;
        }
    }
    return XCG_OK;
}

xcg_status tl_mark(xcg_ctx *c, cudaStream_t ss, int tag) {
    const size_t i = c->tl_tags.size();
    if (i >= 64) return XCG_OK;                  // the stats hold 64 marks
    if (c->tl_events.size() <= i) {
        cudaEvent_t ev;
        XCG_CK(cudaEventCreate(&ev), "cudaEventCreate");
        c->tl_events.push_back(ev);
    }
    XCG_CK(cudaEventRecord(c->tl_events[i], ss), "cudaEventRecord");
    c->tl_tags.push_back(tag);
    return XCG_OK;
}

xcg_status tl_finish(xcg_ctx *c, cudaStream_t s) {
    XCG_CK(cudaStreamSynchronize(s), "cudaStreamSynchronize");
    const int n = (int)c->tl_tags.size();
    c->stats.timeline_n = n;
    for (int i = 0; i < n; i++) {
        float ms = 0.f;
        XCG_CK(cudaEventElapsedTime(&ms, c->tl_events[0], c->tl_events[i]), "cudaEventElapsedTime");
        c->stats.timeline_tag[i] = c->tl_tags[i];
        c->stats.timeline_ms[i] = ms;
    }
    return XCG_OK;
}

}  // namespace xcg

extern "C" {

xcg_status xcg_correlate(xcg_ctx *c, const void *master, int32_t m_nx, int32_t m_ny,
                         const void *slave, int32_t s_nx, int32_t s_ny,
                         int32_t x_offset, int32_t y_offset, double astretcha,
                         const xcg_loc *locs, int32_t nlocs, int32_t strip_len,
                         xcg_result *results) {
    if (!c || nlocs < 0 || (nlocs > 0 && (!master || !slave || !locs || !results))) return XCG_ERR_ARG;
    if (m_nx <= 0 || m_ny <= 0 || s_nx <= 0 || s_ny <= 0) return XCG_ERR_ARG;
    if (nlocs == 0) return XCG_OK;
    const auto t_entry = std::chrono::steady_clock::now();
    XCG_CK(cudaSetDevice(c->device), "cudaSetDevice");
    const size_t es = 4;     // bytes per sample: an int16 I/Q pair or a float32
    const size_t need[2] = {(size_t)m_nx * m_ny * es, (size_t)s_nx * s_ny * es};
    for (int i = 0; i < 2; i++) {
        if (need[i] > c->img_bytes[i]) {
            cudaFree(c->d_img[i]);
            c->d_img[i] = nullptr;
            c->img_bytes[i] = 0;
            XCG_CK(cudaMalloc(&c->d_img[i], need[i]), "cudaMalloc image");
            c->img_bytes[i] = need[i];
        }
    }
    if (nlocs > c->io_cap) {
        cudaFree(c->d_locs); cudaFree(c->d_res); cudaFreeHost(c->h_io);
        c->d_locs = nullptr; c->d_res = nullptr; c->h_io = nullptr; c->io_cap = 0;
        XCG_CK(cudaMalloc(&c->d_locs, (size_t)nlocs * sizeof(xcg_loc)), "cudaMalloc locs");
        XCG_CK(cudaMalloc(&c->d_res, (size_t)nlocs * sizeof(xcg_result)), "cudaMalloc results");
        // pinned staging for the locations and results: both copies stay asynchronous
        XCG_CK(cudaHostAlloc(&c->h_io, (size_t)nlocs * (sizeof(xcg_loc) + sizeof(xcg_result)), cudaHostAllocDefault),
               "cudaHostAlloc");
        c->io_cap = nlocs;
    }
    xcg_loc *h_locs = reinterpret_cast<xcg_loc *>(c->h_io);
    xcg_result *h_res = reinterpret_cast<xcg_result *>(h_locs + c->io_cap);
    cudaStream_t s = c->stream;
    XCG_CK(cudaStreamSynchronize(s), "cudaStreamSynchronize");      // the staging buffer is free again
    memcpy(h_locs, locs, (size_t)nlocs * sizeof(xcg_loc));
    c->tl_tags.clear();
    if (c->profiling == 2) XCG_TRY_ST(xcg::tl_mark(c, s, 1));
    XCG_CK(cudaMemcpyAsync(c->d_locs, h_locs, (size_t)nlocs * sizeof(xcg_loc), cudaMemcpyHostToDevice, s), "copy locs");
    // Copy the images in row bands on one stream and launch the row stage of
    // each batch in sub-ranges of about XCG_ROW_SUB windows, each right after
    // the copy of the rows its windows read (master rows y - npy/2 .. y + npy/2,
    // slave rows shifted by y_offset + ishft), master band before slave band:
    // only the first band's copy is exposed; later bands copy while earlier
    // rows are transformed (a band copies in about half the time its rows'
    // kernels take).  Rows no window reads are not copied.
    // Four batches of whole strips in the half-slot lanes when they fit
    // (shared row segments): the first batch's column and peak stages start
    // while later bands are still copying.  0.640 against 0.654 ms per call
    // on 1000 windows of 128 x 128 (two batches); on the device entry, with
    // the images resident, two batches are faster (0.461 against 0.499 ms).
    int bw = xcg::ctx_batch_windows(c, nlocs, strip_len);
    if (c->batches_cfg == 0 && c->base.rc && !c->base.tc_form && c->base.corr_mode == 2 && nlocs >= 800) {
        int q = (nlocs + 3) / 4;
        if (strip_len > 0) q = ((q + strip_len - 1) / strip_len) * strip_len;
        if (q <= c->lay[1].windows) bw = q;
    }
    std::vector<int> bounds;
    for (int w = 0; w < nlocs; w += bw) bounds.push_back(w);
    bounds.push_back(nlocs);
    const int nb = (int)bounds.size() - 1;
    XCG_CK(cudaEventRecord(c->ev_fork, s), "cudaEventRecord");     // after whatever the caller queued on s
    XCG_CK(cudaStreamWaitEvent(c->copy_stream, c->ev_fork, 0), "cudaStreamWaitEvent");
    const int npy = c->base.npy;
    const int ny[2] = {m_ny, s_ny};
    const size_t rowb[2] = {(size_t)m_nx * es, (size_t)s_nx * es};
    const void *src[2] = {master, slave};
    // rows [lo, hi) of image k that windows [w0, w1) read
    auto rows_of = [&](int w0, int w1, int k, int &lo, int &hi) {
        lo = ny[k]; hi = 0;
        for (int w = w0; w < w1; w++) {
            const int y = locs[w].y;
            const int y0 = k == 0 ? y - npy / 2 : y + y_offset + (int)((double)y * astretcha) - npy / 2;
            lo = std::min(lo, std::max(y0, 0));
            hi = std::max(hi, std::min(y0 + npy, ny[k]));
        }
    };
    // columns [c0, c1) of image k that any window reads: the copies move only
    // that part of each row (the rest of the device image is never read)
    int c0[2], c1[2];
    {
        const int nx[2] = {m_nx, s_nx};
        const int npx = c->base.npx;
        for (int k = 0; k < 2; k++) {
            c0[k] = nx[k]; c1[k] = 0;
            for (int w = 0; w < nlocs; w++) {
                const int x0 = locs[w].x + (k ? x_offset : 0) - npx / 2;
                c0[k] = std::min(c0[k], std::max(x0, 0));
                c1[k] = std::max(c1[k], std::min(x0 + npx, nx[k]));
            }
            if (c1[k] <= c0[k]) { c0[k] = 0; c1[k] = 0; }      // every window outside: nothing to copy
        }
    }
    // rows [r0, r1) of image k, columns [c0, c1), on the copy stream
    auto copy_rows = [&](int k, int r0, int r1) -> xcg_status {
        if (r1 <= r0 || c1[k] <= c0[k]) return XCG_OK;
        const size_t off = (size_t)r0 * rowb[k] + (size_t)c0[k] * es;
        XCG_CK(cudaMemcpy2DAsync((char *)c->d_img[k] + off, rowb[k], (const char *)src[k] + off, rowb[k],
                                 (size_t)(c1[k] - c0[k]) * es, (size_t)(r1 - r0), cudaMemcpyHostToDevice,
                                 c->copy_stream),
               k ? "copy slave" : "copy master");
        c->stats.h2d_bytes += (int64_t)(c1[k] - c0[k]) * (int64_t)es * (r1 - r0);
        return XCG_OK;
    };
    int done[2];
    for (int k = 0; k < 2; k++) {
        int lo, hi;
        rows_of(0, nlocs, k, lo, hi);
        done[k] = lo;            // bands grow from the first row any window reads
    }
    size_t nev = 0;
    auto rows_hook = [&](const xcg::Plan &Q, cudaStream_t ss) -> xcg_status {
        if (Q.rc) {
            // shared row segments: the planner (which reads only the
            // locations) orders the batch's chunks by row band of each image;
            // band b's rows are copied, then its row-stage launch runs, so
            // only the first band's copy is exposed
            int lo[2], hi[2];
            for (int k = 0; k < 2; k++) rows_of(Q.win0, Q.win0 + Q.nwin, k, lo[k], hi[k]);
            xcg::Plan Qb = Q;
            const int nb = std::max(1, std::min(8, Q.nwin / 128));
            Qb.rc_nbands = nb;
            for (int b = 0; b < nb; b++)
                for (int k = 0; k < 2; k++)
                    Qb.rc_band_end[k][b] = (b == nb - 1) ? INT32_MAX
                                                         : lo[k] + (int)((long long)(hi[k] - lo[k]) * (b + 1) / nb);
            xcg::launch_rc_plan(Qb, ss);
            for (int b = 0; b < nb; b++) {
                for (int k = 0; k < 2; k++) {
                    const int end = std::min(hi[k], Qb.rc_band_end[k][b]);
                    if (end > done[k]) {
                        const xcg_status cs = copy_rows(k, done[k], end);
                        if (cs != XCG_OK) return cs;
                        done[k] = end;
                    }
                }
                if (c->band_ready.size() <= nev) {
                    cudaEvent_t ev;
                    XCG_CK(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming), "cudaEventCreate");
                    c->band_ready.push_back(ev);
                }
                XCG_CK(cudaEventRecord(c->band_ready[nev], c->copy_stream), "cudaEventRecord");
                XCG_CK(cudaStreamWaitEvent(ss, c->band_ready[nev], 0), "cudaStreamWaitEvent");
                if (c->profiling == 2) XCG_TRY_ST(xcg::tl_mark(c, c->copy_stream, 100 + (int)nev));
                nev++;
                Qb.rc_band = b;
                xcg::launch_segrows(Qb, ss);
            }
            c->stats.launches += nb;          // the planner and the band launches; ctx_launch counts one
            return XCG_OK;
        }
        const int nsub = std::max(1, (Q.nwin + XCG_ROW_SUB / 2) / XCG_ROW_SUB);
        for (int j = 0; j < nsub; j++) {
            const int o0 = (int)((long long)Q.nwin * j / nsub), o1 = (int)((long long)Q.nwin * (j + 1) / nsub);
            if (o1 <= o0) continue;
            for (int k = 0; k < 2; k++) {
                int lo, hi;
                rows_of(Q.win0 + o0, Q.win0 + o1, k, lo, hi);
                if (hi > done[k]) {
                    const xcg_status cs = copy_rows(k, done[k], hi);
                    if (cs != XCG_OK) return cs;
                    done[k] = hi;
                }
            }
            if (c->band_ready.size() <= nev) {
                cudaEvent_t ev;
                XCG_CK(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming), "cudaEventCreate");
                c->band_ready.push_back(ev);
            }
            XCG_CK(cudaEventRecord(c->band_ready[nev], c->copy_stream), "cudaEventRecord");
            XCG_CK(cudaStreamWaitEvent(ss, c->band_ready[nev], 0), "cudaStreamWaitEvent");
            if (c->profiling == 2) XCG_TRY_ST(xcg::tl_mark(c, c->copy_stream, 100 + (int)nev));
            nev++;
            xcg::launch_rows(xcg::rows_subrange(Q, o0, o1 - o0), ss);
        }
        c->stats.launches += nsub - 1;       // ctx_launch counts the row stage once
        return XCG_OK;
    };
    memset(&c->stats, 0, sizeof c->stats);
    c->stats.scratch_bytes = c->scratch_bytes;
    c->stats.h2d_bytes = (int64_t)nlocs * (int64_t)sizeof(xcg_loc);
    c->stats.d2h_bytes = (int64_t)nlocs * (int64_t)sizeof(xcg_result);
    xcg::Plan P = xcg::ctx_plan(c);
    P.single.master = c->d_img[0]; P.single.m_nx = m_nx; P.single.m_ny = m_ny;
    P.single.slave = c->d_img[1]; P.single.s_nx = s_nx; P.single.s_ny = s_ny;
    P.single.x_offset = x_offset; P.single.y_offset = y_offset; P.single.astretcha = astretcha;
    P.single.strip_len = strip_len;
    P.single.nlocs = nlocs;
    P.single.out = c->d_res;
    P.single.feat = c->features;
    P.pairs = nullptr;
    P.winref = nullptr;
    P.locs = c->d_locs;
    xcg_status st = xcg::ctx_launch(c, P, bounds.data(), nb, s, rows_hook);
    if (st != XCG_OK) {
        // band copies already queued read the caller's images: let them end
        // before the caller may free those buffers
        cudaStreamSynchronize(c->copy_stream);
        return st;
    }
    XCG_CK(cudaMemcpyAsync(h_res, c->d_res, (size_t)nlocs * sizeof(xcg_result), cudaMemcpyDeviceToHost, s), "copy results");
    if (c->profiling == 2) XCG_TRY_ST(xcg::tl_mark(c, s, 3));
    c->stats.host_enqueue_ms =
        std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t_entry).count();
    XCG_CK(cudaStreamSynchronize(s), "cudaStreamSynchronize");
    if (c->profiling == 2) XCG_TRY_ST(xcg::tl_finish(c, s));
    if (c->base.tc_form && c->tc_err) {     // a tensor-core wait that ran out leaves its block unwritten
        int herr = 0;
        XCG_CK(cudaMemcpy(&herr, c->tc_err, sizeof(int), cudaMemcpyDeviceToHost), "read tensor-core status");
        if (herr) { xcg::set_last_error("tensor-core stage: a wait ran out"); return XCG_ERR_CUDA; }
    }
    memcpy(results, h_res, (size_t)nlocs * sizeof(xcg_result));
    return XCG_OK;
}

}  // extern "C"
