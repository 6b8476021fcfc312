// C ABI of the subpixel refiner (xcg_refiner_*) and the refined correlation
// path (xcg_correlate_device_refined).  No counterpart in the reference.
#include <cuda_runtime.h>
#include <math.h>
#include <string.h>

#include <string>
#include <vector>

#include "refiner.cuh"
#include "xcorr_ctx.cuh"
#include "xcorr_gb300.h"
#include "segment_rows.cuh"
#include "xcorr_kernels.cuh"

struct xcg_refiner {
    int device = 0;
    int max_batch = 0;
    int step = 0;
    void *mem = nullptr;
    float *out_int = nullptr;       // training-forward outputs for gradient/train calls
    xcg::RefPlan R;
};

namespace {
xcg_status ck(cudaError_t e, const char *what) {
    if (e == cudaSuccess) return XCG_OK;
    std::string m = std::string(what) + ": " + cudaGetErrorString(e);
    xcg::set_last_error(m.c_str());
    return e == cudaErrorMemoryAllocation ? XCG_ERR_NOMEM : XCG_ERR_CUDA;
}
#define XCG_TRY(x)                     \
    do {                               \
        xcg_status st_ = (x);          \
        if (st_ != XCG_OK) return st_; \
    } while (0)
size_t a256(size_t v) { return (v + 255) & ~(size_t)255; }
}  // namespace

extern "C" {

xcg_status xcg_refiner_create(int32_t device, int32_t max_batch, xcg_refiner **out) {
    if (!out || max_batch <= 0) return XCG_ERR_ARG;
    *out = nullptr;
    XCG_TRY(ck(cudaSetDevice(device), "cudaSetDevice"));
    xcg_refiner *r = new xcg_refiner();
    r->device = device;
    r->max_batch = max_batch;
    const size_t np = xcg::RP_N;
    size_t off = 0;
    auto take = [&](size_t bytes) { size_t o = off; off += a256(bytes); return o; };
    const size_t o_th = take(np * 4), o_m = take(np * 4), o_v = take(np * 4), o_g = take(np * 4);
    const size_t o_w2t = take(9216 * 4), o_w3t = take(9216 * 4), o_f1t = take(18432 * 4), o_bf = take(xcg::INF_PACK_BYTES);
    const size_t o_act = take((size_t)max_batch * xcg::REF_ACT * 4), o_gact = take((size_t)max_batch * xcg::REF_ACT * 4);
    const size_t o_loss = take((size_t)max_batch * 4), o_out = take((size_t)max_batch * 12);
    xcg_status st = ck(cudaMalloc(&r->mem, off), "cudaMalloc refiner");
    if (st != XCG_OK) { delete r; return st; }
    char *b = (char *)r->mem;
    r->R.theta = (float *)(b + o_th); r->R.m = (float *)(b + o_m); r->R.v = (float *)(b + o_v); r->R.grad = (float *)(b + o_g);
    r->R.w2t = (float *)(b + o_w2t); r->R.w3t = (float *)(b + o_w3t); r->R.f1t = (float *)(b + o_f1t);
    r->R.wpack = (unsigned char *)(b + o_bf);
    r->R.act = (float *)(b + o_act); r->R.grad_act = (float *)(b + o_gact);
    r->R.loss = (float *)(b + o_loss);
    r->out_int = (float *)(b + o_out);
    r->R.out = nullptr;
    if ((st = ck(cudaMemset(r->mem, 0, off), "cudaMemset")) != XCG_OK || (st = ck(xcg::ref_setup(), "refiner attributes")) != XCG_OK) {
        cudaFree(r->mem); delete r; return st;
    }
    xcg::ref_launch_derive(r->R, 0);
    *out = r;
    return ck(cudaDeviceSynchronize(), "refiner init");
}

void xcg_refiner_destroy(xcg_refiner *r) {
    if (!r) return;
    cudaSetDevice(r->device);
    cudaFree(r->mem);
    delete r;
}

xcg_status xcg_refiner_set_params(xcg_refiner *r, const float *host_params) {
    if (!r || !host_params) return XCG_ERR_ARG;
    XCG_TRY(ck(cudaSetDevice(r->device), "cudaSetDevice"));
    XCG_TRY(ck(cudaMemcpy(r->R.theta, host_params, xcg::RP_N * 4, cudaMemcpyHostToDevice), "upload parameters"));
    XCG_TRY(ck(cudaMemset(r->R.m, 0, xcg::RP_N * 4), "cudaMemset"));
    XCG_TRY(ck(cudaMemset(r->R.v, 0, xcg::RP_N * 4), "cudaMemset"));
    r->step = 0;
    xcg::ref_launch_derive(r->R, 0);
    return ck(cudaDeviceSynchronize(), "derive");
}

xcg_status xcg_refiner_get_params(xcg_refiner *r, float *host_params) {
    if (!r || !host_params) return XCG_ERR_ARG;
    XCG_TRY(ck(cudaSetDevice(r->device), "cudaSetDevice"));
    return ck(cudaMemcpy(host_params, r->R.theta, xcg::RP_N * 4, cudaMemcpyDeviceToHost), "download parameters");
}

xcg_status xcg_refiner_forward(xcg_refiner *r, const float *d_feat, int32_t n, float *d_out, int32_t tensor_cores,
                               void *stream) {
    if (!r || n < 0 || (n > 0 && (!d_feat || !d_out))) return XCG_ERR_ARG;
    if (n == 0) return XCG_OK;
    XCG_TRY(ck(cudaSetDevice(r->device), "cudaSetDevice"));
    cudaStream_t s = (cudaStream_t)stream;
    if (tensor_cores) {
        xcg::ref_launch_infer(r->R, d_feat, d_out, n, s);
    } else {
        for (int c0 = 0; c0 < n; c0 += r->max_batch) {
            xcg::RefPlan R = r->R;
            R.out = d_out + (size_t)c0 * 3;
            R.loss = nullptr;
            const int m = (n - c0 < r->max_batch) ? n - c0 : r->max_batch;
            xcg::ref_launch_fwd(R, d_feat + (size_t)c0 * 81, m, s);
        }
    }
    return ck(cudaGetLastError(), "refiner forward");
}

static void run_grad(xcg_refiner *r, const float *d_feat, const float *d_target, int n, cudaStream_t s) {
    xcg::RefPlan R = r->R;
    R.out = r->out_int;
    xcg::ref_launch_fwd(R, d_feat, n, s);
    xcg::ref_launch_bwd(R, d_target, n, s);
    xcg::ref_launch_wgrad(R, d_feat, n, s);
}

xcg_status xcg_refiner_gradient(xcg_refiner *r, const float *d_feat, const float *d_target, int32_t n,
                                float *host_grad, double *host_loss, float *host_out, void *stream) {
    if (!r || n <= 0 || n > r->max_batch || !d_feat || !d_target) return XCG_ERR_ARG;
    XCG_TRY(ck(cudaSetDevice(r->device), "cudaSetDevice"));
    cudaStream_t s = (cudaStream_t)stream;
    run_grad(r, d_feat, d_target, n, s);
    XCG_TRY(ck(cudaGetLastError(), "refiner gradient"));
    XCG_TRY(ck(cudaStreamSynchronize(s), "cudaStreamSynchronize"));
    if (host_grad) XCG_TRY(ck(cudaMemcpy(host_grad, r->R.grad, xcg::RP_N * 4, cudaMemcpyDeviceToHost), "download gradient"));
    if (host_out) XCG_TRY(ck(cudaMemcpy(host_out, r->out_int, (size_t)n * 12, cudaMemcpyDeviceToHost), "download outputs"));
    if (host_loss) {
        std::vector<float> l(n);
        XCG_TRY(ck(cudaMemcpy(l.data(), r->R.loss, (size_t)n * 4, cudaMemcpyDeviceToHost), "download loss"));
        double t = 0.0;
        for (float v : l) t += v;
        *host_loss = t / n;
    }
    return XCG_OK;
}

xcg_status xcg_refiner_train_step(xcg_refiner *r, const float *d_feat, const float *d_target, int32_t n, float lr,
                                  void *stream) {
    if (!r || n <= 0 || n > r->max_batch || !d_feat || !d_target || !(lr > 0.f)) return XCG_ERR_ARG;
    XCG_TRY(ck(cudaSetDevice(r->device), "cudaSetDevice"));
    cudaStream_t s = (cudaStream_t)stream;
    run_grad(r, d_feat, d_target, n, s);
    r->step++;
    xcg::ref_launch_adam(r->R, lr, r->step, s);
    xcg::ref_launch_derive(r->R, s);
    return ck(cudaGetLastError(), "refiner train step");
}

// The plain path with the refiner standing in for the FFT interpolation
// where it is confident (see RefDecide); the other windows get the plain
// subpixel result.  Per batch: rows, columns, peak (+ 9x9 neighbourhoods),
// refiner inference, decision, subpixel for the rest; the batches as
// xcg_correlate_device runs them.
xcg_status xcg_correlate_device_refined(xcg_ctx *c, xcg_refiner *r, const void *d_master, int32_t m_nx, int32_t m_ny,
                                        const void *d_slave, int32_t s_nx, int32_t s_ny,
                                        int32_t x_offset, int32_t y_offset, double astretcha,
                                        const xcg_loc *d_locs, int32_t nlocs, int32_t strip_len,
                                        xcg_result *d_results, float max_sigma, float max_disagree, void *stream) {
    if (!c || !r || nlocs < 0 || (nlocs > 0 && (!d_master || !d_slave || !d_locs || !d_results))) return XCG_ERR_ARG;
    if (m_nx <= 0 || m_ny <= 0 || s_nx <= 0 || s_ny <= 0 || strip_len < 0) return XCG_ERR_ARG;
    if (!c->base.interp_flag) { xcg::set_last_error("the refined path needs interp_flag = 1"); return XCG_ERR_ARG; }
    if (c->base.corr_mode != 2) { xcg::set_last_error("the refined path runs the frequency-domain mode only"); return XCG_ERR_UNSUPPORTED; }
    XCG_TRY(ck(cudaSetDevice(c->device), "cudaSetDevice"));
    memset(&c->stats, 0, sizeof c->stats);
    c->stats.scratch_bytes = c->scratch_bytes;
    if (nlocs == 0) return XCG_OK;
    if (nlocs > c->ref_cap) {
        cudaFree(c->ref_feat); cudaFree(c->ref_pred); cudaFree(c->ref_skip);
        c->ref_feat = nullptr; c->ref_pred = nullptr; c->ref_skip = nullptr; c->ref_cap = 0;
        XCG_TRY(ck(cudaMalloc(&c->ref_feat, (size_t)nlocs * 81 * 4), "cudaMalloc features"));
        XCG_TRY(ck(cudaMalloc(&c->ref_pred, (size_t)nlocs * 12), "cudaMalloc predictions"));
        XCG_TRY(ck(cudaMalloc(&c->ref_skip, (size_t)nlocs), "cudaMalloc skip"));
        c->ref_cap = nlocs;
    }
    const int bw = xcg::ctx_batch_windows(c, nlocs, strip_len);
    xcg::Plan P = xcg::ctx_plan(c);
    P.single.master = d_master; P.single.m_nx = m_nx; P.single.m_ny = m_ny;
    P.single.slave = d_slave; P.single.s_nx = s_nx; P.single.s_ny = s_ny;
    P.single.x_offset = x_offset; P.single.y_offset = y_offset; P.single.astretcha = astretcha;
    P.single.strip_len = strip_len;
    P.single.nlocs = nlocs;
    P.single.out = d_results;
    P.single.feat = c->ref_feat;
    P.pairs = nullptr;
    P.winref = nullptr;
    P.locs = d_locs;
    P.skip = nullptr;
    std::vector<int> starts;
    for (int w = 0; w < nlocs; w += bw) starts.push_back(w);
    starts.push_back(nlocs);
    // the batches run through the plain path's scheduler (two scratch slots
    // on their own streams, the planners ahead); each batch's subpixel launch
    // becomes inference with the decision, and the subpixel stage for the
    // windows the refiner left alone
    auto tail = [&](const xcg::Plan &Q, cudaStream_t ss) -> xcg_status {
        const xcg::RefDecide D{d_results + Q.win0, c->ref_skip + Q.win0, max_sigma, max_disagree};
        xcg::ref_launch_infer(r->R, c->ref_feat + (size_t)Q.win0 * 81, c->ref_pred + (size_t)Q.win0 * 3, Q.nwin, ss, &D);
        xcg::Plan Qs = Q;
        Qs.skip = c->ref_skip + Q.win0;
        xcg::launch_subpix(Qs, ss);
        c->stats.launches += 1;               // ctx_launch counts one
        return XCG_OK;
    };
    cudaStream_t s = (cudaStream_t)stream;
    c->tl_tags.clear();
    if (c->profiling == 2) XCG_TRY(xcg::tl_mark(c, s, 1));
    XCG_TRY(xcg::ctx_launch(c, P, starts.data(), (int)starts.size() - 1, s, {}, tail));
    if (c->profiling == 2) XCG_TRY(xcg::tl_finish(c, s));
    return ck(cudaGetLastError(), "refined path launch");
}

}  // extern "C"
