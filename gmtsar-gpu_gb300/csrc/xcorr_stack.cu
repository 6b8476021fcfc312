// Stack scheduler: every window of a stack of interferogram pairs in one
// pass, bucketed by window geometry (FFT size), with strip-preserving
// batches, an optional CUDA graph of the whole stack and a batch-size
// autotuner.  No counterpart in the reference, which correlates one pair per
// process, one strip of locations at a time (xcorr.cu:322-375).
//
// Per bucket (one xsearch x ysearch geometry) the stack keeps one context
// (tables + scratch) and device copies of three window tables: the pairs
// (images, offsets, result arrays), and per window its location and its
// (pair, index) reference.  A run uploads the tables from pinned staging and
// launches the four kernels per batch; a window's results land in its own
// pair's result array.
#include <cuda_runtime.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <map>
#include <string>
#include <vector>

#include "xcorr_ctx.cuh"
#include "xcorr_gb300.h"
#include "xcorr_kernels.cuh"

namespace {

struct Bucket {
    int xs = 0, ys = 0;
    xcg_ctx *ctx = nullptr;
    int batch = 0;                       // windows per batch (0: the context's maximum)
    // pinned staging and device tables
    xcg::PairDev *h_pairs = nullptr, *d_pairs = nullptr;
    int2 *h_ref = nullptr, *d_ref = nullptr;
    xcg_loc *h_locs = nullptr, *d_locs = nullptr;
    size_t cap_pairs = 0, cap_win = 0;
    cudaEvent_t staged = nullptr;        // staging may be rewritten once this has passed
    // this run
    std::vector<int> starts;
    int nwin = 0, npairs = 0;
};

xcg_status fail(xcg_status s, const std::string &m) {
    xcg::set_last_error(m.c_str());
    return s;
}

xcg_status ck(cudaError_t e, const char *what) {
    if (e == cudaSuccess) return XCG_OK;
    std::string m = std::string(what) + ": " + cudaGetErrorString(e);
    return fail(e == cudaErrorMemoryAllocation ? XCG_ERR_NOMEM : XCG_ERR_CUDA, m);
}

#define XCG_TRY(x)                           \
    do {                                     \
        xcg_status st_ = (x);                \
        if (st_ != XCG_OK) return st_;       \
    } while (0)

uint64_t fnv1a(const void *p, size_t n, uint64_t h) {
    const unsigned char *b = (const unsigned char *)p;
    for (size_t i = 0; i < n; i++) { h ^= b[i]; h *= 1099511628211ull; }
    return h;
}

}  // namespace

struct xcg_stack {
    xcg_params common;
    int device = 0;
    std::vector<Bucket> buckets;
    std::map<std::pair<int, int>, int> index;
    int use_graph = 0;
    cudaGraphExec_t graph = nullptr;
    uint64_t graph_key = 0;
    xcg_stack_stats stats;
};

static xcg_status get_bucket(xcg_stack *st, int xs, int ys, Bucket **out) {
    auto key = std::make_pair(xs, ys);
    auto it = st->index.find(key);
    if (it != st->index.end()) { *out = &st->buckets[it->second]; return XCG_OK; }
    xcg_params p = st->common;
    p.xsearch = xs; p.ysearch = ys;
    p.nx_corr = 2 * xs; p.ny_corr = 2 * ys;
    Bucket b;
    b.xs = xs; b.ys = ys;
    XCG_TRY(xcg_create(&p, st->device, 0, &b.ctx));
    XCG_TRY(ck(cudaEventCreateWithFlags(&b.staged, cudaEventDisableTiming), "cudaEventCreate"));
    // autotuned settings for this geometry, if the cache file has them: lines
    // "npx npy ri interp_factor batch [cols_cfg peak_cfg]", the last matching
    // line winning
    const char *cache = getenv("XCG_TUNE_CACHE");
    if (cache) {
        FILE *f = fopen(cache, "r");
        if (f) {
            char line[256];
            while (fgets(line, sizeof line, f)) {
                int a, bb, r, i, bt, cc = 0, pc = 0, sh = 1;
                const int n = sscanf(line, "%d %d %d %d %d %d %d %d", &a, &bb, &r, &i, &bt, &cc, &pc, &sh);
                if (n < 5 || a != 4 * xs || bb != 4 * ys || r != p.ri || i != p.interp_factor) continue;
                b.batch = bt;
                b.ctx->base.cols_cfg = (n >= 7 && cc >= 0 && cc <= 2) ? cc : 0;
                b.ctx->base.peak_cfg = (n >= 7 && pc >= 0 && pc <= 2) ? pc : 0;
                b.ctx->base.rc = (n >= 8 && sh == 0) ? 0 : 1;
            }
            fclose(f);
        }
    }
    st->buckets.push_back(b);
    st->index[key] = (int)st->buckets.size() - 1;
    *out = &st->buckets.back();
    return XCG_OK;
}

static xcg_status reserve(Bucket &b, size_t npairs, size_t nwin) {
    if (npairs > b.cap_pairs) {
        cudaFreeHost(b.h_pairs); cudaFree(b.d_pairs);
        b.h_pairs = nullptr; b.d_pairs = nullptr; b.cap_pairs = 0;
        XCG_TRY(ck(cudaMallocHost(&b.h_pairs, npairs * sizeof(xcg::PairDev)), "cudaMallocHost pairs"));
        XCG_TRY(ck(cudaMalloc(&b.d_pairs, npairs * sizeof(xcg::PairDev)), "cudaMalloc pairs"));
        b.cap_pairs = npairs;
    }
    if (nwin > b.cap_win) {
        cudaFreeHost(b.h_ref); cudaFree(b.d_ref); cudaFreeHost(b.h_locs); cudaFree(b.d_locs);
        b.h_ref = nullptr; b.d_ref = nullptr; b.h_locs = nullptr; b.d_locs = nullptr; b.cap_win = 0;
        XCG_TRY(ck(cudaMallocHost(&b.h_ref, nwin * sizeof(int2)), "cudaMallocHost refs"));
        XCG_TRY(ck(cudaMalloc(&b.d_ref, nwin * sizeof(int2)), "cudaMalloc refs"));
        XCG_TRY(ck(cudaMallocHost(&b.h_locs, nwin * sizeof(xcg_loc)), "cudaMallocHost locs"));
        XCG_TRY(ck(cudaMalloc(&b.d_locs, nwin * sizeof(xcg_loc)), "cudaMalloc locs"));
        b.cap_win = nwin;
    }
    return XCG_OK;
}

// Group the pairs into buckets and fill each bucket's staging tables and
// strip-preserving batch boundaries (no allocation happens after this).
static xcg_status plan_run(xcg_stack *st, const xcg_pair *pairs, int npairs) {
    for (Bucket &b : st->buckets) { b.nwin = 0; b.npairs = 0; b.starts.clear(); }
    std::vector<int> which(npairs);
    std::vector<size_t> bp, bw;
    for (int i = 0; i < npairs; i++) {
        const xcg_pair &q = pairs[i];
        if (q.nlocs < 0 || (q.nlocs > 0 && (!q.d_master || !q.d_slave || !q.locs || !q.d_results)) ||
            q.m_nx <= 0 || q.m_ny <= 0 || q.s_nx <= 0 || q.s_ny <= 0 || q.strip_len < 0)
            return fail(XCG_ERR_ARG, "stack pair " + std::to_string(i) + ": bad buffers or sizes");
        Bucket *b;
        XCG_TRY(get_bucket(st, q.xsearch, q.ysearch, &b));
        which[i] = (int)(b - st->buckets.data());
    }
    bp.assign(st->buckets.size(), 0);
    bw.assign(st->buckets.size(), 0);
    for (int i = 0; i < npairs; i++) { bp[which[i]]++; bw[which[i]] += pairs[i].nlocs; }
    for (size_t k = 0; k < st->buckets.size(); k++) {
        Bucket &b = st->buckets[k];
        if (bw[k] == 0) continue;
        XCG_TRY(ck(cudaEventSynchronize(b.staged), "cudaEventSynchronize"));   // previous upload done
        XCG_TRY(reserve(b, bp[k], bw[k]));
    }
    for (int i = 0; i < npairs; i++) {
        const xcg_pair &q = pairs[i];
        Bucket &b = st->buckets[which[i]];
        const int pi = b.npairs++;
        xcg::PairDev &pd = b.h_pairs[pi];
        pd.master = q.d_master; pd.m_nx = q.m_nx; pd.m_ny = q.m_ny;
        pd.slave = q.d_slave; pd.s_nx = q.s_nx; pd.s_ny = q.s_ny;
        pd.x_offset = q.x_offset; pd.y_offset = q.y_offset; pd.astretcha = q.astretcha;
        pd.out = q.d_results; pd.nlocs = q.nlocs; pd.strip_len = q.strip_len; pd.feat = q.d_features;
        for (int l = 0; l < q.nlocs; l++) {
            b.h_locs[b.nwin + l] = q.locs[l];
            b.h_ref[b.nwin + l] = make_int2(pi, l);
        }
        b.nwin += q.nlocs;
    }
    // batches: whole strips (of each pair) up to the batch size
    for (Bucket &b : st->buckets) {
        if (b.nwin == 0) continue;
        // the row-segment planner keys pairs by a 15-bit index
        if (b.npairs >= (1 << 15)) b.ctx->base.rc = 0;
        const int cap = (b.batch > 0 && b.batch <= b.ctx->max_batch) ? b.batch : b.ctx->max_batch;
        b.starts.push_back(0);
        int bstart = 0, w = 0;
        while (w < b.nwin) {
            const int pi = b.h_ref[w].x;
            const int sl = b.h_pairs[pi].strip_len > 0 ? b.h_pairs[pi].strip_len : 1;
            int end = w + sl - (b.h_ref[w].y % sl);                 // end of this strip
            const int pend = w - b.h_ref[w].y + b.h_pairs[pi].nlocs;  // end of this pair
            if (end > pend) end = pend;
            if (w > bstart && end - bstart > cap) { b.starts.push_back(w); bstart = w; }
            while (end - bstart > cap) { bstart += cap; b.starts.push_back(bstart); }   // strip longer than a batch
            w = end;
        }
        if (b.starts.back() != b.nwin) b.starts.push_back(b.nwin);
    }
    return XCG_OK;
}

static xcg_status enqueue(xcg_stack *st, cudaStream_t s, bool capturing = false) {
    for (Bucket &b : st->buckets) {
        if (b.nwin == 0) continue;
        XCG_TRY(ck(cudaMemcpyAsync(b.d_pairs, b.h_pairs, b.npairs * sizeof(xcg::PairDev), cudaMemcpyHostToDevice, s),
                   "upload pairs"));
        XCG_TRY(ck(cudaMemcpyAsync(b.d_ref, b.h_ref, b.nwin * sizeof(int2), cudaMemcpyHostToDevice, s), "upload refs"));
        XCG_TRY(ck(cudaMemcpyAsync(b.d_locs, b.h_locs, b.nwin * sizeof(xcg_loc), cudaMemcpyHostToDevice, s),
                   "upload locs"));
        if (!capturing) XCG_TRY(ck(cudaEventRecord(b.staged, s), "cudaEventRecord"));
        xcg::Plan P = xcg::ctx_plan(b.ctx);
        memset(&P.single, 0, sizeof P.single);
        P.pairs = b.d_pairs;
        P.winref = b.d_ref;
        P.locs = b.d_locs;
        memset(&b.ctx->stats, 0, sizeof b.ctx->stats);
        XCG_TRY(xcg::ctx_launch(b.ctx, P, b.starts.data(), (int)b.starts.size() - 1, s));
        st->stats.launches += b.ctx->stats.launches;
        st->stats.batches += b.ctx->stats.batches;
    }
    return XCG_OK;
}

extern "C" {

xcg_status xcg_stack_create(const xcg_params *common, int32_t device, xcg_stack **out) {
    if (!common || !out) return XCG_ERR_ARG;
    *out = nullptr;
    if (common->corr_mode != 2) {
        xcg::set_last_error("stacks run the frequency-domain mode only");
        return XCG_ERR_UNSUPPORTED;
    }
    xcg_stack *st = new xcg_stack();
    st->common = *common;
    st->device = device;
    memset(&st->stats, 0, sizeof st->stats);
    *out = st;
    return XCG_OK;
}

void xcg_stack_destroy(xcg_stack *st) {
    if (!st) return;
    cudaSetDevice(st->device);
    if (st->graph) cudaGraphExecDestroy(st->graph);
    for (Bucket &b : st->buckets) {
        if (b.staged) { cudaEventSynchronize(b.staged); cudaEventDestroy(b.staged); }
        cudaFreeHost(b.h_pairs); cudaFree(b.d_pairs);
        cudaFreeHost(b.h_ref); cudaFree(b.d_ref);
        cudaFreeHost(b.h_locs); cudaFree(b.d_locs);
        xcg_destroy(b.ctx);
    }
    delete st;
}

void xcg_stack_set_graph(xcg_stack *st, int32_t enable) {
    if (st) st->use_graph = enable ? 1 : 0;
}

void xcg_stack_get_stats(const xcg_stack *st, xcg_stack_stats *out) {
    if (!st || !out) return;
    *out = st->stats;
    out->buckets = (int32_t)st->buckets.size();
    for (size_t k = 0; k < st->buckets.size() && k < 8; k++) {
        out->bucket_npx[k] = 4 * st->buckets[k].xs;
        out->bucket_npy[k] = 4 * st->buckets[k].ys;
        out->bucket_batch[k] = st->buckets[k].batch > 0 ? st->buckets[k].batch : st->buckets[k].ctx->max_batch;
        out->bucket_cols_cfg[k] = st->buckets[k].ctx->base.cols_cfg;
        out->bucket_peak_cfg[k] = st->buckets[k].ctx->base.peak_cfg;
        out->bucket_row_sharing[k] = st->buckets[k].ctx->base.rc;
    }
}

xcg_status xcg_stack_run(xcg_stack *st, const xcg_pair *pairs, int32_t npairs, void *stream) {
    if (!st || npairs < 0 || (npairs > 0 && !pairs)) return XCG_ERR_ARG;
    XCG_TRY(ck(cudaSetDevice(st->device), "cudaSetDevice"));
    cudaStream_t s = (cudaStream_t)stream;
    const int64_t launches0 = st->stats.launches;
    st->stats.launches = 0;
    st->stats.batches = 0;
    st->stats.windows = 0;
    for (int i = 0; i < npairs; i++) st->stats.windows += pairs[i].nlocs;
    if (st->use_graph) {
        if (!s) return fail(XCG_ERR_ARG, "graph mode needs a non-default stream");
        uint64_t key = fnv1a(pairs, sizeof(xcg_pair) * (size_t)npairs, 1469598103934665603ull);
        for (int i = 0; i < npairs; i++)
            key = fnv1a(pairs[i].locs, sizeof(xcg_loc) * (size_t)pairs[i].nlocs, key);
        if (st->graph && key == st->graph_key) {
            XCG_TRY(ck(cudaGraphLaunch(st->graph, s), "cudaGraphLaunch"));
            st->stats.graph_replays++;
            st->stats.launches = st->stats.last_graph_launches;
            st->stats.batches = st->stats.last_graph_batches;
            return XCG_OK;
        }
        XCG_TRY(ck(cudaStreamSynchronize(s), "cudaStreamSynchronize"));   // the old graph no longer reads the staging
        XCG_TRY(plan_run(st, pairs, npairs));              // allocations happen before the capture
        for (Bucket &b : st->buckets) b.ctx->profiling = 0;
        cudaGraph_t g = nullptr;
        XCG_TRY(ck(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal), "cudaStreamBeginCapture"));
        xcg_status es = enqueue(st, s, true);
        cudaError_t ce = cudaStreamEndCapture(s, &g);
        if (es != XCG_OK) { if (g) cudaGraphDestroy(g); return es; }
        XCG_TRY(ck(ce, "cudaStreamEndCapture"));
        if (st->graph) { cudaGraphExecDestroy(st->graph); st->graph = nullptr; }
        cudaError_t ie = cudaGraphInstantiate(&st->graph, g, 0);
        cudaGraphDestroy(g);
        XCG_TRY(ck(ie, "cudaGraphInstantiate"));
        st->graph_key = key;
        st->stats.last_graph_launches = st->stats.launches;
        st->stats.last_graph_batches = st->stats.batches;
        XCG_TRY(ck(cudaGraphLaunch(st->graph, s), "cudaGraphLaunch"));
        (void)launches0;
        return XCG_OK;
    }
    XCG_TRY(plan_run(st, pairs, npairs));
    return enqueue(st, s);
}

// Pick each bucket's windows per batch and launch shapes by timing
// candidates on these pairs: batch sizes first (shared row segments, default
// shapes), then the row/column stages (shared row segments, or one row stage
// per window with each of the per-window column stage's shapes: columns per
// CTA, staging depth), then the peak stage's residency, each keeping the best
// so far.
xcg_status xcg_stack_autotune(xcg_stack *st, const xcg_pair *pairs, int32_t npairs, void *stream) {
    if (!st || npairs <= 0 || !pairs) return XCG_ERR_ARG;
    XCG_TRY(ck(cudaSetDevice(st->device), "cudaSetDevice"));
    cudaStream_t s = (cudaStream_t)stream;
    const int saved_graph = st->use_graph;
    st->use_graph = 0;
    XCG_TRY(plan_run(st, pairs, npairs));                 // creates every bucket
    cudaEvent_t e0, e1;
    XCG_TRY(ck(cudaEventCreate(&e0), "cudaEventCreate"));
    XCG_TRY(ck(cudaEventCreate(&e1), "cudaEventCreate"));
    const char *cache = getenv("XCG_TUNE_CACHE");
    for (size_t k = 0; k < st->buckets.size(); k++) {
        Bucket &b = st->buckets[k];
        // only this bucket's pairs
        std::vector<xcg_pair> mine;
        int nwin = 0;
        for (int i = 0; i < npairs; i++)
            if (pairs[i].xsearch == b.xs && pairs[i].ysearch == b.ys) { mine.push_back(pairs[i]); nwin += pairs[i].nlocs; }
        if (nwin == 0) continue;
        xcg::Plan &B = b.ctx->base;
        // time the bucket's pairs with the current settings: one warm run, two timed
        auto time_it = [&](float *out) -> xcg_status {
            XCG_TRY(plan_run(st, mine.data(), (int)mine.size()));
            XCG_TRY(enqueue(st, s));
            float tot = 0.f;
            for (int rep = 0; rep < 2; rep++) {
                XCG_TRY(plan_run(st, mine.data(), (int)mine.size()));
                XCG_TRY(ck(cudaEventRecord(e0, s), "cudaEventRecord"));
                XCG_TRY(enqueue(st, s));
                XCG_TRY(ck(cudaEventRecord(e1, s), "cudaEventRecord"));
                XCG_TRY(ck(cudaEventSynchronize(e1), "cudaEventSynchronize"));
                float ms = 0.f;
                XCG_TRY(ck(cudaEventElapsedTime(&ms, e0, e1), "cudaEventElapsedTime"));
                tot += ms;
            }
            *out = tot;
            return XCG_OK;
        };
        B.cols_cfg = 0;
        B.peak_cfg = 0;
        B.rc = 1;
        std::vector<int> cands;
        for (int c : {128, 256, 512, 1024, 2048, 4096})
            if (c < b.ctx->max_batch && c < nwin) cands.push_back(c);
        cands.push_back(std::min(b.ctx->max_batch, std::max(nwin, 1)));
        float best = 1e30f;
        int bestc = cands.back();
        for (int c : cands) {
            b.batch = c;
            float t;
            XCG_TRY(time_it(&t));
            if (t < best) { best = t; bestc = c; }
        }
        b.batch = bestc;
        int best_cols = 0, best_peak = 0, best_share = 1;
        for (int cfg = 1; cfg <= 2; cfg++) {              // shared rows: one column-stage CTA per tile;
            B.cols_cfg = cfg;                             // the other persistent form
            float t;
            XCG_TRY(time_it(&t));
            if (t < best) { best = t; best_cols = cfg; }
        }
        B.rc = 0;                                         // one row stage per window, each column shape
        for (int cfg = 0; cfg <= 2; cfg++) {
            B.cols_cfg = cfg;
            float t;
            XCG_TRY(time_it(&t));
            if (t < best) { best = t; best_cols = cfg; best_share = 0; }
        }
        B.rc = best_share;
        B.cols_cfg = best_cols;
        for (int pc = 1; pc <= 2; pc++) {                 // the peak stage's residency, then 512 threads
            B.peak_cfg = pc;
            float t;
            XCG_TRY(time_it(&t));
            if (t < best) { best = t; best_peak = pc; }
        }
        B.peak_cfg = best_peak;
        if (cache) {
            FILE *f = fopen(cache, "a");
            if (f) {
                fprintf(f, "%d %d %d %d %d %d %d %d\n", 4 * b.xs, 4 * b.ys, st->common.ri, st->common.interp_factor,
                        bestc, B.cols_cfg, best_peak, best_share);
                fclose(f);
            }
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    st->use_graph = saved_graph;
    if (st->graph) { cudaGraphExecDestroy(st->graph); st->graph = nullptr; st->graph_key = 0; }
    return XCG_OK;
}

}  // extern "C"
