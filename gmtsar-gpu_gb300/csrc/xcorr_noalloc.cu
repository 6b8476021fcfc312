// Allocation-free entry point: xcg_correlate_device_noalloc.
//
// Who needs it: code that runs inside another framework's device-memory
// budget (a deep-learning or array runtime whose caching allocator already
// owns the free memory, where a stray cudaMalloc can fail or force that
// allocator to release its cache), and code on a latency-critical stream,
// where cudaMalloc/cudaFree would synchronise the device.  Those callers pass
// inputs and outputs they allocated themselves and cannot let the library
// allocate scratch or a context.
//
// How: all scratch (the transform tables and the per-window intermediates)
// lives in one fixed array of XCG_NOALLOC_SCRATCH_BYTES bytes declared below.
// The CUDA runtime places it in device memory when the library's module is
// loaded on a device and every device that loads the library keeps it until
// the process exits.  A call that needs more than that is refused with
// XCG_ERR_TOO_LARGE.  Nothing in this file calls cudaMalloc, cudaFree or a
// library routine that allocates.
//
// On the host the array's name is only a stand-in for the device object: its
// device address is looked up with cudaGetSymbolAddress, once per device, on
// the first call made with that device current, and that address is what the
// kernels receive.  That first call therefore does set-up work and should be
// made before any stream capture starts.
//
// All calls share the array and it keeps whatever the last call left there.
// The kernels write every scratch element they later read, so nothing has to
// be cleared; two calls that overlap on the GPU (different streams, or
// different host threads) race on the array and must be serialised by the
// caller.
#include <cuda_runtime.h>
#include <math.h>
#include <stdio.h>
#include <string.h>

#include "team_fft.cuh"
#include "xcorr_gb300.h"
#include "xcorr_kernels.cuh"

static __device__ __align__(256) unsigned char g_xcg_noalloc_scratch[XCG_NOALLOC_SCRATCH_BYTES];

namespace {

constexpr int kMaxDevices = 64;
void *s_scratch_addr[kMaxDevices];   // device address of the array, per device (set up once)

// host-side table staging; thread-local so concurrent host threads do not share it
constexpr size_t kMaxTable = 32768;  // float2 entries, enough for npx/npy <= 1024, ri <= 8, factor <= 64
thread_local float2 t_tables[kMaxTable];
thread_local char t_msg[256];

size_t a256(size_t v) { return (v + 255) & ~(size_t)255; }

// Stockham pass twiddles (same construction as the context's tables).
size_t put_twiddles(float2 *dst, int n) {
    size_t k0 = 0;
    int ns = 1;
    for (int p = 0; p < xcg::fft_npasses(n); p++) {
        const int r = xcg::fft_radix(n, p);
        if (p > 0)
            for (int rr = 1; rr < r; rr++)
                for (int k = 0; k < ns; k++) {
                    const double a = -2.0 * M_PI * (double)k * rr / ((double)ns * r);
                    dst[k0++] = make_float2((float)cos(a), (float)sin(a));
                }
        ns *= r;
    }
    return k0;
}

size_t put_interp(float2 *dst, int n, int m) {
    for (int X = 0; X < m; X++)
        for (int c = 0; c < n; c++) {
            double sr = 0.0, si = 0.0;
            for (int f = 0; f < n; f++) {
                const int fp = (f < n / 2) ? f : f - n;
                const double a = -2.0 * M_PI * f * c / n + 2.0 * M_PI * fp * X / m;
                sr += cos(a);
                si += sin(a);
            }
            dst[(size_t)X * n + c] = make_float2((float)(sr / n), (float)(si / n));
        }
    return (size_t)m * n;
}

size_t put_box(float2 *dst, int n, int lo) {
    for (int k = 0; k < n; k++) {
        double sr = 0.0, si = 0.0;
        for (int c = lo; c < n - lo; c++) {
            const double a = -2.0 * M_PI * (double)k * c / n;
            sr += cos(a);
            si += sin(a);
        }
        dst[k] = make_float2((float)sr, (float)si);
    }
    return (size_t)n;
}

xcg_status fail(xcg_status st, const char *msg) {
    xcg::set_last_error(msg);
    return st;
}
xcg_status fail_msg(xcg_status st) {
    xcg::set_last_error(t_msg);
    return st;
}

}  // namespace

extern "C" xcg_status xcg_correlate_device_noalloc(const xcg_params *p,
                                                   const void *d_master, int32_t m_nx, int32_t m_ny,
                                                   const void *d_slave, int32_t s_nx, int32_t s_ny,
                                                   int32_t x_offset, int32_t y_offset, double astretcha,
                                                   const xcg_loc *d_locs, int32_t nlocs, int32_t strip_len,
                                                   xcg_result *d_results, void *stream) {
    if (!p || nlocs < 0 || strip_len < 0) return fail(XCG_ERR_ARG, "bad argument");
    if (nlocs == 0) return XCG_OK;
    if (!d_master || !d_slave || !d_locs || !d_results || m_nx <= 0 || m_ny <= 0 || s_nx <= 0 || s_ny <= 0)
        return fail(XCG_ERR_ARG, "null buffer or empty image");
    const int xs = p->xsearch, ys = p->ysearch;
    auto pow2 = [](int v) { return v > 0 && (v & (v - 1)) == 0; };
    if (!pow2(xs) || !pow2(ys) || xs < 32 || ys < 32 || xs > 256 || ys > 256)
        return fail(XCG_ERR_ARG, "xsearch/ysearch must be powers of two in 32..256");
    if (p->nx_corr != 2 * xs || p->ny_corr != 2 * ys)
        return fail(XCG_ERR_UNSUPPORTED, "nx_corr/ny_corr must be 2*xsearch/2*ysearch");
    if (!(p->ri == 1 || p->ri == 2 || p->ri == 4 || p->ri == 8)) return fail(XCG_ERR_ARG, "ri must be 1, 2, 4 or 8");
    if (p->corr_mode != 2) return fail(XCG_ERR_UNSUPPORTED, "the allocation-free entry runs the frequency-domain mode only");
    if (p->interp_flag && !(p->interp_factor == 8 || p->interp_factor == 16 || p->interp_factor == 32 ||
                            p->interp_factor == 64))
        return fail(XCG_ERR_ARG, "interp_factor must be 8, 16, 32 or 64");
    if (p->n2x != 8 || p->n2y != 8) return fail(XCG_ERR_UNSUPPORTED, "n2x = n2y = 8 only");
    if (p->format != 0 && p->format != 1) return fail(XCG_ERR_ARG, "format must be 0 or 1");

    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return fail(XCG_ERR_NO_DEVICE, "no current device");
    if (!s_scratch_addr[dev]) {        // once per device, with that device current
        void *ptr = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&ptr, g_xcg_noalloc_scratch);
        if (e != cudaSuccess || !ptr) {
            snprintf(t_msg, sizeof t_msg, "cudaGetSymbolAddress: %s", cudaGetErrorString(e));
            return fail_msg(XCG_ERR_CUDA);
        }
        s_scratch_addr[dev] = ptr;
    }
    char *base = (char *)s_scratch_addr[dev];

    xcg::Plan P;
    memset(&P, 0, sizeof P);
    P.xsearch = xs; P.ysearch = ys;
    P.npx = 4 * xs; P.npy = 4 * ys;
    P.nxc = 2 * xs; P.nyc = 2 * ys;
    P.nx_corr = 2 * xs; P.ny_corr = 2 * ys;
    P.ri = p->ri;
    P.log2ri = (p->ri == 1) ? 0 : (p->ri == 2) ? 1 : (p->ri == 4) ? 2 : 3;
    P.interp_flag = p->interp_flag;
    P.ifc = p->interp_flag ? p->interp_factor : 16;
    P.n2x = p->n2x; P.n2y = p->n2y;
    P.nx2 = P.n2x * P.ifc; P.ny2 = P.n2y * P.ifc;
    P.format = p->format;
    P.nchunks = P.npx * P.npy / 1024;
    P.qpitch = P.npx / 2 + 16;

    // tables into the thread-local staging buffer
    size_t o = 0, o_twr, o_twc, o_ph, o_bx, o_by, o_kx, o_ky;
    auto align = [&]() { o = (o + 31) & ~(size_t)31; };     // 256-byte boundaries
    o_twr = o; o += put_twiddles(t_tables + o, P.npx); align();
    o_twc = o; o += put_twiddles(t_tables + o, P.npy); align();
    o_ph = o; o += xcg::put_row_phase(t_tables + o, P.npx, P.ri); align();
    o_bx = o; o += put_box(t_tables + o, P.npx, xs); align();
    o_by = o; o += put_box(t_tables + o, P.npy, ys); align();
    o_kx = o; o += put_interp(t_tables + o, P.n2x, P.nx2); align();
    o_ky = o; o += put_interp(t_tables + o, P.n2y, P.ny2); align();
    const size_t table_bytes = o * sizeof(float2);

    // per-window scratch, same arrays as a context batch
    const size_t nw = (size_t)nlocs;
    size_t off = a256(table_bytes);
    auto take = [&](size_t per_window) { size_t r = off; off += a256(per_window * nw); return r; };
    const size_t s_zrow = take((size_t)P.npy * P.npx * sizeof(float2));
    const size_t s_amp1 = take((size_t)P.npy * P.npx * sizeof(float));
    const size_t s_amp2c = take((size_t)P.ny_corr * P.nx_corr * sizeof(float));
    const size_t s_part = take((size_t)2 * P.nchunks * sizeof(float));
    const size_t s_oob = take((size_t)P.nchunks);
    const size_t s_minmax = take((size_t)4 * P.nchunks * sizeof(float));
    const size_t s_means = take(2 * sizeof(double));
    const size_t s_qspec = take((size_t)P.nyc * P.qpitch * sizeof(float2));
    const size_t s_surf = take((size_t)P.nyc * P.nxc * sizeof(float));
    const size_t s_md = take(64 * sizeof(float));
    const size_t s_mdnext = take(64);
    const size_t s_corr0n = take(sizeof(double));
    if (o > kMaxTable || off > (size_t)XCG_NOALLOC_SCRATCH_BYTES) {
        const size_t per = (off - a256(table_bytes)) / nw;
        snprintf(t_msg, sizeof t_msg,
                 "%d windows need %zu bytes of scratch; the fixed array holds %zu bytes (at most %zu windows of this size per call)",
                 (int)nlocs, off, (size_t)XCG_NOALLOC_SCRATCH_BYTES,
                 per ? ((size_t)XCG_NOALLOC_SCRATCH_BYTES - a256(table_bytes)) / (per + 256) : 0);
        return fail_msg(XCG_ERR_TOO_LARGE);
    }

    cudaStream_t s = (cudaStream_t)stream;
    cudaError_t e = cudaMemcpyAsync(base, t_tables, table_bytes, cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess) { snprintf(t_msg, sizeof t_msg, "table upload: %s", cudaGetErrorString(e)); return fail_msg(XCG_ERR_CUDA); }
    const float2 *tb = (const float2 *)base;
    P.tw_row = tb + o_twr; P.tw_col = tb + o_twc; P.phase = tb + o_ph;
    P.box_x = tb + o_bx; P.box_y = tb + o_by; P.kx = tb + o_kx; P.ky = tb + o_ky;
    P.zrow = (float2 *)(base + s_zrow);
    P.amp1 = (float *)(base + s_amp1);
    P.amp2c = (float *)(base + s_amp2c);
    P.part = (float *)(base + s_part);
    P.oobmap = (unsigned char *)(base + s_oob);
    P.minmax = (float *)(base + s_minmax);
    P.means = (double *)(base + s_means);
    P.qspec = (float2 *)(base + s_qspec);
    P.surf = (float *)(base + s_surf);
    P.md = (float *)(base + s_md);
    P.mdnext = (unsigned char *)(base + s_mdnext);
    P.corr0n = (double *)(base + s_corr0n);

    P.single.master = d_master; P.single.m_nx = m_nx; P.single.m_ny = m_ny;
    P.single.slave = d_slave; P.single.s_nx = s_nx; P.single.s_ny = s_ny;
    P.single.x_offset = x_offset; P.single.y_offset = y_offset; P.single.astretcha = astretcha;
    P.single.strip_len = strip_len;
    P.single.nlocs = nlocs;
    P.single.out = d_results;
    P.pairs = nullptr;
    P.winref = nullptr;
    P.locs = d_locs; P.nwin = nlocs; P.win0 = 0;

    e = xcg::kernels_setup(P);
    if (e != cudaSuccess) { snprintf(t_msg, sizeof t_msg, "kernel attributes: %s", cudaGetErrorString(e)); return fail_msg(XCG_ERR_CUDA); }
    xcg::launch_rows(P, s);
    xcg::launch_cols(P, s);
    xcg::launch_peak(P, s);
    if (P.interp_flag) xcg::launch_subpix(P, s);
    e = cudaGetLastError();
    if (e != cudaSuccess) { snprintf(t_msg, sizeof t_msg, "kernel launch: %s", cudaGetErrorString(e)); return fail_msg(XCG_ERR_CUDA); }
    return XCG_OK;
}
