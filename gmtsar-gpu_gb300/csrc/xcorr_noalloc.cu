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
// library routine that allocates, and nothing copies from host memory: the
// transform tables are computed by a small kernel straight into the array,
// so every call is one run of kernels on the caller's stream.
//
// On the host the array's name is only a stand-in for the device object: its
// device address is looked up with cudaGetSymbolAddress, once per device, on
// the first call made with that device current, and that address is what the
// kernels receive.  That first call therefore does set-up work and should be
// made before any stream capture starts.
//
// All calls share the array and it keeps whatever the last call left there.
// Each call rewrites the tables, and the kernels write every scratch element
// they later read, so nothing has to be cleared; two calls that overlap on
// the GPU (different streams, or different host threads) race on the array
// and must be serialised by the caller.
#include <cuda_runtime.h>
#include <math.h>
#include <stdio.h>
#include <string.h>

#include <atomic>

#include "team_fft.cuh"
#include "xcorr_gb300.h"
#include "xcorr_kernels.cuh"

static __device__ __align__(256) unsigned char g_xcg_noalloc_scratch[XCG_NOALLOC_SCRATCH_BYTES];

namespace {

constexpr int kMaxDevices = 64;
// device address of the array, per device; written once per device (every
// writer stores the same value, and the atomic makes concurrent first calls
// from several host threads well defined)
std::atomic<void *> s_scratch_addr[kMaxDevices];

thread_local char t_msg[256];

size_t a256(size_t v) { return (v + 255) & ~(size_t)255; }

// The seven tables of a plan, as entry offsets (float2) into the start of the
// array, each on a 256-byte boundary, in the order of the Plan fields.
enum { T_TWR, T_TWC, T_PH, T_BX, T_BY, T_KX, T_KY, T_N };
struct TableSet {
    int off[T_N], len[T_N];
    int total;                 // entries up to the end of the last table
    int npx, npy, ri, xs, ys, n2x, nx2, n2y, ny2;
};

// Entries put_row_phase writes for n-point rows and factor ri.
int row_phase_len(int n, int ri) { return ri == 1 ? 1 : (ri == 2 && n <= 512) ? n : (ri - 1) * n; }

TableSet table_set(int npx, int npy, int ri, int xs, int ys, int n2x, int nx2, int n2y, int ny2) {
    TableSet t;
    const int len[T_N] = {xcg::fft_twiddle_len(npx), xcg::fft_twiddle_len(npy), row_phase_len(npx, ri), npx, npy,
                          nx2 * n2x, ny2 * n2y};
    int o = 0;
    for (int k = 0; k < T_N; k++) {
        t.off[k] = o;
        t.len[k] = len[k];
        o = (o + len[k] + 31) & ~31;
    }
    t.total = o;
    t.npx = npx; t.npy = npy; t.ri = ri; t.xs = xs; t.ys = ys;
    t.n2x = n2x; t.nx2 = nx2; t.n2y = n2y; t.ny2 = ny2;
    return t;
}

// Products and sums below are written with explicit rounding so that no
// multiply-add is fused: each entry is the double value the host-side table
// builders of the context (xcorr_api.cu, put_row_phase) compute, rounded to
// float.
__device__ double2 d_polar(double a) { return make_double2(cos(a), sin(a)); }
__device__ double2 d_cmul(double2 x, double2 y) {
    return make_double2(__dsub_rn(__dmul_rn(x.x, y.x), __dmul_rn(x.y, y.y)),
                        __dadd_rn(__dmul_rn(x.x, y.y), __dmul_rn(x.y, y.x)));
}

// Stockham pass twiddle i of an n-point FFT ([pass >= 1][r-1][k], forward sign).
__device__ float2 stockham_twiddle(int n, int i) {
    int ns = 1;
    for (int p = 0; p < xcg::fft_npasses(n); p++) {
        const int r = xcg::fft_radix(n, p);
        if (p > 0) {
            const int seg = (r - 1) * ns;
            if (i < seg) {
                const int rr = i / ns + 1, k = i % ns;
                const double a = -2.0 * M_PI * (double)k * rr / ((double)ns * r);
                return make_float2((float)cos(a), (float)sin(a));
            }
            i -= seg;
        }
        ns *= r;
    }
    return make_float2(0.f, 0.f);
}

// Entry i of the row kernel's range-interpolation table (put_row_phase).
__device__ float2 row_phase(int n, int ri, int i) {
    if (ri == 1) return make_float2(0.f, 0.f);
    if (ri == 2 && n <= 512) {
        const int r1 = n <= 256 ? n / 16 : 16;     // radix of the second pass
        const int r = i / 16 + 1, k = i % 16;
        if (r < r1) {
            const double a = -2.0 * M_PI * r * (k + 0.5) / (16.0 * r1);
            return make_float2((float)cos(a), (float)sin(a));
        }
        const int k3 = i - 16 * (r1 - 1);           // n = 512: the third pass's entries
        if (n != 512 || k3 >= 256) return make_float2(0.f, 0.f);
        const double a = -2.0 * M_PI * (k3 + 0.5) / 512.0;
        return make_float2((float)cos(a), (float)sin(a));
    }
    const int q = i / n + 1, f = i % n;
    const int fp = (f < n / 2) ? f : f - n;
    const double a = 2.0 * M_PI * fp * q / ((double)ri * n);
    return make_float2((float)(cos(a) / n), (float)(sin(a) / n));
}

// DFT bin k of the 0/1 mask with ones on [lo, n - lo) (box_spectrum).
__device__ float2 box_bin(int n, int lo, int k) {
    double2 s = make_double2(0.0, 0.0);
    for (int c = lo; c < n - lo; c++) {
        const double2 w = d_polar(-2.0 * M_PI * (double)k * c / n);
        s.x = __dadd_rn(s.x, w.x);
        s.y = __dadd_rn(s.y, w.y);
    }
    return make_float2((float)s.x, (float)s.y);
}

// Entry (X, c) of the zero-pad interpolation operator from n to m samples (interp_operator).
__device__ float2 interp_entry(int n, int m, int i) {
    const int X = i / n, c = i % n;
    double2 s = make_double2(0.0, 0.0);
    for (int f = 0; f < n; f++) {
        const int fp = (f < n / 2) ? f : f - n;
        const double2 v = d_cmul(d_polar(-2.0 * M_PI * f * c / n), d_polar(2.0 * M_PI * fp * X / m));
        s.x = __dadd_rn(s.x, v.x);
        s.y = __dadd_rn(s.y, v.y);
    }
    return make_float2((float)__ddiv_rn(s.x, (double)n), (float)__ddiv_rn(s.y, (double)n));
}

__global__ void k_noalloc_tables(TableSet t, float2 *dst) {
    for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < t.total; g += gridDim.x * blockDim.x) {
        int k = T_N - 1;
        while (k > 0 && g < t.off[k]) k--;
        const int i = g - t.off[k];
        if (i >= t.len[k]) continue;              // alignment gap
        float2 v;
        switch (k) {
            case T_TWR: v = stockham_twiddle(t.npx, i); break;
            case T_TWC: v = stockham_twiddle(t.npy, i); break;
            case T_PH: v = row_phase(t.npx, t.ri, i); break;
            case T_BX: v = box_bin(t.npx, t.xs, i); break;
            case T_BY: v = box_bin(t.npy, t.ys, i); break;
            case T_KX: v = interp_entry(t.n2x, t.nx2, i); break;
            default: v = interp_entry(t.n2y, t.ny2, i); break;
        }
        dst[g] = v;
    }
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
    if (!pow2(xs) || !pow2(ys) || xs < 16 || ys < 16 || xs > 256 || ys > 256)
        return fail(XCG_ERR_ARG, "xsearch/ysearch must be powers of two in 16..256");
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
    void *addr = s_scratch_addr[dev].load(std::memory_order_acquire);
    if (!addr) {        // once per device, with that device current
        void *ptr = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&ptr, g_xcg_noalloc_scratch);
        if (e != cudaSuccess || !ptr) {
            snprintf(t_msg, sizeof t_msg, "cudaGetSymbolAddress: %s", cudaGetErrorString(e));
            return fail_msg(XCG_ERR_CUDA);
        }
        s_scratch_addr[dev].store(ptr, std::memory_order_release);
        addr = ptr;
    }
    char *base = (char *)addr;

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
    P.corr_mode = 2;            // frequency domain, the only mode this entry runs
    P.nchunks = P.npx * P.npy / 1024;
    P.qpitch = P.npx / 2 + 16;

    // tables at the start of the array, computed on the device
    const TableSet ts = table_set(P.npx, P.npy, P.ri, xs, ys, P.n2x, P.nx2, P.n2y, P.ny2);
    const size_t table_bytes = (size_t)ts.total * sizeof(float2);

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
    if (off > (size_t)XCG_NOALLOC_SCRATCH_BYTES) {
        const size_t per = (off - a256(table_bytes)) / nw;
        snprintf(t_msg, sizeof t_msg,
                 "%d windows need %zu bytes of scratch; the fixed array holds %zu bytes (at most %zu windows of this size per call)",
                 (int)nlocs, off, (size_t)XCG_NOALLOC_SCRATCH_BYTES,
                 per ? ((size_t)XCG_NOALLOC_SCRATCH_BYTES - a256(table_bytes)) / (per + 256) : 0);
        return fail_msg(XCG_ERR_TOO_LARGE);
    }

    cudaStream_t s = (cudaStream_t)stream;
    float2 *tb = (float2 *)base;
    k_noalloc_tables<<<(ts.total + 255) / 256, 256, 0, s>>>(ts, tb);
    P.tw_row = tb + ts.off[T_TWR]; P.tw_col = tb + ts.off[T_TWC]; P.phase = tb + ts.off[T_PH];
    P.box_x = tb + ts.off[T_BX]; P.box_y = tb + ts.off[T_BY]; P.kx = tb + ts.off[T_KX]; P.ky = tb + ts.off[T_KY];
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

    cudaError_t e = xcg::kernels_setup(P);
    if (e != cudaSuccess) { snprintf(t_msg, sizeof t_msg, "kernel attributes: %s", cudaGetErrorString(e)); return fail_msg(XCG_ERR_CUDA); }
    xcg::launch_rows(P, s);
    xcg::launch_cols(P, s);
    xcg::launch_peak(P, s);
    if (P.interp_flag) xcg::launch_subpix(P, s);
    e = cudaGetLastError();
    if (e != cudaSuccess) { snprintf(t_msg, sizeof t_msg, "kernel launch: %s", cudaGetErrorString(e)); return fail_msg(XCG_ERR_CUDA); }
    return XCG_OK;
}
