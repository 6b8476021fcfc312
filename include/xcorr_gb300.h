/* xcorr_gb300: GB300 (sm_103a) implementation of GMTSAR's xcorr
 * frequency-domain patch-offset estimator, behind a plain C ABI.
 *
 * One call correlates a list of locations between a master and an aligned
 * (slave) SLC image and returns, per location, the fields of the reference's
 * `struct locs` (xcorr.h:6-17) plus the reduction diagnostics.  It replaces
 * the reference's `do_correlation(struct xcorr)` (xcorr.cu:299-378) together
 * with the stages it drives: range interpolation and amplitude/demean
 * (xcorr.cu:237-292), do_freq_xcorr (do_freq_xcorr.cu:123-200),
 * do_time_int_xcorr's GPU score (do_time_int_xcorr.cu:71-100) and
 * highres_corr (highres_corr.cu:23-79).  Errors come back as status codes
 * instead of exit() (gpu_err.h:13-32).
 *
 * Threading: a context may be used by one host thread at a time.
 */
#ifndef XCORR_GB300_H
#define XCORR_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
    XCG_OK = 0,
    XCG_ERR_ARG = 1,          /* bad argument or parameter combination */
    XCG_ERR_UNSUPPORTED = 2,  /* valid for the reference but not built here */
    XCG_ERR_CUDA = 3,         /* a CUDA runtime call failed (see xcg_last_error) */
    XCG_ERR_NOMEM = 4,        /* device or pinned allocation failed */
    XCG_ERR_NO_DEVICE = 5,    /* no CUDA device / extension cannot run */
    XCG_ERR_TOO_LARGE = 6     /* a size exceeds a fixed limit */
} xcg_status;

/* Correlation parameters (struct xcorr fields, xcorr.h:19-63, with the
 * defaults of set_defaults, parse_xcorr_input.c:38-88). */
typedef struct {
    int32_t xsearch, ysearch;   /* search half-widths, powers of two in 16..256 (default 64); 16 (windows of
                                   32) in the frequency-domain mode only */
    int32_t nx_corr, ny_corr;   /* correlation window; the reference ties them to 2*xsearch, 2*ysearch */
    int32_t ri;                 /* range interpolation factor: 1 (-norange), 2 (default), 4 or 8 */
    int32_t interp_flag;        /* 1: subpixel refinement (default); 0: -nointerp */
    int32_t interp_factor;      /* subpixel factor: 8, 16 (default) or 32 */
    int32_t n2x, n2y;           /* peak neighbourhood, 8 x 8 (parse_xcorr_input.c:75-76) */
    int32_t format;             /* 0: complex int16 I/Q samples; 1: float32 real samples (-real) */
    int32_t corr_mode;          /* 2: frequency domain (default, -freq); 0: -time, 1: -time4 full-search
                                   time-domain correlation (do_time_int_xcorr.cu:146-189) */
} xcg_params;

/* A location: master pixel (range x, azimuth y) of the window centre,
 * struct locs x/y (xcorr.h:7-8) as get_locations (get_locations.c:29-40) sets them. */
typedef struct {
    int32_t x, y;
} xcg_loc;

enum { XCG_FLAG_OOB = 1,        /* part of a patch fell outside its image and was zero-filled */
       XCG_FLAG_NEXTREAD = 2,   /* the 8x8 neighbourhood used the next window's first surface value */
       XCG_FLAG_REFINED = 4,    /* xfrac/yfrac come from the subpixel refiner, not the FFT interpolation */
       XCG_FLAG_STAGE_TIMEOUT = 8 };  /* precision form: a tensor-core stage's bounded wait ran out during this
                                         call, so this window's surface may be incomplete; the result is not valid */

/* Per-location result. */
typedef struct {
    float xoff, yoff;    /* integer offset = -(peak - surface centre), struct locs xoff/yoff */
    float xfrac, yfrac;  /* subpixel fraction, struct locs xfrac/yfrac */
    float corr;          /* time-domain correlation at the integer peak (percent), struct locs corr */
    int32_t ip, jp;      /* integer peak row/column in the nyc x nxc surface */
    int32_t fip, fjp;    /* subpixel peak row/column in the interpolated surface (-1 if none) */
    int32_t flags;       /* XCG_FLAG_* */
    float fmax;          /* interpolated peak value (real part) */
    double cmax;         /* surface maximum */
    double cave;         /* the reference's surface mean (half-block sums / count) */
    double cave_true;    /* mean over the whole surface */
    double gamma;        /* time-domain correlation in double */
    double mean1, mean2; /* patch amplitude means, master and slave */
    double corr0n;       /* normalised surface value at lag (-xsearch, -ysearch) */
} xcg_result;

typedef struct xcg_ctx xcg_ctx;

/* Kernel timing/launch statistics of the most recent correlate call. */
typedef struct {
    int64_t launches;          /* kernels launched by this library */
    int32_t batches;
    int32_t batch_windows;     /* windows per batch */
    double kernel_ms[8];       /* per launch slot, summed CUDA-event time when profiling: rows, columns,
                                  peak, subpixel (frequency domain); rows, surface, peak, subpixel (-time);
                                  rows, row DFT, column DFT, product + inverse column DFT, peak, subpixel
                                  (tensor-core precision form); with shared row segments slot 0 holds
                                  the planner and the rows, and slot 7 the planner alone (device entry) */
    size_t scratch_bytes;      /* device scratch held by the context */
    int32_t nkernels;          /* launch slots used in kernel_ms */
    int32_t pad;
    int64_t row_chunks;        /* with profiling and shared row segments: 1024-sample chunks the row stage
                                  computed (2 x nchunks per window without sharing) */
    int64_t h2d_bytes;         /* xcg_correlate: bytes copied host to device (the image rows and columns
                                  the windows read, the locations); 0 for the device entries */
    int64_t d2h_bytes;         /* xcg_correlate: bytes copied device to host (the result records) */
    double host_enqueue_ms;    /* xcg_correlate: host time from entry until every copy and launch was
                                  enqueued (the rest of the call waits for the device) */
    /* timeline (xcg_set_profiling(ctx, 2)): device times, ms after the call's first device work, at which
       each mark was passed; tags: 1 start, 2 every batch joined, 3 results on the host, 100 + i image band
       i copied (host entry), 1000 + 10 b + k stage k of batch b done (the stages of kernel_ms) */
    int32_t timeline_n;
    int32_t timeline_tag[64];
    float timeline_ms[64];
} xcg_stats;

const char *xcg_status_string(xcg_status s);
/* Message of the last CUDA error seen by this thread. */
const char *xcg_last_error(void);

/* Fill p with the reference defaults (xsearch=ysearch=64, ri=2, interp 16). */
void xcg_default_params(xcg_params *p);

/* Create a context on `device`: validates p, builds the transform tables and
 * allocates scratch for up to `max_batch` windows per launch (0: automatic). */
xcg_status xcg_create(const xcg_params *p, int32_t device, int32_t max_batch, xcg_ctx **out);
void xcg_destroy(xcg_ctx *ctx);

/* Correlate `nlocs` locations; all buffers are HOST memory.
 * master: m_ny lines of m_nx samples (format 0: int16 I,Q pairs; 1: float32).
 * x_offset/y_offset: rshift/ashift of the aligned PRM; astretcha: (prf2-prf1)/prf1.
 * The slave window of location (x,y) starts at x + x_offset - npx/2,
 * y + y_offset + (int)(y*astretcha) - npy/2 (read_xcorr_data.c:65-75, xcorr.cu:332-333).
 * strip_len: locations per strip (nxl) for the one cross-window read the
 * reference makes; 0 disables it.  Synchronous.  Only the image lines the
 * windows read are copied to the device, in bands that overlap the kernels;
 * page-locked (pinned) image buffers make those copies asynchronous. */
xcg_status xcg_correlate(xcg_ctx *ctx,
                         const void *master, int32_t m_nx, int32_t m_ny,
                         const void *slave, int32_t s_nx, int32_t s_ny,
                         int32_t x_offset, int32_t y_offset, double astretcha,
                         const xcg_loc *locs, int32_t nlocs, int32_t strip_len,
                         xcg_result *results);

/* Same with DEVICE pointers (images, locations, results), enqueued on
 * `stream` (a cudaStream_t, NULL for the legacy stream); returns after the
 * launches are enqueued. */
xcg_status xcg_correlate_device(xcg_ctx *ctx,
                                const void *d_master, int32_t m_nx, int32_t m_ny,
                                const void *d_slave, int32_t s_nx, int32_t s_ny,
                                int32_t x_offset, int32_t y_offset, double astretcha,
                                const xcg_loc *d_locs, int32_t nlocs, int32_t strip_len,
                                xcg_result *d_results, void *stream);

/* Size of the fixed device array behind xcg_correlate_device_noalloc. */
#define XCG_NOALLOC_SCRATCH_BYTES (32u << 20)

/* Correlate without allocating any device memory.  No counterpart in the
 * reference; it exists for callers that must not allocate: code running
 * inside another framework's device-memory budget (whose caching allocator
 * owns the free memory, so a cudaMalloc from this library could fail or make
 * that allocator give back its cache) and code on a latency-critical stream
 * (cudaMalloc and cudaFree synchronise the device).  The caller passes device
 * buffers for the images, locations and results, as for
 * xcg_correlate_device; there is no context.  All scratch, the transform
 * tables included, comes from one fixed array of XCG_NOALLOC_SCRATCH_BYTES
 * (32 MiB) that every device loading this library holds until the process
 * exits: about 30 windows of 128x128 (256x256 FFT) or 120 windows of 64x64
 * per call.  A call needing more returns XCG_ERR_TOO_LARGE and
 * xcg_last_error() says how many windows fit.  The first call on each device
 * looks the array up (set-up work, so make it before any stream capture).
 * Every call computes its transform tables on the device into the array (no
 * copy from host memory), then runs the correlation kernels; the host does
 * not wait for the stream.  Calls share the array: two calls that overlap on
 * the GPU race and must be serialised by the caller.  Enqueued on `stream` (a
 * cudaStream_t) of the current device; returns after enqueueing. */
xcg_status xcg_correlate_device_noalloc(const xcg_params *p,
                                        const void *d_master, int32_t m_nx, int32_t m_ny,
                                        const void *d_slave, int32_t s_nx, int32_t s_ny,
                                        int32_t x_offset, int32_t y_offset, double astretcha,
                                        const xcg_loc *d_locs, int32_t nlocs, int32_t strip_len,
                                        xcg_result *d_results, void *stream);

/* ---- Stack scheduler ----
 * A stack of interferogram pairs correlated in one pass: windows are
 * bucketed by geometry (xsearch x ysearch, i.e. FFT size), each bucket runs
 * in batches of whole strips, and the whole stack can be captured into one
 * CUDA graph and replayed.  No counterpart in the reference, which runs one
 * pair per xcorr process (xcorr.cu:437-490). */
typedef struct {
    const void *d_master;  int32_t m_nx, m_ny;   /* DEVICE image, format as the stack's params */
    const void *d_slave;   int32_t s_nx, s_ny;
    int32_t x_offset, y_offset;                  /* rshift, ashift */
    double astretcha;
    const xcg_loc *locs;                         /* HOST array of nlocs locations */
    int32_t nlocs, strip_len;
    int32_t xsearch, ysearch;                    /* this pair's window geometry */
    xcg_result *d_results;                       /* DEVICE array of nlocs results */
    float *d_features;                           /* DEVICE [nlocs][81] 9x9 neighbourhoods, or NULL */
} xcg_pair;

typedef struct {
    int64_t windows, launches, graph_replays, last_graph_launches;
    int32_t batches, last_graph_batches, buckets, pad;
    int32_t bucket_npx[8], bucket_npy[8], bucket_batch[8];
    int32_t bucket_cols_cfg[8];  /* column-stage launch shape (xcg_set_launch_shapes) */
    int32_t bucket_peak_cfg[8];  /* peak-stage launch shape (xcg_set_launch_shapes) */
    int32_t bucket_row_sharing[8];  /* 1: shared row segments, 0: one row stage per window */
} xcg_stack_stats;

typedef struct xcg_stack xcg_stack;

/* common: ri, interp_flag, interp_factor, n2x/n2y, format of every pair
 * (its xsearch/ysearch are ignored: each pair carries its own). */
xcg_status xcg_stack_create(const xcg_params *common, int32_t device, xcg_stack **out);
void xcg_stack_destroy(xcg_stack *st);
/* Correlate every window of every pair; enqueued on `stream`.  The location
 * arrays are read before return; images and result arrays are used
 * asynchronously. */
xcg_status xcg_stack_run(xcg_stack *st, const xcg_pair *pairs, int32_t npairs, void *stream);
/* Graph mode: a run captures the stack's uploads and launches into a CUDA
 * graph on `stream` (not the legacy stream); later runs with identical pairs
 * and locations replay it. */
void xcg_stack_set_graph(xcg_stack *st, int32_t enable);
/* Time candidates per bucket on these pairs and keep the fastest: windows per
 * batch, then the row/column stages (shared row segments, or one row stage
 * per window with each column-stage launch shape: column pairs per CTA,
 * cp.async staging depth), then the peak stage's residency (appended to the
 * file named by XCG_TUNE_CACHE as "npx npy ri interp_factor batch cols_cfg
 * peak_cfg row_sharing", read back by new buckets). */
xcg_status xcg_stack_autotune(xcg_stack *st, const xcg_pair *pairs, int32_t npairs, void *stream);
void xcg_stack_get_stats(const xcg_stack *st, xcg_stack_stats *out);

/* Row stage of the frequency-domain FP32 path: 1 (the default) computes the
 * range interpolation, amplitudes and row spectra once per image row segment
 * that one or more windows of a batch read (windows of one column of the
 * location grid share most of their rows) and gives every window a view of
 * its rows; 0 computes them once per window, as the reference's
 * do_correlation does (xcorr.cu:330-338 with d_assign_values, :237-292).
 * Amplitudes, means and the time-domain correlation are the same bits either
 * way; the spectra differ by FP32 rounding.  The precision form and the
 * -time/-time4 modes always run the per-window row stage. */
xcg_status xcg_set_row_sharing(xcg_ctx *ctx, int32_t enable);

/* Launch shapes of this context's column and peak stages (the choices
 * xcg_stack_autotune makes per bucket).  cols_cfg with shared row segments:
 * 0 (default) persistent CTAs taking (window, column group) tiles from a
 * counter, the next tile's rows staged during the current one, in the
 * faster form for the size (up to 256-point columns the slave's column
 * spectrum kept in registers at one CTA per SM fewer); 1 one CTA per tile;
 * 2 persistent in the other form.  Without sharing: 0 128-thread CTAs, two cp.async staging groups;
 * 1 256-thread CTAs; 2 one staging group.  peak_cfg: 0 four CTAs per SM of
 * 256 threads per window (three for 512-point transforms), 1 one fewer,
 * 2 512 threads per window (transforms up to 512 points; the others take
 * 0).  Every shape gives the same bits. */
xcg_status xcg_set_launch_shapes(xcg_ctx *ctx, int32_t cols_cfg, int32_t peak_cfg);

/* Split each later call's windows into this many batches (whole strips; at
 * most the context's max_batch windows each); 0 (default) lets the library
 * choose.  Batches alternate between two scratch slots on their own streams,
 * so one batch's column and peak stages overlap the next one's row stage;
 * more batches than slots, each fitting in half a slot, run four at a time.
 * Every split gives the same bits. */
xcg_status xcg_set_batches(xcg_ctx *ctx, int32_t batches);

/* Make later xcg_correlate_device calls on this context also write, per
 * window, the 9x9 neighbourhood of the integer peak normalised by the surface
 * maximum (DEVICE [nlocs][81]; NULL stops it): the subpixel refiner's input. */
void xcg_set_features(xcg_ctx *ctx, float *d_features);

/* ---- Subpixel refiner ----
 * A small CNN (3 valid 3x3 convolutions of 32 channels, GELU, dense 64,
 * dense 3; XCG_REFINER_NPARAM FP32 parameters) that reads the 9x9
 * neighbourhood and predicts (fx, fy, s): the subpixel peak position in
 * surface pixels (the xfrac/yfrac of highres_corr.cu:67-76) and the log
 * variance of that estimate.  Trained by its own CUDA kernels (forward,
 * backward, Adam).  No counterpart in the reference. */
#define XCG_REFINER_NPARAM 37507
typedef struct xcg_refiner xcg_refiner;
/* max_batch: largest training/gradient batch (inference takes any size). */
xcg_status xcg_refiner_create(int32_t device, int32_t max_batch, xcg_refiner **out);
void xcg_refiner_destroy(xcg_refiner *r);
/* Host parameter vector, FP32, in this order: W1 [32][1][3][3], b1,
 * W2 [32][32][3][3], b2, W3, b3, F1 [64][288], c1, F2 [3][64], c2); resets Adam. */
xcg_status xcg_refiner_set_params(xcg_refiner *r, const float *host_params);
xcg_status xcg_refiner_get_params(xcg_refiner *r, float *host_params);
/* d_out [n][3]; tensor_cores = 1: BF16 tensor-core inference kernel, 0: FP32 training forward. */
xcg_status xcg_refiner_forward(xcg_refiner *r, const float *d_feat, int32_t n, float *d_out, int32_t tensor_cores,
                               void *stream);
/* Loss, parameter gradient and outputs of one batch (n <= max_batch), to host; synchronous. */
xcg_status xcg_refiner_gradient(xcg_refiner *r, const float *d_feat, const float *d_target, int32_t n,
                                float *host_grad, double *host_loss, float *host_out, void *stream);
/* One Adam step (beta 0.9/0.999, eps 1e-8) on one batch; d_target [n][2] = (fx, fy). */
xcg_status xcg_refiner_train_step(xcg_refiner *r, const float *d_feat, const float *d_target, int32_t n, float lr,
                                  void *stream);
/* The correlation with the refiner in place of the FFT interpolation where
 * its predicted standard deviation is below max_sigma and it agrees with a
 * 3-point parabola fit within max_disagree (both in surface pixels); those
 * windows carry XCG_FLAG_REFINED, the others get the plain subpixel result. */
xcg_status xcg_correlate_device_refined(xcg_ctx *ctx, xcg_refiner *r,
                                        const void *d_master, int32_t m_nx, int32_t m_ny,
                                        const void *d_slave, int32_t s_nx, int32_t s_ny,
                                        int32_t x_offset, int32_t y_offset, double astretcha,
                                        const xcg_loc *d_locs, int32_t nlocs, int32_t strip_len,
                                        xcg_result *d_results, float max_sigma, float max_disagree, void *stream);

/* Affine fit of one pair's offsets, computed on the device from the result
 * array: the step GMTSAR's fitoffset.csh performs on freq_xcorr.dat (named at
 * xcorr.cu:52; the script is not in the reference sources) to produce the PRM
 * parameters rshift/sub_int_r/stretch_r/a_stretch_r and ashift/sub_int_a/
 * stretch_a/a_stretch_a.  Offsets are taken as print_results.c:37-38 forms
 * them; locations with corr <= snr_min are left out.  Per axis the model is
 * shift + stretch*x + a_stretch*y (npar 3), without a_stretch (npar 2), or a
 * constant (npar 1).  robust_iters > 0: that many Tukey-biweight reweighted
 * passes after the least-squares one. */
typedef struct {
    double shift;          /* constant term: shift + stretch*x + a_stretch*y */
    double stretch;        /* per range pixel (x) */
    double a_stretch;      /* per azimuth line (y) */
    double sub_int;        /* shift - ishift */
    double rms;            /* weighted rms residual of the final pass */
    double weight;         /* sum of the final pass's weights */
    int32_t ishift;        /* (int) shift: rshift / ashift */
    int32_t npts;          /* locations passing snr_min */
} xcg_fit_axis;
typedef struct {
    xcg_fit_axis range, azimuth;
} xcg_fit;
/* d_out: device pointer; asynchronous on stream. */
xcg_status xcg_fit_offsets(const xcg_result *d_results, const xcg_loc *d_locs, int32_t nlocs, int32_t ri,
                           int32_t x_offset, int32_t y_offset, double astretcha, float snr_min,
                           int32_t npar_range, int32_t npar_azimuth, int32_t robust_iters, xcg_fit *d_out,
                           void *stream);

/* DFT form of the frequency-domain path: 0 (default) FP32 SIMT team FFTs; 1
 * the precision form, in which the forward row and column DFTs of the 2-D
 * correlation and the inverse column DFT of the product run as split-FP16
 * (hi + lo) tensor-core matmuls with FP32 accumulation (tcgen05), the range
 * interpolation and the inverse row transform staying FP32.  Form 1 needs
 * square windows of 64 or 128 (xsearch = ysearch = 32 or 64: 128- or
 * 256-point transforms); other shapes return XCG_ERR_UNSUPPORTED. */
xcg_status xcg_set_dft_form(xcg_ctx *ctx, int32_t form);

/* Diagnostic: the next call on this context that uses the precision form
 * proceeds as if one of its tensor-core waits had run out (the error flag the
 * stages raise is set on the host side instead of cleared at the start of the
 * call): its windows carry XCG_FLAG_STAGE_TIMEOUT and xcg_correlate returns
 * XCG_ERR_CUDA.  The call after it clears the flag again.  For tests of the
 * error path; nothing on the device times out. */
void xcg_debug_inject_stage_timeout(xcg_ctx *ctx);

/* Diagnostic: the split-FP16 tensor-core GEMM engine of the precision form
 * (tcgen05, FP32 accumulation in tensor memory) on caller matrices:
 * C (m_tiles*128 x n_total) = A (m_tiles*128 x k) * B (k x n_total), all FP32
 * row-major device arrays; (m_tiles, n_tile) one of (4, 128), (2, 144),
 * (1, 256); k a multiple of 32, n_total of n_tile.  Synchronous. */
xcg_status xcg_tc_gemm_check(int32_t m_tiles, int32_t n_tile, int32_t k, int32_t n_total,
                             const float *d_a, const float *d_b, float *d_c, void *stream);

/* Diagnostic: FP32 fused multiply-add throughput of `device` (TFLOP/s, two
 * flops per FMA), measured by a kernel of this library over tens of
 * milliseconds (CUDA events, best of five launches after a warm-up): the
 * FP32 SIMT ceiling against which the FFT kernels' rates are reported.  No
 * counterpart in the reference. */
xcg_status xcg_fp32_fma_rate(int32_t device, double *tflops);

/* 1: record CUDA events around every kernel launch, the batches run one
 * after another (adds a synchronisation at the end of each correlate call to
 * read them; kernel_ms).  2: timeline, the batches overlapping as usual, an
 * event after every stage and image band (timeline_*).  0: off. */
void xcg_set_profiling(xcg_ctx *ctx, int32_t enable);
void xcg_get_stats(const xcg_ctx *ctx, xcg_stats *out);

#ifdef __cplusplus
}
#endif
#endif /* XCORR_GB300_H */
