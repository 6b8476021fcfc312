/* Oracle for the xcorr frequency-domain patch-offset path.
 *
 * TEST INFRASTRUCTURE: a CPU restatement of the reference algorithm, used
 * only by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg, as
 * the checker.  The product (libxcorr_gb300.so and the xcorr program) never
 * links or calls it.
 *
 * Two precisions:
 *   XO_F32  follows the reference's float data path step by step (float
 *           patches and FFTs, float-product/double-sum complex multiply,
 *           FP32 block partial sums finished in double, (int) truncation,
 *           double correlation surface, powf(.,0.25f)); the timed CPU baseline.
 *   XO_F64  the same steps in double: the accuracy oracle every GPU result's
 *           error is stated against.
 * FFTs are this file's own radix-2 transforms (the reference uses cuFFT), so
 * XO_F32 agrees with the reference to rounding, not bit for bit.
 */
#ifndef XCORR_ORACLE_H
#define XCORR_ORACLE_H
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

enum { XO_F32 = 32, XO_F64 = 64 };

typedef struct {
    int npx, npy;          /* patch size; 4*xsearch x 4*ysearch (parse_xcorr_input.c:143-155) */
    int nxc, nyc;          /* correlation surface; 2*xsearch x 2*ysearch */
    int nx_corr, ny_corr;  /* time-correlation window; 2*xsearch x 2*ysearch */
    int xsearch, ysearch;
    int ri;                /* range interpolation factor, 1 = none */
    int interp_flag;       /* 1: subpixel refinement */
    int ifc;               /* interpolation factor (16) */
    int n2x, n2y;          /* peak neighbourhood (8 x 8, parse_xcorr_input.c:75-76) */
    int corr_mode;         /* 2: frequency domain (default); 0: -time, 1: -time4 full search */
} xo_params;

/* flags */
enum { XO_FLAG_OOB = 1,        /* a patch sample fell outside its image (zero-filled) */
       XO_FLAG_NEXTREAD = 2 }; /* the 8x8 neighbourhood read the next window's corr[0] */

typedef struct {
    float xoff, yoff, xfrac, yfrac, corr;   /* struct locs fields (xcorr.h:6-17) */
    int32_t ip, jp;        /* integer peak row/col in the nyc x nxc surface */
    int32_t fip, fjp;      /* fine peak row/col in the interpolated surface */
    int32_t flags;
    float fmax;            /* fine peak value (Re) */
    double cmax;           /* surface maximum */
    double cave;           /* reference mean: half-surface sum / count (reduce6, conv_ampl_demean.cu:389) */
    double cave_true;      /* mean over the whole surface */
    double gamma;          /* time-domain correlation at the integer peak */
    double mean1, mean2;   /* patch means of the amplitudes */
    double corr0n;         /* normalised surface value at (0,0) */
} xo_result;

/* Run the whole path over a list of locations (x,y pairs, master pixel
 * coordinates).  format 0: complex int16 I/Q images, 1: float32 real images.
 * strip_len > 0 groups consecutive locations into strips of that length (the
 * reference's rows of nxl locations) for the one cross-window read the
 * reference makes (conv_ampl_demean.cu:89).  nthreads <= 0: all cores. */
int xo_run(const xo_params *p, int precision, int format,
           const void *master, int m_nx, int m_ny,
           const void *slave, int s_nx, int s_ny,
           int x_offset, int y_offset, double astretcha,
           const int32_t *loc_xy, int nlocs, int strip_len, int nthreads,
           xo_result *out);

/* One location run in full, also returning the interpolated real surface
 * (ny2 x nx2 doubles) the subpixel argmax is taken over (no cross-window read). */
int xo_fine_surface(const xo_params *p, int precision, int format,
                    const void *master, int m_nx, int m_ny, const void *slave, int s_nx, int s_ny,
                    int x_offset, int y_offset, double astretcha, int x, int y,
                    double *re_out, xo_result *r);

/* Stage-level views, for kernel parity tests. */
/* One patch row range-interpolated by ri (xcorr.cu:237-250); in/out npx complex. */
void xo_range_interp_row(int precision, int npx, int ri, const double *in_c, double *out_c);
/* Amplitude patch after range interpolation, the patch mean, and the
 * (int) demeaned values (xcorr.cu:261-292); slave=1 applies the mask. */
void xo_prepare_patch(const xo_params *p, int precision, int slave, const float *patch_c,
                      float *amp, double *mean, int32_t *ints);
/* Correlation surface (nyc x nxc doubles) for one pair of complex patches. */
void xo_surface(const xo_params *p, int precision, const float *pm_c, const float *ps_c,
                double *corr, double *mean1, double *mean2);
/* Full-search time-domain surface (nyc x nxc doubles) of the -time / -time4
 * modes (p->corr_mode 0 / 1) on one window's (int) demeaned patches i1, i2
 * (npy x npx each), and the peak do_time_corr picks (xoff, yoff, corr, ip,
 * jp, cmax in r). */
void xo_time_surface(const xo_params *p, const int32_t *i1, const int32_t *i2, double *corr, xo_result *r);
/* The reference's argmax (value, index) over n elements in 2048-element blocks
 * with its exact tie-breaking; returns the flat index. */
int64_t xo_argmax_ref(const double *x, int64_t n, double *vmax);

#ifdef __cplusplus
}
#endif
#endif
