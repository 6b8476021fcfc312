/* Oracle for the xcorr frequency-domain path: CPU restatement of the
 * reference algorithm (test infrastructure only; see xcorr_oracle.h).
 *
 * Reference pipeline per location (reference file:line):
 *   patch cut            xcorr.cu:330-338, read_xcorr_data.c:52-85
 *   range interpolation  xcorr.cu:237-250, fft_interpolate_routines.cu:76-113
 *   amplitude/mean/mask  xcorr.cu:261-292, conv_ampl_demean.cu:98-139,703-726
 *   2-D FFT correlation  do_freq_xcorr.cu:26-117
 *   peak + mean          conv_ampl_demean.cu:642-675 (reduce6/6b :350-554)
 *   time correlation     do_freq_xcorr.cu:150-178, do_time_int_xcorr.cu:19-100
 *   normalisation        do_freq_xcorr.cu:181-199, conv_ampl_demean.cu:50-68
 *   subpixel             highres_corr.cu:23-79, conv_ampl_demean.cu:75-95,227-346,730-756,
 *                        fft_interpolate_routines.cu:19-147
 * Build with -ffp-contract=off so both hosts (x86-64 and aarch64) round alike.
 */
#include "xcorr_oracle.h"
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define XCAT_(a, b) a##_##b
#define XCAT(a, b) XCAT_(a, b)

/* ---- twiddle tables: cos and -sin of 2*pi*k/n in double, plus float copies ---- */
typedef struct {
    int n;
    int *rev;
    double *cd, *sd;
    float *cf, *sf;
} xo_tab;

static xo_tab *g_tabs[31];

static int ilog2i(int n) { int l = 0; while ((1 << l) < n) l++; return l; }

static const xo_tab *tab_get(int n)
{
    int lg = ilog2i(n);
    if (g_tabs[lg]) return g_tabs[lg];
#ifdef _OPENMP
#pragma omp critical(xo_tab_build)
#endif
    {
        if (!g_tabs[lg]) {
            xo_tab *t = (xo_tab *)calloc(1, sizeof(xo_tab));
            t->n = n;
            t->rev = (int *)malloc(sizeof(int) * (size_t)n);
            t->cd = (double *)malloc(sizeof(double) * (size_t)(n / 2 + 1));
            t->sd = (double *)malloc(sizeof(double) * (size_t)(n / 2 + 1));
            t->cf = (float *)malloc(sizeof(float) * (size_t)(n / 2 + 1));
            t->sf = (float *)malloc(sizeof(float) * (size_t)(n / 2 + 1));
            for (int i = 0; i < n; i++) {
                int r = 0;
                for (int b = 0; b < lg; b++) if (i & (1 << b)) r |= 1 << (lg - 1 - b);
                t->rev[i] = r;
            }
            for (int k = 0; k <= n / 2; k++) {
                double a = 2.0 * M_PI * (double)k / (double)n;
                t->cd[k] = cos(a);
                t->sd[k] = -sin(a);
                t->cf[k] = (float)t->cd[k];
                t->sf[k] = (float)t->sd[k];
            }
            g_tabs[lg] = t;
        }
    }
    return g_tabs[lg];
}

static const float *tab_cos_f32(const xo_tab *t) { return t->cf; }
static const float *tab_sin_f32(const xo_tab *t) { return t->sf; }
static const double *tab_cos_f64(const xo_tab *t) { return t->cd; }
static const double *tab_sin_f64(const xo_tab *t) { return t->sd; }

/* ---- reference reductions ---- */

static unsigned bitrev11(unsigned e)
{
    unsigned r = 0;
    for (int b = 0; b < 11; b++) if (e & (1u << b)) r |= 1u << (10 - b);
    return r;
}

/* argmax with the tie-breaking of reduce6b/reduce6bC (conv_ampl_demean.cu:227-346,
 * 434-554, launched with 1024 threads over 2048-element blocks) and the host
 * finish (h_reduce_strip :655-673, h_reduceCr_strip :739-754).  Each thread
 * starts from value 0 at its first element and takes a later element only if
 * strictly greater; the shared-memory and shuffle tree keeps the lower thread
 * unless the upper one is strictly greater; the host keeps the earliest block
 * unless a later one is strictly greater.  Equivalently: the winner has the
 * largest effective value, ties going to the smallest key
 * (block, bit-reversed 11-bit local index), where the effective value of an
 * element that is not > 0 is 0 in the first half of its block and "never
 * wins" in the second half (NaN included). */
int64_t xo_argmax_ref(const double *x, int64_t n, double *vmax)
{
    int64_t best = 0;
    double bv = -2.0;
    unsigned bkey = 0xffffffffu;
    int64_t bbest = -1;
    for (int64_t b0 = 0; b0 < n; b0 += 2048) {
        double blk_v = -2.0;
        unsigned blk_key = 0xffffffffu;
        int64_t blk_i = b0;
        int64_t len = (n - b0 < 2048) ? n - b0 : 2048;
        for (int64_t e = 0; e < len; e++) {
            double v = x[b0 + e];
            double eff = (v > 0.0) ? v : ((e < 1024) ? 0.0 : -1.0);
            unsigned key = bitrev11((unsigned)e);
            if (eff > blk_v || (eff == blk_v && key < blk_key)) { blk_v = eff; blk_key = key; blk_i = b0 + e; }
        }
        if (bbest < 0 || blk_v > bv) { bv = blk_v; bbest = blk_i; }
    }
    best = bbest;
    (void)bkey;
    if (vmax) *vmax = bv;
    return best;
}

/* Sum of reduce6<double,1024> (conv_ampl_demean.cu:350-429) as launched by
 * h_reduce_strip (:644-651): thread t of each 2048-element block adds
 * x[t] + x[t+1024], but the block has no 512-stride step, so threads 512..1023
 * are dropped; the tree then halves 256,128,64,32 and shuffles 16..1.  Block
 * sums are added in order in double (:666). */
static double half_block_sum(const double *x)
{
    double s[512];
    for (int t = 0; t < 512; t++) s[t] = x[t] + x[t + 1024];
    for (int st = 256; st >= 1; st >>= 1)
        for (int t = 0; t < st; t++) s[t] = s[t] + s[t + st];
    return s[0];
}

/* Surfaces that are a whole number of 2048-element blocks (every window of
 * 64 or more) are summed block by block as above.  A 32 x 32 surface (1024
 * elements) is less than one block: reduce6 zero-pads the elements past n,
 * but h_reduce_strip computes its block count as n / 2048 = 0 and launches
 * nothing (conv_ampl_demean.cu:645,660), so the reference has no value
 * there; this restatement takes the zero-padded block reduce6 would have
 * reduced, the sum of elements [0, 512) of the partial block. */
static double xo_half_sum_ref(const double *x, int64_t n)
{
    double acc = 0.0;
    int64_t b0 = 0;
    for (; b0 + 2048 <= n; b0 += 2048) acc += half_block_sum(x + b0);
    if (b0 < n) {
        double pad[2048] = {0};
        memcpy(pad, x + b0, sizeof(double) * (size_t)(n - b0));
        acc += half_block_sum(pad);
    }
    return acc;
}

/* Full-search time-domain correlation surface of the -time / -time4 modes
 * (do_time_corr, do_time_int_xcorr.cu:146-189): for every lag (ioff, joff) in
 * [-ysearch, ysearch) x [-xsearch, xsearch), row ic = ioff + ysearch, column
 * jc = joff + xsearch, calc_time_corr (:30-68, mode 0) or calc_time_corr_hat
 * (:103-144, mode 1) over the ny_corr x nx_corr window of the (int) demeaned
 * amplitudes.  The long long sums are kept modulo 2^64, which is what the
 * reference's signed arithmetic does on its platform when the fourth powers
 * overflow. */
static void time_surface(const xo_params *p, const int32_t *i1, const int32_t *i2, double *corr)
{
    const int N = p->npx;
    for (int ic = 0; ic < p->nyc; ic++) {
        const int ioff = ic - p->ysearch;
        for (int jc = 0; jc < p->nxc; jc++) {
            const int joff = jc - p->xsearch;
            uint64_t num = 0, d1 = 0, d2 = 0;
            for (int y = 0; y < p->ny_corr; y++) {
                const int32_t *ar = i1 + (size_t)(p->ysearch + y + ioff) * N + joff + p->xsearch;
                const int32_t *br = i2 + (size_t)(p->ysearch + y) * N + p->xsearch;
                for (int x = 0; x < p->nx_corr; x++) {
                    const uint64_t a = (uint64_t)(int64_t)ar[x], b = (uint64_t)(int64_t)br[x];
                    if (p->corr_mode == 0) {
                        num += a * b; d1 += a * a; d2 += b * b;
                    } else {
                        num += a * a * b * b; d1 += a * a * a * a; d2 += b * b * b * b;
                    }
                }
            }
            const double dd = 1.0 * (double)(int64_t)d1 * (double)(int64_t)d2;
            double g;
            if (p->corr_mode == 0) {
                const double den = sqrt(dd);
                g = (den == 0.0) ? 0.0 : 100.0 * fabs((double)(int64_t)num / den);
            } else {
                const double den = (double)sqrtl((long double)dd);
                g = (den == 0.0) ? 0.0 : fabs((double)(int64_t)num / den);
                g = (g <= 0.5) ? 0.0 : 100.0 * sqrt((g * 2.0) - 1.0);
            }
            corr[(size_t)ic * p->nxc + jc] = g;
        }
    }
}

/* The peak rule of do_time_corr (:160-177): scan ioff, then joff, and move
 * the peak when |corr| exceeds the float-rounded running maximum. */
static void time_peak(const xo_params *p, const double *corr, xo_result *r)
{
    float max_corr = -1.0f, ipeak = -9999.0f, jpeak = -9999.0f;
    double vmax = 0.0;
    for (int ic = 0; ic < p->nyc; ic++)
        for (int jc = 0; jc < p->nxc; jc++) {
            const double v = fabs(corr[(size_t)ic * p->nxc + jc]);
            if (v > vmax) vmax = v;
            if (v > max_corr) {
                max_corr = (float)v;
                jpeak = (float)(jc - p->xsearch);
                ipeak = (float)(ic - p->ysearch);
            }
        }
    r->xoff = -1 * jpeak;
    r->yoff = -1 * ipeak;
    r->corr = max_corr;
    r->gamma = max_corr;
    r->cmax = vmax;
    r->ip = (int32_t)ipeak + p->ysearch;
    r->jp = (int32_t)jpeak + p->xsearch;
    r->corr0n = corr[0];
}

/* ---- per-precision bodies ---- */
#define R float
#define SFX f32
#define XO_IS_F32 1
#include "xcorr_oracle_body.h"
#undef R
#undef SFX
#undef XO_IS_F32

#define R double
#define SFX f64
#define XO_IS_F32 0
#include "xcorr_oracle_body.h"
#undef R
#undef SFX
#undef XO_IS_F32

/* ---- patch cut (xcorr.cu:330-338 on lines read by read_xcorr_data.c:52-85) ---- */
static int cut_patch(int format, const void *img, int nx, int ny, int x0, int y0,
                     int npx, int npy, float *out)
{
    int oob = 0;
    for (int r = 0; r < npy; r++) {
        int y = y0 + r;
        for (int c = 0; c < npx; c++) {
            int x = x0 + c;
            float re = 0.f, im = 0.f;
            if (y < 0 || y >= ny || x < 0 || x >= nx) {
                oob = 1;
            } else if (format == 0) {
                const int16_t *s = (const int16_t *)img + 2 * ((size_t)y * nx + x);
                re = (float)s[0];
                im = (float)s[1];
            } else {
                re = ((const float *)img)[(size_t)y * nx + x];
            }
            out[2 * ((size_t)r * npx + c)] = re;
            out[2 * ((size_t)r * npx + c) + 1] = im;
        }
    }
    return oob;
}

static void prewarm(const xo_params *p)
{
    tab_get(p->npx); tab_get(p->npy);
    if (p->ri > 1) tab_get(p->ri * p->npx);
    tab_get(p->n2x); tab_get(p->n2y);
    tab_get(p->n2x * p->ifc); tab_get(p->n2y * p->ifc);
}

int xo_run(const xo_params *p, int precision, int format,
           const void *master, int m_nx, int m_ny,
           const void *slave, int s_nx, int s_ny,
           int x_offset, int y_offset, double astretcha,
           const int32_t *loc_xy, int nlocs, int strip_len, int nthreads,
           xo_result *out)
{
    if (!p || !out || nlocs < 0) return 1;
    /* patches are whole 1024-sample reduction blocks; a 32 x 32 surface is half
     * of one 2048-element argmax block (see xo_half_sum_ref) */
    if ((p->npx * p->npy) % 1024 || ((int64_t)p->nxc * p->nyc) % 1024) return 2;
    prewarm(p);
    const int n2 = p->n2x * p->n2y;
    double *mds = (double *)calloc((size_t)nlocs * n2 + 1, sizeof(double));
    unsigned char *nexts = (unsigned char *)calloc((size_t)nlocs * n2 + 1, 1);
#ifdef _OPENMP
    int nt = nthreads > 0 ? nthreads : omp_get_max_threads();
#else
    int nt = 1; (void)nthreads;
#endif
    (void)nt;
#ifdef _OPENMP
#pragma omp parallel num_threads(nt)
#endif
    {
        float *pm = (float *)malloc(sizeof(float) * 2 * (size_t)p->npx * p->npy);
        float *ps = (float *)malloc(sizeof(float) * 2 * (size_t)p->npx * p->npy);
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 1)
#endif
        for (int w = 0; w < nlocs; w++) {
            int x = loc_xy[2 * w], y = loc_xy[2 * w + 1];
            int ishft = (int)((double)y * astretcha);
            xo_result *r = &out[w];
            memset(r, 0, sizeof *r);
            int oob = cut_patch(format, master, m_nx, m_ny, x - p->npx / 2, y - p->npy / 2, p->npx, p->npy, pm);
            oob |= cut_patch(format, slave, s_nx, s_ny, x + x_offset - p->npx / 2,
                             y + y_offset + ishft - p->npy / 2, p->npx, p->npy, ps);
            if (precision == XO_F64) window_a_f64(p, pm, ps, r, mds + (size_t)w * n2, nexts + (size_t)w * n2);
            else window_a_f32(p, pm, ps, r, mds + (size_t)w * n2, nexts + (size_t)w * n2);
            if (oob) r->flags |= XO_FLAG_OOB;
        }
        free(pm); free(ps);
    }
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 4) num_threads(nt)
#endif
    for (int w = 0; w < nlocs; w++) {
        xo_result *r = &out[w];
        if (!p->interp_flag) { r->xfrac = r->yfrac = 0.f; r->fip = r->fjp = -1; continue; }
        double *md = mds + (size_t)w * n2;
        for (int k = 0; k < n2; k++) {
            if (!nexts[(size_t)w * n2 + k]) continue;
            r->flags |= XO_FLAG_NEXTREAD;
            int same_strip = strip_len > 0 && (w + 1) < nlocs && ((w + 1) % strip_len) != 0;
            md[k] = same_strip ? (precision == XO_F64 ? pow_quarter_f64(out[w + 1].corr0n)
                                                      : pow_quarter_f32(out[w + 1].corr0n)) : 0.0;
        }
        if (precision == XO_F64) window_b_f64(p, md, r, NULL);
        else window_b_f32(p, md, r, NULL);
    }
    free(mds);
    free(nexts);
    return 0;
}

void xo_range_interp_row(int precision, int npx, int ri, const double *in_c, double *out_c)
{
    tab_get(npx); tab_get(npx * ri);
    if (precision == XO_F64) {
        double *row = (double *)malloc(sizeof(double) * 2 * (size_t)npx);
        double *w = (double *)malloc(sizeof(double) * 2 * (size_t)npx * ri);
        memcpy(row, in_c, sizeof(double) * 2 * (size_t)npx);
        range_row_f64(row, npx, ri, w);
        memcpy(out_c, row, sizeof(double) * 2 * (size_t)npx);
        free(row); free(w);
    } else {
        float *row = (float *)malloc(sizeof(float) * 2 * (size_t)npx);
        float *w = (float *)malloc(sizeof(float) * 2 * (size_t)npx * ri);
        for (int i = 0; i < 2 * npx; i++) row[i] = (float)in_c[i];
        range_row_f32(row, npx, ri, w);
        for (int i = 0; i < 2 * npx; i++) out_c[i] = row[i];
        free(row); free(w);
    }
}

void xo_prepare_patch(const xo_params *p, int precision, int slave, const float *patch_c,
                      float *amp, double *mean, int32_t *ints)
{
    prewarm(p);
    const int n = p->npx * p->npy;
    if (precision == XO_F64) {
        double *c = (double *)malloc(sizeof(double) * 2 * (size_t)n);
        double *w = (double *)malloc(sizeof(double) * 2 * (size_t)p->npx * (p->ri > 1 ? p->ri : 1));
        for (int i = 0; i < 2 * n; i++) c[i] = patch_c[i];
        if (p->ri > 1) for (int r = 0; r < p->npy; r++) range_row_f64(c + 2 * (size_t)r * p->npx, p->npx, p->ri, w);
        *mean = prep_patch_f64(p, c, slave, ints, amp);
        free(c); free(w);
    } else {
        float *c = (float *)malloc(sizeof(float) * 2 * (size_t)n);
        float *w = (float *)malloc(sizeof(float) * 2 * (size_t)p->npx * (p->ri > 1 ? p->ri : 1));
        memcpy(c, patch_c, sizeof(float) * 2 * (size_t)n);
        if (p->ri > 1) for (int r = 0; r < p->npy; r++) range_row_f32(c + 2 * (size_t)r * p->npx, p->npx, p->ri, w);
        *mean = prep_patch_f32(p, c, slave, ints, amp);
        free(c); free(w);
    }
}

void xo_time_surface(const xo_params *p, const int32_t *i1, const int32_t *i2, double *corr, xo_result *r)
{
    memset(r, 0, sizeof *r);
    time_surface(p, i1, i2, corr);
    time_peak(p, corr, r);
}

void xo_surface(const xo_params *p, int precision, const float *pm_c, const float *ps_c,
                double *corr, double *mean1, double *mean2)
{
    prewarm(p);
    const int n = p->npx * p->npy;
    int32_t *ints = (int32_t *)malloc(sizeof(int32_t) * (size_t)n);
    if (precision == XO_F64) {
        double *c1 = (double *)malloc(sizeof(double) * 2 * (size_t)n);
        double *c2 = (double *)malloc(sizeof(double) * 2 * (size_t)n);
        double *w = (double *)malloc(sizeof(double) * 2 * (size_t)p->npx * (p->ri > 1 ? p->ri : 1));
        for (int i = 0; i < 2 * n; i++) { c1[i] = pm_c[i]; c2[i] = ps_c[i]; }
        if (p->ri > 1)
            for (int r = 0; r < p->npy; r++) {
                range_row_f64(c1 + 2 * (size_t)r * p->npx, p->npx, p->ri, w);
                range_row_f64(c2 + 2 * (size_t)r * p->npx, p->npx, p->ri, w);
            }
        *mean1 = prep_patch_f64(p, c1, 0, ints, NULL);
        *mean2 = prep_patch_f64(p, c2, 1, ints, NULL);
        surface_f64(p, c1, c2, corr);
        free(c1); free(c2); free(w);
    } else {
        float *c1 = (float *)malloc(sizeof(float) * 2 * (size_t)n);
        float *c2 = (float *)malloc(sizeof(float) * 2 * (size_t)n);
        float *w = (float *)malloc(sizeof(float) * 2 * (size_t)p->npx * (p->ri > 1 ? p->ri : 1));
        memcpy(c1, pm_c, sizeof(float) * 2 * (size_t)n);
        memcpy(c2, ps_c, sizeof(float) * 2 * (size_t)n);
        if (p->ri > 1)
            for (int r = 0; r < p->npy; r++) {
                range_row_f32(c1 + 2 * (size_t)r * p->npx, p->npx, p->ri, w);
                range_row_f32(c2 + 2 * (size_t)r * p->npx, p->npx, p->ri, w);
            }
        *mean1 = prep_patch_f32(p, c1, 0, ints, NULL);
        *mean2 = prep_patch_f32(p, c2, 1, ints, NULL);
        surface_f32(p, c1, c2, corr);
        free(c1); free(c2); free(w);
    }
    free(ints);
}

int xo_fine_surface(const xo_params *p, int precision, int format,
                    const void *master, int m_nx, int m_ny, const void *slave, int s_nx, int s_ny,
                    int x_offset, int y_offset, double astretcha, int x, int y,
                    double *re_out, xo_result *r)
{
    if (!p || !re_out || !r) return 1;
    prewarm(p);
    const int n2 = p->n2x * p->n2y;
    double md[256];
    unsigned char nx[256];
    float *pm = (float *)malloc(sizeof(float) * 2 * (size_t)p->npx * p->npy);
    float *ps = (float *)malloc(sizeof(float) * 2 * (size_t)p->npx * p->npy);
    int ishft = (int)((double)y * astretcha);
    memset(r, 0, sizeof *r);
    cut_patch(format, master, m_nx, m_ny, x - p->npx / 2, y - p->npy / 2, p->npx, p->npy, pm);
    cut_patch(format, slave, s_nx, s_ny, x + x_offset - p->npx / 2, y + y_offset + ishft - p->npy / 2, p->npx, p->npy, ps);
    if (precision == XO_F64) window_a_f64(p, pm, ps, r, md, nx);
    else window_a_f32(p, pm, ps, r, md, nx);
    for (int k = 0; k < n2; k++) if (nx[k]) md[k] = 0.0;
    if (precision == XO_F64) window_b_f64(p, md, r, re_out);
    else window_b_f32(p, md, r, re_out);
    free(pm); free(ps);
    return 0;
}
