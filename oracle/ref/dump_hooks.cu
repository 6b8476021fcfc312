/* Full-precision dump hooks for the reference xcorr-gpu build.
 *
 * Test infrastructure (oracle side): linked only into oracle/_ref/xcorr-gpu-dump,
 * the reference program built from its own unchanged sources by
 * oracle/ref/build_ref.sh.  The recipe renames four reference functions at
 * their call sites with -D, so that each call lands here first; every hook
 * calls the real function and records what it returned:
 *   h_reduceFD_strip  (conv_ampl_demean.cu:703, called xcorr.cu:277,287)  patch means
 *   h_reduce_strip    (conv_ampl_demean.cu:642, called do_freq_xcorr.cu:147) cave, cmax, ip, jp
 *   h_reduceCr_strip  (conv_ampl_demean.cu:730, called highres_corr.cu:57)  fine peak
 *   print_results     (print_results.c:12, called xcorr.cu:371)            struct locs
 * One line per location goes to $XCG_REF_DUMP (default ref_dump.txt). */
#include <stdio.h>
#include <stdlib.h>
extern "C" {
#include "gmtsar_ext.h"
#include "xcorr_d.h"
void xcg_ref_orig_print_results(struct xcorr xc, int iloc);
}

void h_reduceFD_strip(float *d_in, int nx, int ny, int nl, double *gmean, struct d_xcorr d_xc);
void h_reduce_strip(double *d_in, int nx, int ny, int nl, double *gmean, double *gmax, int *ip, int *jp, struct d_xcorr d_xc);
void h_reduceCr_strip(cufftComplex *d_in, int nx, int ny, int nl, float *gmax, int *ip, int *jp, struct d_xcorr d_xc);

#define XCG_MAXNL 4096
static double s_mean[2][XCG_MAXNL];
static int s_mean_calls = 0;
static double s_cave[XCG_MAXNL], s_cmax[XCG_MAXNL];
static int s_ip[XCG_MAXNL], s_jp[XCG_MAXNL];
static float s_fmax[XCG_MAXNL];
static int s_fip[XCG_MAXNL], s_fjp[XCG_MAXNL], s_have_fine = 0;
static int s_cursor = 0;
static FILE *s_dump = NULL;

void xcg_hook_h_reduceFD_strip(float *d_in, int nx, int ny, int nl, double *gmean, struct d_xcorr d_xc)
{
    h_reduceFD_strip(d_in, nx, ny, nl, gmean, d_xc);
    int which = s_mean_calls++ & 1;          /* master first, then slave (xcorr.cu:277,287) */
    for (int j = 0; j < nl && j < XCG_MAXNL; j++) s_mean[which][j] = gmean[j];
}

void xcg_hook_h_reduce_strip(double *d_in, int nx, int ny, int nl, double *gmean, double *gmax, int *ip, int *jp, struct d_xcorr d_xc)
{
    h_reduce_strip(d_in, nx, ny, nl, gmean, gmax, ip, jp, d_xc);
    for (int j = 0; j < nl && j < XCG_MAXNL; j++) {
        s_cave[j] = gmean[j]; s_cmax[j] = gmax[j]; s_ip[j] = ip[j]; s_jp[j] = jp[j];
    }
    s_cursor = 0;
    s_have_fine = 0;
}

void xcg_hook_h_reduceCr_strip(cufftComplex *d_in, int nx, int ny, int nl, float *gmax, int *ip, int *jp, struct d_xcorr d_xc)
{
    h_reduceCr_strip(d_in, nx, ny, nl, gmax, ip, jp, d_xc);
    for (int j = 0; j < nl && j < XCG_MAXNL; j++) { s_fmax[j] = gmax[j]; s_fip[j] = ip[j]; s_fjp[j] = jp[j]; }
    s_have_fine = 1;
}

extern "C" void print_results(struct xcorr xc, int iloc)
{
    if (!s_dump) {
        const char *p = getenv("XCG_REF_DUMP");
        s_dump = fopen(p ? p : "ref_dump.txt", "w");
        if (!s_dump) { perror("ref dump"); exit(3); }
        fprintf(s_dump, "# iloc x y xoff yoff xfrac yfrac corr cmax cave ip jp fip fjp fmax mean1 mean2\n");
    }
    int j = s_cursor++;
    struct locs *L = &xc.loc[iloc];
    fprintf(s_dump, "%d %d %d %.9g %.9g %.9g %.9g %.9g %.17g %.17g %d %d %d %d %.9g %.17g %.17g\n",
            iloc, L->x, L->y, L->xoff, L->yoff, L->xfrac, L->yfrac, L->corr,
            s_cmax[j], s_cave[j], s_ip[j], s_jp[j],
            s_have_fine ? s_fip[j] : -1, s_have_fine ? s_fjp[j] : -1, s_have_fine ? s_fmax[j] : 0.0f,
            s_mean[0][j], s_mean[1][j]);
    fflush(s_dump);
    xcg_ref_orig_print_results(xc, iloc);
}
