/* The drop-in xcorr program: same command line, PRM handling, location grid
 * and freq_xcorr.dat lines as the reference (xcorr.cu:437-490), with the
 * correlation of every location done by libxcorr_gb300 in one call.
 *
 *   xcorr master.PRM aligned.PRM [-nx n] [-ny n] [-xsearch xs] [-ysearch ys]
 *         [-range_interp ri] [-norange] [-interp f] [-nointerp] [-noshift]
 *         [-real] [-freq] [-v]
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#include "xcorr_cli.h"

const char *XCLI_USAGE =
    "xcorr [GMT5SAR] - Compute 2-D cross-correlation of two images\n\n"
    "\nUsage: xcorr master.PRM slave.PRM [-time] [-real] [-freq] [-nx n] [-ny n] [-xsearch xs] [-ysearch ys]\n"
    "master.PRM     	PRM file for reference image\n"
    "slave.PRM     	 	PRM file of secondary image\n"
    "-time      		use time cross-correlation\n"
    "-freq      		use frequency cross-correlation (default)\n"
    "-real      		read float numbers instead of complex numbers\n"
    "-noshift  		ignore ashift and rshift in prm file (set to 0)\n"
    "-nx  nx    		number of locations in x (range) direction (int)\n"
    "-ny  ny    		number of locations in y (azimuth) direction (int)\n"
    "-nointerp     		do not interpolate correlation function\n"
    "-range_interp ri  	interpolate range by ri (power of two) [default: 2]\n"
    "-norange     		do not range interpolate \n"
    "-xsearch xs		search window size in x (range) direction (int power of 2 [32 64 128 256])\n"
    "-ysearch ys		search window size in y (azimuth) direction (int power of 2 [32 64 128 256])\n"
    "-interp  factor    	interpolate correlation function by factor (int) [default, 16]\n"
    "-v			verbose\n"
    "output: \n freq_xcorr.dat (default) \n time_xcorr.dat (if -time option))\n"
    "\nuse fitoffset.csh to convert output to PRM format\n"
    "\nExample:\n"
    "xcorr IMG-HH-ALPSRP075880660-H1.0__A.PRM IMG-HH-ALPSRP129560660-H1.0__A.PRM -nx 20 -ny 50 \n";

/* utils.c:39-43 */
void xcli_die(const char *s1, const char *s2)
{
    fprintf(stderr, " %s %s \n", s1, s2);
    exit(1);
}

/* set_defaults, parse_xcorr_input.c:38-88 (frequency-domain branch) */
void xcli_set_defaults(xcli *xc)
{
    xc->format = 0;
    xc->ri = 2;
    xc->nxl = 16;
    xc->nyl = 32;
    xc->x_offset = 0;
    xc->y_offset = 0;
    xc->nx_corr = 128;
    xc->ny_corr = 128;
    xc->xsearch = 64;
    xc->ysearch = 64;
    xc->n2x = 8;
    xc->n2y = 8;
    xc->npx = xc->nx_corr + 2 * xc->xsearch;
    xc->npy = xc->ny_corr + 2 * xc->ysearch;
    xc->nxc = 2 * xc->xsearch;
    xc->nyc = 2 * xc->ysearch;
    xc->astretcha = 0.0;
    xc->interp_flag = 1;
    xc->interp_factor = 16;
}

static int need_arg(int n, int na, const char *flag)
{
    if (n == na) {
        char buf[64];
        snprintf(buf, sizeof buf, " no option after %s!\n", flag);
        xcli_die(buf, "");
    }
    return n;
}

/* parse_command_line, parse_xcorr_input.c:93-183.  Unknown options are
 * rejected (the reference sends any option starting with '-' that it does not
 * know down its -input branch, parse_xcorr_input.c:165). */
void xcli_parse_command_line(int na, char **a, xcli *xc)
{
    for (int n = 3; n < na; n++) {
        if (!strcmp(a[n], "-freq")) {
            xc->corr_flag = 2;
            fprintf(stderr, " using frequency cross correlation\n");
        } else if (!strcmp(a[n], "-time")) {
            xc->corr_flag = 0;
            fprintf(stderr, " using time cross correlation\n");
        } else if (!strcmp(a[n], "-time4")) {
            xc->corr_flag = 1;
            fprintf(stderr, " using 4th power time cross correlation\n");
        } else if (!strcmp(a[n], "-real")) {
            xc->format = 1;
            fprintf(stderr, " no interpolation\n");
        } else if (!strcmp(a[n], "-nointerp")) {
            xc->interp_flag = 0;
            fprintf(stderr, " no interpolation\n");
        } else if (!strcmp(a[n], "-noshift")) {
            xc->offset_flag = 1;
            fprintf(stderr, " ignoring shift in prm\n");
        } else if (!strcmp(a[n], "-interp")) {
            n = need_arg(n + 1, na, "-interp");
            xc->interp_flag = 1;
            xc->interp_factor = atoi(a[n]);
            fprintf(stderr, " setting interpolation factor to %d\n", xc->interp_factor);
        } else if (!strcmp(a[n], "-range_interp")) {
            n = need_arg(n + 1, na, "-range_interp");
            xc->ri = atoi(a[n]);
            fprintf(stderr, " setting range interpolation factor to %d\n", xc->ri);
        } else if (!strcmp(a[n], "-nx")) {
            n = need_arg(n + 1, na, "-nx");
            xc->nxl = atoi(a[n]);
            fprintf(stderr, " setting nx to %d\n", xc->nxl);
        } else if (!strcmp(a[n], "-ny")) {
            n = need_arg(n + 1, na, "-ny");
            xc->nyl = atoi(a[n]);
            fprintf(stderr, " setting ny to %d\n", xc->nyl);
        } else if (!strcmp(a[n], "-xsearch")) {
            n = need_arg(n + 1, na, "-xsearch");
            xc->xsearch = atoi(a[n]);
            xc->nx_corr = 2 * xc->xsearch;
            xc->npx = xc->nx_corr + 2 * xc->xsearch;
            xc->nxc = 2 * xc->xsearch;
            if (((xc->xsearch - 1) & xc->xsearch)) xcli_die(" xsearch needs to be power of 2! (32 64 128 256) \n", "");
            fprintf(stderr, " setting xsearch to %d\n", xc->xsearch);
            fprintf(stderr, " setting nx_corr to %d\n", xc->nx_corr);
        } else if (!strcmp(a[n], "-ysearch")) {
            n = need_arg(n + 1, na, "-ysearch");
            xc->ysearch = atoi(a[n]);
            xc->ny_corr = 2 * xc->ysearch;
            xc->npy = xc->ny_corr + 2 * xc->ysearch;
            xc->nyc = 2 * xc->ysearch;
            if (((xc->ysearch - 1) & xc->ysearch)) xcli_die(" ysearch needs to be power of 2! (32 64 128 256) \n", "");
            fprintf(stderr, " setting ysearch to %d\n", xc->ysearch);
            fprintf(stderr, " setting ny_corr to %d\n", xc->ny_corr);
        } else if (!strcmp(a[n], "-v")) {
            xc->verbose = 1;
            fprintf(stderr, " verbose output \n");
        } else if (!strcmp(a[n], "-norange")) {
            xc->ri = 1;
            fprintf(stderr, " no range interpolation \n");
        } else {
            fprintf(stderr, " %s *** option not recognized ***\n\n", a[n]);
            fprintf(stderr, "%s", XCLI_USAGE);
            exit(1);
        }
    }
}

/* get_sio_struct (sio_struct.c:132-223): "name = value" pairs; the keys xcorr uses. */
int xcli_read_prm(const char *path, xcli_prm *p)
{
    FILE *f = fopen(path, "r");
    if (!f) return -1;
    char name[1024], value[1024];
    memset(p, 0, sizeof *p);
    p->prf = -99999.9999;
    while (fscanf(f, "%1023s = %1023s \n", name, value) != EOF) {
        if (!strcmp(name, "SLC_file")) snprintf(p->SLC_file, sizeof p->SLC_file, "%s", value);
        else if (!strcmp(name, "num_rng_bins")) p->num_rng_bins = atoi(value);
        else if (!strcmp(name, "num_patches")) p->num_patches = atoi(value);
        else if (!strcmp(name, "num_valid_az")) p->num_valid_az = atoi(value);
        else if (!strcmp(name, "rshift") || !strcmp(name, "xshift")) p->rshift = atoi(value);
        else if (!strcmp(name, "ashift") || !strcmp(name, "yshift")) p->ashift = atoi(value);
        else if (!strcmp(name, "PRF")) p->prf = atof(value);
    }
    fclose(f);
    return 0;
}

/* handle_prm, parse_xcorr_input.c:185-238 */
void xcli_handle_prm(char **argv, xcli *xc)
{
    xcli_prm r[2];
    for (int i = 0; i < 2; i++) {
        if (xcli_read_prm(argv[i + 1], &r[i]) != 0) xcli_die("Can't open prmfile ", argv[i + 1]);
        FILE *t = fopen(r[i].SLC_file, "r");
        if (!t) xcli_die("Cannot open SLC_file", r[i].SLC_file);
        fclose(t);
    }
    snprintf(xc->data1_name, sizeof xc->data1_name, "%s", r[0].SLC_file);
    xc->m_nx = r[0].num_rng_bins;
    xc->m_ny = r[0].num_patches * r[0].num_valid_az;
    snprintf(xc->data2_name, sizeof xc->data2_name, "%s", r[1].SLC_file);
    xc->s_nx = r[1].num_rng_bins;
    xc->s_ny = r[1].num_patches * r[1].num_valid_az;
    xc->x_offset = r[1].rshift;
    xc->y_offset = r[1].ashift;
    xc->astretcha = (r[0].prf > 0) ? (r[1].prf - r[0].prf) / r[0].prf : 0.0;
    if (xc->offset_flag == 1) {   /* checked once per PRM file in the reference (:228-231) */
        xc->x_offset = xc->y_offset = 0;
        fprintf(stderr, " setting ashift and rshift to zero\n");
        fprintf(stderr, " setting ashift and rshift to zero\n");
    }
    fprintf(stderr, " %d %d %d %d %d %d %f\n", xc->m_nx, xc->m_ny, xc->s_nx, xc->s_ny, xc->x_offset,
            xc->y_offset, xc->astretcha);
}

/* get_locations, get_locations.c:14-46 */
void xcli_get_locations(xcli *xc)
{
    xc->x_inc = (xc->m_nx - 2 * (xc->xsearch + xc->nx_corr)) / (xc->nxl + 3);
    xc->y_inc = (xc->m_ny - 2 * (xc->ysearch + xc->ny_corr)) / (xc->nyl + 1);
    xc->loc = (xcg_loc *)malloc(sizeof(xcg_loc) * (size_t)xc->nyl * (xc->nxl + 1));
    int n = 0;
    for (int j = 1; j <= xc->nyl; j++)
        for (int i = 2; i <= xc->nxl + 1; i++) {
            xc->loc[n].x = xc->npx + i * xc->x_inc;
            xc->loc[n].y = xc->npy + j * xc->y_inc;
            n++;
        }
    xc->nlocs = n;
    fprintf(stderr, " locations  n %d nx %d nyl %d nxl %d x_inc %d y_inc %d\n", n, xc->m_nx, xc->nyl, xc->nxl,
            xc->x_inc, xc->y_inc);
}

/* Whole-image read of an SLC (the lines read_complex_short2 / read_real_float2
 * read, read_xcorr_data.c:11-49).  A file shorter than nx*ny samples leaves
 * the missing lines zero. */
void *xcli_read_slc(const char *path, int nx, int ny, int format)
{
    (void)format;
    const size_t bytes = (size_t)nx * ny * 4;     /* int16 I/Q pair or float32 */
    void *buf = calloc(1, bytes);
    if (!buf) xcli_die("out of memory reading", path);
    FILE *f = fopen(path, "rb");
    if (!f) xcli_die("Cannot open SLC_file", path);
    size_t got = fread(buf, 1, bytes, f);
    if (got < bytes) fprintf(stderr, " warning: %s holds %zu of %zu bytes; missing lines read as zero\n", path, got, bytes);
    fclose(f);
    return buf;
}

/* print_results, print_results.c:12-46 */
void xcli_print_result(FILE *f, const xcli *xc, int iloc, const xcg_result *r)
{
    float xoff = r->xoff, xfrac = r->xfrac, yoff = r->yoff, yfrac = r->yfrac, corr = r->corr;
    int interp = xc->interp_flag ? xc->interp_factor : 1;
    int ishft = (int)(xc->loc[iloc].y * xc->astretcha);
    xoff = (xoff / (float)xc->ri) - (xfrac / (float)xc->ri) + xc->x_offset;
    yoff = yoff - yfrac + xc->y_offset + ishft;
    if (xc->verbose)
        fprintf(stdout, " location %d (%3d,%3d) interpolation (range %d corr %d) correlation %6.2f offset (%6.3f,%6.3f) \n",
                iloc, xc->loc[iloc].x, xc->loc[iloc].y, xc->ri, interp, corr, xoff, yoff);
    fprintf(f, " %d %6.3f %d %6.3f %6.2f \n", xc->loc[iloc].x, xoff, xc->loc[iloc].y, yoff, corr);
}

int main(int argc, char **argv)
{
    xcli xc;
    memset(&xc, 0, sizeof xc);
    xc.corr_flag = 2;
    if (argc < 3) xcli_die(XCLI_USAGE, "");
    xcli_set_defaults(&xc);
    xcli_parse_command_line(argc, argv, &xc);
    xcli_handle_prm(argv, &xc);
    /* xcorr.cu:467-469 */
    if (xc.corr_flag == 0) strcpy(xc.filename, "time_xcorr.dat");
    if (xc.corr_flag == 1) strcpy(xc.filename, "time_xcorr_Gatelli.dat");
    if (xc.corr_flag == 2) strcpy(xc.filename, "freq_xcorr.dat");
    FILE *out = fopen(xc.filename, "w");
    if (!out) xcli_die("Can't open output file", xc.filename);
    xcli_get_locations(&xc);

    /* XCORR_DRY_RUN=1: print the parsed parameters and the location grid and
     * stop before reading images or touching the GPU; with
     * XCORR_PRINT_FILE=<file>, also format each "x y xoff yoff xfrac yfrac corr"
     * line of that file as a freq_xcorr.dat line on stdout. */
    if (getenv("XCORR_DRY_RUN")) {
        printf("params format=%d m_nx=%d m_ny=%d s_nx=%d s_ny=%d nxl=%d nyl=%d x_offset=%d y_offset=%d "
               "nx_corr=%d ny_corr=%d xsearch=%d ysearch=%d npx=%d npy=%d nxc=%d nyc=%d ri=%d "
               "interp_flag=%d interp_factor=%d n2x=%d n2y=%d astretcha=%.17g\n",
               xc.format, xc.m_nx, xc.m_ny, xc.s_nx, xc.s_ny, xc.nxl, xc.nyl, xc.x_offset, xc.y_offset,
               xc.nx_corr, xc.ny_corr, xc.xsearch, xc.ysearch, xc.npx, xc.npy, xc.nxc, xc.nyc, xc.ri,
               xc.interp_flag, xc.interp_factor, xc.n2x, xc.n2y, xc.astretcha);
        printf("locs n=%d x_inc=%d y_inc=%d\n", xc.nlocs, xc.x_inc, xc.y_inc);
        for (int i = 0; i < xc.nlocs; i++) printf("loc %d %d %d\n", i, xc.loc[i].x, xc.loc[i].y);
        const char *pf = getenv("XCORR_PRINT_FILE");
        if (pf) {
            FILE *f = fopen(pf, "r");
            if (!f) xcli_die("Can't open", pf);
            xcg_result r;
            xcg_loc one;
            memset(&r, 0, sizeof r);
            xcli tmp = xc;
            tmp.loc = &one;
            while (fscanf(f, "%d %d %f %f %f %f %f", &one.x, &one.y, &r.xoff, &r.yoff, &r.xfrac, &r.yfrac, &r.corr) == 7)
                xcli_print_result(stdout, &tmp, 0, &r);
            fclose(f);
        }
        fclose(out);
        return 0;
    }

    xcg_params p;
    xcg_default_params(&p);
    p.xsearch = xc.xsearch; p.ysearch = xc.ysearch;
    p.nx_corr = xc.nx_corr; p.ny_corr = xc.ny_corr;
    p.ri = xc.ri;
    p.interp_flag = xc.interp_flag;
    p.interp_factor = xc.interp_factor;
    p.n2x = xc.n2x; p.n2y = xc.n2y;
    p.format = xc.format;
    p.corr_mode = xc.corr_flag;

    struct timespec t0, t1;
    clock_gettime(CLOCK_MONOTONIC, &t0);
    /* scratch for this job's batches only: two batches of whole strips (the
     * library's default holds 2048 windows per slot) */
    int max_batch = xc.nlocs >= 512 ? (xc.nlocs + 1) / 2 : xc.nlocs;
    if (xc.nxl > 0) max_batch = ((max_batch + xc.nxl - 1) / xc.nxl) * xc.nxl;
    if (max_batch > 2048 || max_batch < 1) max_batch = 0;
    xcg_ctx *ctx = NULL;
    xcg_status st = xcg_create(&p, 0, max_batch, &ctx);
    if (st != XCG_OK) {
        fprintf(stderr, "xcorr: %s: %s\n", xcg_status_string(st), xcg_last_error());
        return 1;
    }
    xcg_result *res = (xcg_result *)calloc((size_t)xc.nlocs + 1, sizeof(xcg_result));
    void *m = NULL, *s = NULL;
    if (getenv("XCORR_WHOLE_READ")) {
        /* read both images whole, then one call over all locations */
        m = xcli_read_slc(xc.data1_name, xc.m_nx, xc.m_ny, xc.format);
        s = xcli_read_slc(xc.data2_name, xc.s_nx, xc.s_ny, xc.format);
        st = xcg_correlate(ctx, m, xc.m_nx, xc.m_ny, s, xc.s_nx, xc.s_ny, xc.x_offset, xc.y_offset, xc.astretcha,
                           xc.loc, xc.nlocs, xc.nxl, res);
        if (st != XCG_OK) {
            fprintf(stderr, "xcorr: %s: %s\n", xcg_status_string(st), xcg_last_error());
            return 1;
        }
    } else if (xcli_correlate_streamed(&xc, ctx, res) != 0) {
        return 1;
    }
    for (int i = 0; i < xc.nlocs; i++) xcli_print_result(out, &xc, i, &res[i]);
    clock_gettime(CLOCK_MONOTONIC, &t1);
    fprintf(stdout, " elapsed time: %lf \n", (t1.tv_sec - t0.tv_sec) + 1e-9 * (t1.tv_nsec - t0.tv_nsec));
    fclose(out);
    xcg_destroy(ctx);
    free(res);
    free(m);
    free(s);
    free(xc.loc);
    return 0;
}
