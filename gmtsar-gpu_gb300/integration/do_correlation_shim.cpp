/* do_correlation_shim.cpp: the reference program's do_correlation
 * (xcorr.cu:299-378) replaced by one libxcorr_gb300 call.  A maintainer keeps
 * the reference's main, set_defaults, parse_command_line, handle_prm,
 * get_locations and print_results; compile this file with the reference's
 * headers and link -lxcorr_gb300 instead of -lcufft (config.mk:23).
 * xcorr.cu is CUDA C++, so do_correlation has C++ linkage there and this
 * file is C++ too; the reference's C headers are included as xcorr.cu
 * includes them, inside extern "C" (xcorr.cu:24-26). */
#include <stdio.h>
#include <stdlib.h>
extern "C" {
#include "gmtsar_d.h"
#include "xcorr.h"
}
#include "xcorr_gb300.h"

static void *read_image(FILE *f, int nx, int ny)          /* whole SLC, as read_xcorr_data.c reads lines */
{
    size_t bytes = (size_t)nx * ny * 4;                    /* int16 I,Q or float32 */
    void *buf = calloc(1, bytes);
    fseek(f, 0, SEEK_SET);
    if (fread(buf, 1, bytes, f) < bytes) { /* short file: missing lines stay zero */ }
    return buf;
}

void do_correlation(struct xcorr xc)                       /* replaces xcorr.cu:299-378 */
{
    xcg_params p;
    xcg_default_params(&p);
    p.xsearch = xc.xsearch;   p.ysearch = xc.ysearch;
    p.nx_corr = xc.nx_corr;   p.ny_corr = xc.ny_corr;
    p.ri = xc.ri;             p.interp_flag = xc.interp_flag;
    p.interp_factor = xc.interp_factor;
    p.n2x = xc.n2x;           p.n2y = xc.n2y;
    p.format = xc.format;
    p.corr_mode = xc.corr_flag;

    void *m = read_image(xc.data1, xc.m_nx, xc.m_ny);
    void *s = read_image(xc.data2, xc.s_nx, xc.s_ny);
    xcg_loc *locs = (xcg_loc *)malloc(sizeof(xcg_loc) * xc.nlocs);
    xcg_result *res = (xcg_result *)malloc(sizeof(xcg_result) * xc.nlocs);
    for (int i = 0; i < xc.nlocs; i++) { locs[i].x = xc.loc[i].x; locs[i].y = xc.loc[i].y; }

    fprintf(stderr, " correlating %d locations with libxcorr_gb300\n", xc.nlocs);
    xcg_ctx *ctx;
    xcg_status st = xcg_create(&p, 0, 0, &ctx);
    if (st == XCG_OK)
        st = xcg_correlate(ctx, m, xc.m_nx, xc.m_ny, s, xc.s_nx, xc.s_ny,
                           xc.x_offset, xc.y_offset, xc.astretcha,
                           locs, xc.nlocs, xc.nxl, res);
    if (st != XCG_OK) die(xcg_status_string(st), xcg_last_error());

    for (int i = 0; i < xc.nlocs; i++) {                   /* back into struct locs, then the reference's writer */
        xc.loc[i].xoff = res[i].xoff;   xc.loc[i].yoff = res[i].yoff;
        xc.loc[i].xfrac = res[i].xfrac; xc.loc[i].yfrac = res[i].yfrac;
        xc.loc[i].corr = res[i].corr;
        print_results(xc, i);
    }
    xcg_destroy(ctx);
    free(m); free(s); free(locs); free(res);
}
