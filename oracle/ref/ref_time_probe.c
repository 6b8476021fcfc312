/* Driver for the reference's time-domain correlation (test infrastructure).
 *
 * Runs the reference's own do_time_corr (do_time_int_xcorr.cu:146-189), with
 * calc_time_corr (:30-68) for -time and calc_time_corr_hat (:103-144) for
 * -time4, on one window's integer patches read from files, and writes the
 * full correlation surface and the location fields it sets.  The reference's
 * GPU program never fills the integer patches xc.i1/xc.i2 these functions
 * read (xcorr.cu:364-368), so this driver supplies them: the (int) demeaned
 * amplitudes of the master and the masked slave patch, npy x npx each.
 *
 * usage: ref_time_probe xsearch ysearch corr_flag i1.bin i2.bin out.bin
 *   i1.bin, i2.bin: npy*npx int32 (npx = 4 xsearch, npy = 4 ysearch)
 *   out.bin: nyc*nxc float64 surface (nyc = 2 ysearch, nxc = 2 xsearch),
 *            then xoff, yoff, corr as float32 (struct locs fields)
 * Built by oracle/ref/build_ref.sh against the reference sources. */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include "gmtsar_d.h"
#include "xcorr.h"

void do_time_corr(struct xcorr xc, int iloc);

static int read_all(const char *path, void *buf, size_t bytes)
{
    FILE *f = fopen(path, "rb");
    if (!f) return -1;
    size_t got = fread(buf, 1, bytes, f);
    fclose(f);
    return got == bytes ? 0 : -1;
}

int main(int argc, char **argv)
{
    if (argc != 7) {
        fprintf(stderr, "usage: ref_time_probe xsearch ysearch corr_flag i1.bin i2.bin out.bin\n");
        return 1;
    }
    struct xcorr xc;
    struct locs loc;
    memset(&xc, 0, sizeof xc);
    memset(&loc, 0, sizeof loc);
    verbose = 0;
    debug = 0;
    xc.xsearch = atoi(argv[1]);
    xc.ysearch = atoi(argv[2]);
    xc.corr_flag = atoi(argv[3]);
    /* the geometry parse_xcorr_input.c:139-158 derives from the search sizes */
    xc.nx_corr = 2 * xc.xsearch;
    xc.ny_corr = 2 * xc.ysearch;
    xc.npx = 4 * xc.xsearch;
    xc.npy = 4 * xc.ysearch;
    xc.nxc = 2 * xc.xsearch;
    xc.nyc = 2 * xc.ysearch;
    const size_t n = (size_t)xc.npx * xc.npy, ns = (size_t)xc.nxc * xc.nyc;
    xc.i1 = (int *)malloc(n * sizeof(int));
    xc.i2 = (int *)malloc(n * sizeof(int));
    xc.corr = (double *)calloc(ns, sizeof(double));
    xc.loc = &loc;
    if (!xc.i1 || !xc.i2 || !xc.corr) return 2;
    if (read_all(argv[4], xc.i1, n * sizeof(int)) || read_all(argv[5], xc.i2, n * sizeof(int))) {
        fprintf(stderr, "ref_time_probe: cannot read the integer patches\n");
        return 3;
    }
    do_time_corr(xc, 0);
    FILE *f = fopen(argv[6], "wb");
    if (!f) return 4;
    fwrite(xc.corr, sizeof(double), ns, f);
    float lf[3] = {loc.xoff, loc.yoff, loc.corr};
    fwrite(lf, sizeof(float), 3, f);
    fclose(f);
    return 0;
}
