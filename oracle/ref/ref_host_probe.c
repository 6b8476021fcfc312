/* Driver for the reference's host C functions (test infrastructure).
 *
 * Runs the reference's own set_defaults / parse_command_line / handle_prm /
 * get_locations (parse_xcorr_input.c:38-238, get_locations.c:14-46) on the
 * given command line, exactly as main() does (xcorr.cu:444-475), and prints
 * the resulting parameters and location grid.  With XCG_PROBE_PRINT=<file>
 * it also feeds each line "x y xoff yoff xfrac yfrac corr" of that file through
 * the reference's print_results (print_results.c:12-46) to stdout, and with
 * XCG_PROBE_PATCHES=<n> it reads the first n strips with read_xcorr_data
 * (read_xcorr_data.c:52-85) and prints per-location patch checksums.
 * Built by oracle/ref/build_ref.sh against the reference sources. */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include "gmtsar_d.h"
#include "xcorr.h"

int main(int argc, char **argv)
{
    struct xcorr xc;
    int input_flag = 0, nfiles = 2;
    memset(&xc, 0, sizeof xc);
    verbose = 0; debug = 0;
    xc.interp_flag = 0;
    xc.corr_flag = 2;
    if (argc < 3) { fprintf(stderr, "usage: ref_host_probe master.PRM aligned.PRM [flags]\n"); return 1; }
    set_defaults(&xc);
    parse_command_line(argc, argv, &xc, &nfiles, &input_flag, "usage");
    if (input_flag == 0) handle_prm(argv, &xc, nfiles);
    get_locations(&xc);

    printf("params format=%d m_nx=%d m_ny=%d s_nx=%d s_ny=%d nxl=%d nyl=%d x_offset=%d y_offset=%d "
           "nx_corr=%d ny_corr=%d xsearch=%d ysearch=%d npx=%d npy=%d nxc=%d nyc=%d ri=%d "
           "interp_flag=%d interp_factor=%d n2x=%d n2y=%d astretcha=%.17g\n",
           xc.format, xc.m_nx, xc.m_ny, xc.s_nx, xc.s_ny, xc.nxl, xc.nyl, xc.x_offset, xc.y_offset,
           xc.nx_corr, xc.ny_corr, xc.xsearch, xc.ysearch, xc.npx, xc.npy, xc.nxc, xc.nyc, xc.ri,
           xc.interp_flag, xc.interp_factor, xc.n2x, xc.n2y, xc.astretcha);
    printf("locs n=%d x_inc=%d y_inc=%d\n", xc.nlocs, xc.x_inc, xc.y_inc);
    for (int i = 0; i < xc.nlocs; i++) printf("loc %d %d %d\n", i, xc.loc[i].x, xc.loc[i].y);

    const char *pp = getenv("XCG_PROBE_PATCHES");
    if (pp) {
        int nstrips = atoi(pp);
        xc.d1 = malloc((size_t)xc.m_nx * xc.npy * sizeof(struct FCOMPLEX));
        xc.d2 = malloc((size_t)xc.s_nx * xc.npy * sizeof(struct FCOMPLEX));
        for (int s = 0; s < nstrips && s < xc.nyl; s++) {
            int iloc0 = s * xc.nxl;
            read_xcorr_data(xc, iloc0);
            for (int j = 0; j < xc.nxl; j++) {
                int mx = xc.loc[iloc0 + j].x - xc.npx / 2;
                int sx = xc.loc[iloc0 + j].x + xc.x_offset - xc.npx / 2;
                double s1 = 0, s2 = 0, q1 = 0, q2 = 0;
                for (int r = 0; r < xc.npy; r++)
                    for (int c = 0; c < xc.npx; c++) {
                        struct FCOMPLEX a = xc.d1[(size_t)r * xc.m_nx + mx + c];
                        struct FCOMPLEX b = xc.d2[(size_t)r * xc.s_nx + sx + c];
                        s1 += a.r + 3.0 * a.i; q1 += (double)a.r * a.r + (double)a.i * a.i;
                        s2 += b.r + 3.0 * b.i; q2 += (double)b.r * b.r + (double)b.i * b.i;
                    }
                printf("patch %d %.17g %.17g %.17g %.17g\n", iloc0 + j, s1, q1, s2, q2);
            }
        }
    }

    const char *pf = getenv("XCG_PROBE_PRINT");
    if (pf) {
        FILE *f = fopen(pf, "r");
        if (!f) { perror(pf); return 2; }
        xc.file = stdout;
        struct locs L;
        int n = 0;
        memset(&L, 0, sizeof L);
        xc.loc = &L;
        while (fscanf(f, "%d %d %f %f %f %f %f", &L.x, &L.y, &L.xoff, &L.yoff, &L.xfrac, &L.yfrac, &L.corr) == 7) {
            print_results(xc, 0);
            n++;
        }
        fclose(f);
    }
    return 0;
}
