/* Host side of the drop-in xcorr program: command line, PRM files, location
 * grid, SLC reading and the result writer.  Mirrors the reference's host C
 * code (parse_xcorr_input.c, sio_struct.c, get_locations.c, read_xcorr_data.c,
 * print_results.c); the correlation itself goes through libxcorr_gb300. */
#ifndef XCORR_CLI_H
#define XCORR_CLI_H
#include <stdint.h>
#include <stdio.h>

#include "xcorr_gb300.h"

/* The fields of struct xcorr (xcorr.h:19-63) that this program uses. */
typedef struct {
    int format;         /* 0 complex int16, 1 float32 (-real) */
    int corr_flag;      /* 0 time, 1 time4, 2 frequency (default) */
    int offset_flag;    /* -noshift */
    int interp_flag;
    int interp_factor;
    int nx_corr, ny_corr;
    int xsearch, ysearch;
    int m_nx, m_ny, s_nx, s_ny;
    int nxc, nyc, npx, npy;
    int nxl, nyl;
    int x_offset, y_offset;
    int nlocs, x_inc, y_inc;
    int ri;
    int n2x, n2y;
    double astretcha;
    char data1_name[1024], data2_name[1024];
    char filename[128];
    xcg_loc *loc;
    int verbose;
} xcli;

/* PRM values xcorr reads (sio_struct.c:132-223). */
typedef struct {
    char SLC_file[1024];
    int num_rng_bins, num_patches, num_valid_az, rshift, ashift;
    double prf;
} xcli_prm;

extern const char *XCLI_USAGE;

void xcli_die(const char *s1, const char *s2);
void xcli_set_defaults(xcli *xc);
void xcli_parse_command_line(int na, char **a, xcli *xc);
int xcli_read_prm(const char *path, xcli_prm *p);
void xcli_handle_prm(char **argv, xcli *xc);
void xcli_get_locations(xcli *xc);
void *xcli_read_slc(const char *path, int nx, int ny, int format);
void xcli_print_result(FILE *f, const xcli *xc, int iloc, const xcg_result *r);
/* Correlate every location while streaming both SLCs from disk in bands of
 * lines (slc_ingest.c); returns 0 on success. */
int xcli_correlate_streamed(const xcli *xc, xcg_ctx *ctx, xcg_result *host_results);

#endif
