// Device-side plan shared by the xcorr kernels: sizes, image views, tables
// and the per-batch scratch layout.  Passed to every kernel by value.
#pragma once
#include <stdint.h>

#include "xcorr_gb300.h"

namespace xcg {

// One image pair as the kernels see it: device images, PRM offsets, the
// pair's result array and strip length.
struct PairDev {
    const void *master;
    int m_nx, m_ny;
    const void *slave;
    int s_nx, s_ny;
    int x_offset, y_offset;
    double astretcha;
    xcg_result *out;       // results of this pair, indexed by the window's index within the pair
    int nlocs;             // windows of this pair
    int strip_len;         // 0: no cross-window read
    float *feat;           // [nlocs][81] normalised 9x9 neighbourhood of the integer peak, or null
};

struct Plan {
    // geometry (parse_xcorr_input.c:67-86)
    int npx, npy;          // patch: 4*xsearch x 4*ysearch
    int nxc, nyc;          // surface: 2*xsearch x 2*ysearch
    int nx_corr, ny_corr;  // time-correlation window
    int xsearch, ysearch;
    int ri, log2ri;
    int interp_flag, ifc, n2x, n2y, nx2, ny2;
    int format;            // 0 complex int16, 1 float32 real
    int corr_mode;         // 2 frequency domain; 0 -time, 1 -time4 full search
    // precision form: the correlation's row/column DFTs as split-FP16
    // tensor-core matmuls (tc_dft.cu); 0 = FP32 SIMT FFTs
    int tc_form;
    // launch shapes (xcorr_kernels.cu): k_cols 0 default, 1 256-thread CTAs, 2
    // one staging group; k_peak 0 four CTAs/SM, 1 three
    int cols_cfg, peak_cfg;
    const uint8_t *tc_a_row;   // prepared forward DFT operand for the rows (npx)
    const uint8_t *tc_a_col;   // forward DFT operand for the columns (npy)
    const uint8_t *tc_a_inv;   // inverse DFT rows of the surface band (nyc x npy)
    int *tc_err;               // raised when a tensor-core wait ran out
    int nchunks;           // 1024-sample chunks per patch (npx*npy/1024)
    int qpitch;            // row pitch (complex) of the half-spectrum rows: npx/2 + 16

    // image pairs: one pair by value, or a table with a per-window reference
    PairDev single;        // used when pairs == nullptr
    const PairDev *pairs;  // stack of pairs (device)
    const int2 *winref;    // [nwin] (pair, index within the pair), offset to the batch

    // windows of this batch
    const xcg_loc *locs;   // already offset to the batch's first window
    int nwin;              // windows in this batch
    int win0;              // single pair: index of the batch's first window

    // tables (device, built on the host in double)
    const float2 *tw_row;   // Stockham twiddles for npx
    const float2 *tw_col;   // Stockham twiddles for npy
    const float2 *phase;    // (ri-1) x npx: exp(+2 pi i f' p / (ri npx)) / npx
    const float2 *box_x;    // npx: DFT of the column mask
    const float2 *box_y;    // npy: DFT of the row mask
    const float2 *kx;       // nx2 x n2x interpolation operator (row pass)
    const float2 *ky;       // ny2 x n2y (column pass)

    // scratch (per batch, indexed by batch-local window)
    float2 *zrow;     // [nwin][npy][npx]   row spectra of a1 + i*a2*mask
    float *amp1;      // [nwin][npy][npx]   master amplitudes
    float *amp2c;     // [nwin][ny_corr][nx_corr] slave amplitudes, centre
    float *part;      // [nwin][2][nchunks] FP32 chunk sums (master, slave)
    unsigned char *oobmap;  // [nwin][nchunks] 1 where a chunk read outside its image
    float *minmax;    // [nwin][4][nchunks] master min/max, masked slave min/max
    double *means;    // [nwin][2]
    float2 *qspec;    // [nwin][nyc][qpitch] column-inverted half spectrum
    float *surf;      // [nwin][nyc][nxc]  correlation surface
    float *md;        // [nwin][n2y*n2x]  neighbourhood ^0.25, NaN-safe
    unsigned char *mdnext;  // [nwin][n2y*n2x] 1 where the next window's value goes
    double *corr0n;   // [nwin]
    const unsigned char *skip;  // [nwin] 1: the subpixel stage leaves this window alone (null: none)

    // shared row segments (segment_rows.cu): the row stage runs once per image
    // row segment that one or more windows of the batch read, in chunks of
    // 1024 samples; a window's patch rows are consecutive rows of its chunks
    int rc;                 // 1: this path; 0: one row stage per window (zrow, amp1, ...)
    int rpc;                // rows per chunk: 1024 / npx
    int4 *rc_desc;          // [chunks] (pair, 0 master / 1 slave, first column, first row)
    int2 *rc_wch;           // [nwin] first master (x) and slave (y) chunk of each window
    int *rc_count;          // [2] chunks of the batch (the planner): numbered from 0, then from nwin * nchunks
    float *rc_amp;          // [chunks][rpc][npx] amplitudes of the kept fine samples
    float2 *rc_spec;        // [chunks][rpc][npx/2] half row spectra; bin 0 holds (DC, Nyquist)
    float *rc_part;         // [chunks] FP32 chunk sums in the reference's tree order
    float2 *rc_minmax;      // [chunks] (min, max); slave chunks over the mask columns only
    unsigned char *rc_oob;  // [chunks] 1 where a sample lay outside its image
    // row bands (host entry): the planner also lists the chunks band by band,
    // a chunk in the first band whose end row (per image) lies beyond the
    // chunk's last row, so each band's row-stage launch can wait for its copy
    int rc_nbands;          // 0: no band order, the row stage takes every chunk in planned order
    int rc_band;            // with bands: this row-stage launch's band
    int rc_band_end[2][8];  // master / slave rows [.., end) of each band
    int *rc_order;          // [chunks] chunk indices band by band
    int *rc_band_start;     // [9] first entry of each band in rc_order, then the total
    int *rc_tile_next;      // [1] the persistent column stage's next tile (zeroed by the planner), or null
};

// The pair of batch window w (a copy: taking the address of the kernel
// parameter would force the whole plan into local memory), the window's index
// within that pair and the pair's index in the table.
__device__ __forceinline__ PairDev pair_of(const Plan &P, int w, int &local, int &pidx) {
    if (P.pairs) {
        const int2 r = P.winref[w];
        local = r.y;
        pidx = r.x;
        return P.pairs[r.x];
    }
    local = P.win0 + w;
    pidx = 0;
    return P.single;
}

}  // namespace xcg
