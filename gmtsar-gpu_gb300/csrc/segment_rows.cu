// Shared row segments: the row stage of the frequency-domain path computed
// once per image row segment rather than once per window that reads it.
//
// Windows of one column of the location grid read the same columns of the
// same image rows: with y_inc = 72 and 256-row patches (the 128 x 128
// configuration) each master and slave row segment belongs to about 3.5
// windows, with 512-row patches and y_inc = 74 (the full frame) to about 7.
// The reference cuts, range-interpolates and transforms every window's
// patch on its own (xcorr.cu:330-338, 237-292); the amplitudes of a row
// segment do not depend on the window, so they are computed once here and
// every window's means, (int) copies and time correlation see the same
// numbers the per-window path computes.  The demean and mask enter in the
// frequency domain by linearity (k_cols_rc), so the row spectra do not depend
// on the window either.
//
//   k_rc_plan   one CTA per batch, or one per image when the chunks need no
//               row-band order: every window contributes a master and a
//               slave entry (pair, image, first column, first row); entries
//               with the same pair, image, first column and first row modulo
//               the rows of a chunk are sorted by row and merged where their
//               row ranges overlap or touch; each merged run gets a range of
//               1024-sample chunks, so a window's patch is a run of
//               consecutive chunk rows
//   k_segrows   one warp per chunk (rows per chunk = 1024 / npx): the patch
//               rows of k_rows (read, range interpolation, amplitude, the
//               reference's FP32 chunk sums, extremes, out-of-image flags),
//               then the half spectra of the chunk's rows, two real rows per
//               complex FFT separated by Hermitian symmetry
//   k_cols_rc   per group of columns kx of one window: the column FFTs of
//               the master's and the masked slave's half spectra, the
//               product with the demean/mask corrections and the inverse
//               column FFT of the surface rows, as k_cols; the default form
//               (k_cols_rcp) is persistent, each CTA taking (window, column
//               group) tiles from a counter, the next tile's rows staged while
//               the current one is transformed
#include <cuda_runtime.h>
#include <algorithm>
#include <math.h>
#include <stdint.h>

#include "kernel_util.cuh"
#include "segment_rows.cuh"
#include "team_fft.cuh"

namespace xcg {

// ------------------------------------------------------------------ planner

constexpr int RC_ENTRIES = 2 * RC_MAX_WINDOWS;   // sort capacity, a power of two
constexpr int PLAN_THREADS = 1024;
constexpr int PER_THREAD = RC_ENTRIES / PLAN_THREADS;
// Sort key: pair (15 bits) | image (1) | first column + 2^19 (20) | first row
// modulo the chunk rows (4) | first row + 2^23 (24).  The group of an entry is
// the key without its low 24 bits.
constexpr int KEY_Y_BITS = 24;
constexpr int KEY_Y_BIAS = 1 << 23;
constexpr int KEY_X_BIAS = 1 << 19;

// In-place exclusive scan of a[0, ns) by the whole CTA (ns a multiple of
// PLAN_THREADS up to RC_ENTRIES); returns the total.
__device__ int block_exclusive_scan(int *a, int *wsum, int ns) {
    const int t = threadIdx.x, l32 = t & 31, wp = t >> 5;
    const int per = ns / PLAN_THREADS;
    int v[PER_THREAD];
    int s = 0;
#pragma unroll
    for (int k = 0; k < PER_THREAD; k++) { v[k] = (k < per) ? a[t * per + k] : 0; s += v[k]; }
    int inc = s;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int u = __shfl_up_sync(0xffffffffu, inc, o);
        if (l32 >= o) inc += u;
    }
    if (l32 == 31) wsum[wp] = inc;
    __syncthreads();
    if (wp == 0) {
        int x = (l32 < PLAN_THREADS / 32) ? wsum[l32] : 0;
        int xi = x;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int u = __shfl_up_sync(0xffffffffu, xi, o);
            if (l32 >= o) xi += u;
        }
        wsum[32 + l32] = xi - x;                  // exclusive prefix of the warp totals
        if (l32 == 31) wsum[64] = xi;             // CTA total
    }
    __syncthreads();
    int run = wsum[32 + wp] + inc - s;
#pragma unroll
    for (int k = 0; k < PER_THREAD; k++)
        if (k < per) { a[t * per + k] = run; run += v[k]; }
    const int total = wsum[64];
    __syncthreads();
    return total;
}

__device__ __forceinline__ int key_y(unsigned long long k) {
    return (int)(k & ((1ull << KEY_Y_BITS) - 1)) - KEY_Y_BIAS;
}

__global__ void __launch_bounds__(PLAN_THREADS, 1) k_rc_plan(Plan P) {
    extern __shared__ unsigned long long plan_smem[];
    unsigned long long *key = plan_smem;                        // [RC_ENTRIES] sort keys
    int *pay = reinterpret_cast<int *>(key + RC_ENTRIES);      // [RC_ENTRIES] entry = 2 w + image
    int *cnt = pay + RC_ENTRIES;                               // [RC_ENTRIES] run starts before each entry
    int *rlen = cnt + RC_ENTRIES;                              // [RC_ENTRIES] chunks of each run, then its first chunk
    int *rhead = rlen + RC_ENTRIES;                            // [RC_ENTRIES] first entry of each run
    int *rtail = rhead + RC_ENTRIES;                           // [RC_ENTRIES] last entry of each run
    int *wsum = rtail + RC_ENTRIES;                            // [72] scan scratch

    const int tid = threadIdx.x;
    // Two CTAs (no row bands): CTA i plans image i's entries alone, its runs
    // never meeting the other image's, and numbers its chunks from
    // i * nwin * nchunks (the most chunks the master entries can need), so
    // neither waits for the other's total.  One CTA: both images.
    const bool split = (gridDim.x == 2);
    const int nent = split ? P.nwin : 2 * P.nwin;
    const int cbase = (split && blockIdx.x == 1) ? P.nwin * P.nchunks : 0;
    const int npx = P.npx, npy = P.npy, rpc = P.rpc;
    int n = 2;
    while (n < nent) n <<= 1;
    const int ns = n > PLAN_THREADS ? n : PLAN_THREADS;   // the entries the loops and scans cover
    for (int e = tid; e < ns; e += PLAN_THREADS) {
        unsigned long long k = ~0ull;             // padding sorts last
        const int ge = split ? 2 * e + (int)blockIdx.x : e;    // the entry: 2 w + image
        if (e < nent) {
            const int w = ge >> 1, img = ge & 1;
            const xcg_loc loc = P.locs[w];
            int local, pidx;
            const PairDev pd = pair_of(P, w, local, pidx);
            const int x0 = img ? loc.x + pd.x_offset - npx / 2 : loc.x - npx / 2;
            const int y0 = img ? loc.y + pd.y_offset + slave_row_shift(pd, loc.y) - npy / 2 : loc.y - npy / 2;
            const int ym = ((y0 % rpc) + rpc) % rpc;
            k = ((unsigned long long)pidx << 49) | ((unsigned long long)img << 48) |
                ((unsigned long long)(x0 + KEY_X_BIAS) << 28) | ((unsigned long long)ym << KEY_Y_BITS) |
                (unsigned long long)(y0 + KEY_Y_BIAS);
        }
        key[e] = k;
        pay[e] = ge;
        rlen[e] = 0;
    }
    __syncthreads();
    // bitonic sort of the first n keys, payload alongside
    for (int kk = 2; kk <= n; kk <<= 1) {
        for (int j = kk >> 1; j > 0; j >>= 1) {
            for (int i = tid; i < n; i += PLAN_THREADS) {
                const int ixj = i ^ j;
                if (ixj > i) {
                    const unsigned long long a = key[i], b = key[ixj];
                    const bool up = (i & kk) == 0;
                    if ((a > b) == up) {
                        key[i] = b; key[ixj] = a;
                        const int t = pay[i]; pay[i] = pay[ixj]; pay[ixj] = t;
                    }
                }
            }
            __syncthreads();
        }
    }
    // a run starts where the group changes or the next patch leaves a gap of rows
    auto is_head = [&](int i) {
        return i == 0 || (key[i] >> KEY_Y_BITS) != (key[i - 1] >> KEY_Y_BITS) || key_y(key[i]) > key_y(key[i - 1]) + npy;
    };
    for (int i = tid; i < ns; i += PLAN_THREADS) cnt[i] = (i < nent && is_head(i)) ? 1 : 0;
    __syncthreads();
    const int nruns = block_exclusive_scan(cnt, wsum, ns);
    for (int i = tid; i < nent; i += PLAN_THREADS) {
        const bool h = is_head(i);
        const int r = cnt[i] + (h ? 0 : -1);
        if (h) rhead[r] = i;
        if (i == nent - 1 || is_head(i + 1)) rtail[r] = i;
    }
    __syncthreads();
    // every patch spans npy rows, so a run ends npy rows below its last entry's first row
    for (int r = tid; r < nruns; r += PLAN_THREADS)
        rlen[r] = (key_y(key[rtail[r]]) - key_y(key[rhead[r]]) + npy) / rpc;
    __syncthreads();
    const int total = block_exclusive_scan(rlen, wsum, ns);   // rlen[r] <- first chunk of run r
    for (int i = tid; i < nent; i += PLAN_THREADS) {
        const int r = cnt[i] + (is_head(i) ? 0 : -1);
        const int c0 = rlen[r] + (key_y(key[i]) - key_y(key[rhead[r]])) / rpc;
        reinterpret_cast<int *>(P.rc_wch)[pay[i]] = cbase + c0;   // rc_wch[w].x for the master, .y for the slave
    }
    // chunk descriptors: one warp per run, its lanes writing consecutive chunks
    {
        const int wp = tid >> 5, l32 = tid & 31;
        for (int r = wp; r < nruns; r += PLAN_THREADS / 32) {
            const unsigned long long k = key[rhead[r]];
            const int pidx = (int)(k >> 49), img = (int)((k >> 48) & 1);
            const int x0 = (int)((k >> 28) & ((1u << 20) - 1)) - KEY_X_BIAS;
            const int y0 = key_y(k);
            const int c0 = rlen[r], c1 = (r + 1 < nruns) ? rlen[r + 1] : total;
            for (int c = c0 + l32; c < c1; c += 32) P.rc_desc[cbase + c] = make_int4(pidx, img, x0, y0 + (c - c0) * rpc);
        }
    }
    if (tid == 0) {
        // chunks of the master entries' numbering, then of the slave's (from nwin * nchunks)
        if (split) {
            P.rc_count[blockIdx.x] = total;
        } else {
            P.rc_count[0] = total;
            P.rc_count[1] = 0;
        }
        if (P.rc_tile_next && blockIdx.x == 0) *P.rc_tile_next = 0;   // the persistent column stage's tile counter
    }
    if (P.rc_nbands > 0) {
        // the chunks listed band by band (order within a band is free).  A
        // chunk belongs to the first band whose end row lies beyond its last
        // row (the last band takes the rest).  Chunk k of a run covers rows
        // y0 + k rpc .. y0 + k rpc + rpc - 1, increasing with k, so each band's
        // chunks are one range of the run, found from the band ends alone:
        // one warp per run counts them, then writes its ranges at offsets
        // taken from per-band counters
        int *bcnt = wsum;                         // [0, 8) counts, [8, 16) fill, [16, 24) starts
        const int nb = P.rc_nbands;
        const int wp = tid >> 5, l32 = tid & 31;
        __syncthreads();                          // wsum free (the scans are done)
        if (tid < 24) wsum[tid] = 0;
        __syncthreads();
        // chunks of a run (first row y0, len chunks) whose last row is below row e
        auto below = [&](long long e, int y0, int len) {
            const long long num = e - (long long)y0 - rpc + 1;     // k rpc < num
            const long long k = (num <= 0) ? 0 : (num + rpc - 1) / rpc;
            return (int)(k < len ? k : len);
        };
        for (int pass = 0; pass < 2; pass++) {
            for (int r = wp; r < nruns; r += PLAN_THREADS / 32) {
                const unsigned long long k = key[rhead[r]];
                const int img = (int)((k >> 48) & 1), y0 = key_y(k);
                const int c0 = rlen[r], len = ((r + 1 < nruns) ? rlen[r + 1] : total) - c0;
                int lo = 0, n = 0;                // lane b < nb: band b's chunks c0 + [lo, lo + n)
                if (l32 < nb) {
                    lo = (l32 == 0) ? 0 : below(P.rc_band_end[img][l32 - 1], y0, len);
                    n = ((l32 == nb - 1) ? len : below(P.rc_band_end[img][l32], y0, len)) - lo;
                }
                if (pass == 0) {
                    if (n > 0) atomicAdd(&bcnt[l32], n);
                } else {
                    const int off = (n > 0) ? bcnt[16 + l32] + atomicAdd(&bcnt[8 + l32], n) : 0;
                    for (int b = 0; b < nb; b++) {
                        const int ob = __shfl_sync(0xffffffffu, off, b);
                        const int lb = __shfl_sync(0xffffffffu, lo, b);
                        const int nn = __shfl_sync(0xffffffffu, n, b);
                        for (int j = l32; j < nn; j += 32) P.rc_order[ob + j] = c0 + lb + j;
                    }
                }
            }
            __syncthreads();
            if (pass == 0 && tid == 0) {
                int acc = 0;
                for (int b = 0; b < nb; b++) { bcnt[16 + b] = acc; P.rc_band_start[b] = acc; acc += bcnt[b]; }
                P.rc_band_start[nb] = acc;
            }
            __syncthreads();
        }
    }
}

// ------------------------------------------------------------------ row stage

// One warp per chunk of rows of one image segment; the structure of k_rows
// (teams of T lanes, the rows t and t + 512 of the chunk through one team,
// rows in registers in the team layout) with one image instead of a window's
// two.  Range interpolation and amplitudes are k_rows' (xcorr.cu:237-250,
// fft_interpolate_routines.cu:76-113, conv_ampl_demean.cu:98-108), the chunk
// sum is h_reduceFD_strip's block sum (conv_ampl_demean.cu:703-726).
template <int N, int LG>
__global__ void __launch_bounds__(128, (N >= 1024) ? 2 : (N >= 512 ? 3 : 4)) k_segrows(Plan P) {
    constexpr int T = fft_lanes(N);
    constexpr int TPW = 32 / T;
    constexpr int PADN = fft_padded_len(N);
    constexpr int RPC = (N >= 1024) ? 1 : 1024 / N;
    constexpr int RPT = (N >= 1024) ? 1 : 2;
    static_assert(RPT * TPW == RPC, "chunk rows");
    constexpr int ACC = (N >= 1024) ? 1024 : 512;
    constexpr int TWL = fft_twiddle_len(N);
    constexpr int PER = N / T;
    constexpr int NH = N / 2;
    constexpr bool HSHIFT = (LG == 1) && (N <= 512);
    constexpr int TWS = (N <= 512) ? 2 * TWL : TWL;
    constexpr int RBP = 32;
    constexpr int GOFF = 32 / TPW;

    extern __shared__ float4 smem_raw[];
    float2 *tw = reinterpret_cast<float2 *>(smem_raw);
    const int warp = threadIdx.x >> 5, l32 = threadIdx.x & 31;
    const int lane = l32 % T;
    const int tm = l32 / T;
    const int team = warp * TPW + tm;
    char *tbase = reinterpret_cast<char *>(tw + TWS) + (size_t)team * (PADN * sizeof(float2) + (2 * N + RBP) * sizeof(float));
    float2 *ex = reinterpret_cast<float2 *>(tbase);
    float *rb = reinterpret_cast<float *>(ex + PADN) + tm * GOFF;
    const int rbx = tm & 1;
    float *const rbE = rb + rbx, *const rbO = rb - rbx;
    float *const rbL = (lane & 1) ? rbO : rbE;
    float *acc = reinterpret_cast<float *>(reinterpret_cast<char *>(tw + TWS) +
                                           (size_t)(blockDim.x / T) * (PADN * sizeof(float2) + (2 * N + RBP) * sizeof(float))) +
                 (size_t)warp * (ACC + RBP);           // [ACC + RBP] first-level sums of the warp's chunk

    for (int i = threadIdx.x; i < TWL; i += blockDim.x) tw[i] = P.tw_row[i];
    if constexpr (HSHIFT)
        for (int i = threadIdx.x; i < TWL; i += blockDim.x) tw[TWL + i] = P.phase[i];
    __syncthreads();

    constexpr int ri = 1 << LG;
    constexpr int KM0 = (LG == 0) ? 0 : PER / (2 * ri), KM1 = (LG == 0) ? PER : 3 * PER / (2 * ri);
    // this launch's chunks: all of them in planned order, or one row band's
    const bool banded = P.rc_nbands > 0;
    const int begin = banded ? P.rc_band_start[P.rc_band] : 0;
    // unbanded: the first planner's chunks, then the second's from nwin * nchunks
    const int cm = banded ? 0 : P.rc_count[0];
    const int end = banded ? P.rc_band_start[P.rc_band + 1] : cm + P.rc_count[1];
    const int cbase = P.nwin * P.nchunks;
    const bool iq16 = (P.format == 0);

    // chunks are taken four per CTA, one per warp; warps share no state
    // between chunks, so a warp that runs out leaves without a barrier
    for (int i = begin + 4 * blockIdx.x + warp; i < end; i += 4 * gridDim.x) {
        const int c = banded ? P.rc_order[i] : (i < cm ? i : cbase + (i - cm));
        const int4 d = P.rc_desc[c];
        const int img = d.y;
        const PairDev *q = P.pairs ? P.pairs + d.x : nullptr;
        const void *base = q ? (img ? q->slave : q->master) : (img ? P.single.slave : P.single.master);
        const int nx = q ? (img ? q->s_nx : q->m_nx) : (img ? P.single.s_nx : P.single.m_nx);
        const int ny = q ? (img ? q->s_ny : q->m_ny) : (img ? P.single.s_ny : P.single.m_ny);
        const int x0 = d.z, y0 = d.w;
        bool oob = false;
        float mn = INFINITY, mx = -INFINITY;

        auto load_row = [&](int r, uint32_t *raw) {
            const int y = y0 + r;
            const bool rowok = (y >= 0 && y < ny);
            const uint32_t *row = reinterpret_cast<const uint32_t *>(base) + (size_t)(rowok ? y : 0) * (size_t)nx;
            if (rowok && x0 >= 0 && x0 + N <= nx) {
#pragma unroll
                for (int m = 0; m < PER; m++) raw[m] = __ldg(row + x0 + lane + T * m);
            } else {
#pragma unroll
                for (int m = 0; m < PER; m++) {
                    const int x = x0 + lane + T * m;
                    if (rowok && x >= 0 && x < nx) raw[m] = __ldg(row + x);
                    else { raw[m] = 0u; oob = true; }
                }
            }
        };
        auto to_complex = [&](const uint32_t *raw, float2 *v) {
            if (iq16) {
#pragma unroll
                for (int m = 0; m < PER; m++) {
                    const short lo = (short)(raw[m] & 0xffffu), hi = (short)(raw[m] >> 16);
                    v[m] = make_float2((float)lo, (float)hi);
                }
            } else {
#pragma unroll
                for (int m = 0; m < PER; m++) v[m] = make_float2(__uint_as_float(raw[m]), 0.f);
            }
        };
        // amplitudes of one row into rb slot s (natural order of the kept fine samples)
        auto amp_row = [&](int s, int r, const uint32_t *raw) {
            float *const rowE = rbE + s * N, *const rowO = rbO + s * N;
            float2 v[PER];
            to_complex(raw, v);
            if (LG == 0) {
                float *const rowL = rbL + s * N;
#pragma unroll
                for (int m = 0; m < PER; m++) rowL[lane + T * m] = hypotf(v[m].x, v[m].y);
                return;
            }
#pragma unroll
            for (int m = KM0; m < KM1; m++) {
                const int k = ((lane + T * m) << LG) - N / 2;
                rowE[k] = amp_of(v[m]);
            }
#pragma unroll 1
            for (int p = 1; p < ri; p++) {
                if (p > 1) {
                    uint32_t again[PER];
                    load_row(r, again);
                    to_complex(again, v);
                }
                team_fft_reg<N, -1>(v, ex, tw, lane);
                if constexpr (HSHIFT) {
                    team_ifft_half_shift<N>(v, ex, tw + TWL, lane);
                } else {
                    const float2 *ph = P.phase + (size_t)(p - 1) * N;
#pragma unroll
                    for (int m = 0; m < PER; m++) v[m] = cmulf(v[m], __ldg(ph + lane + T * m));
                    team_fft_reg<N, +1>(v, ex, tw, lane);
                }
#pragma unroll
                for (int m = KM0; m < KM1; m++) {
                    const int k = ((lane + T * m) << LG) + p - N / 2;
                    ((p & 1) ? rowO : rowE)[k] = amp_of(v[m]);
                }
            }
        };

        uint32_t raw[PER];
        load_row(tm, raw);
#pragma unroll 1
        for (int ir = 0; ir < RPT; ir++) {
            uint32_t cur[PER];
#pragma unroll
            for (int m = 0; m < PER; m++) cur[m] = raw[m];
            if (ir + 1 < RPT) load_row((ir + 1) * TPW + tm, raw);     // in flight during this row
            amp_row(ir, ir * TPW + tm, cur);
        }
        __syncwarp();
        // amplitudes out, first reduction level (rows t and t + 512 of the
        // chunk), extremes, and the FFT input: two real rows in one complex
        // sequence; the slave's rows carry its mask columns [N/4, 3N/4) only
        float *ag = P.rc_amp + (size_t)c * RPC * N;
        float *acc1 = acc + tm * (N + GOFF);
        float2 v[PER];
#pragma unroll
        for (int m = 0; m < PER; m++) {
            const int e = lane + T * m;
            const float a0 = rbL[e];
            const float a1 = (RPT == 2) ? rbL[N + e] : 0.f;
            const bool cin = (m >= PER / 4) && (m < 3 * PER / 4);
            const bool use = (img == 0) || cin;
            // the slave's amplitudes are read only inside its mask columns
            // (the time-correlation window, [xsearch, xsearch + nx_corr))
            if (use) {
                ag[(size_t)tm * N + e] = a0;
                if (RPT == 2) ag[(size_t)(TPW + tm) * N + e] = a1;
            }
            acc1[e] = (RPT == 2) ? a0 + a1 : a0;
            if (use) {
                mn = fminf(mn, a0); mx = fmaxf(mx, a0);
                if (RPT == 2) { mn = fminf(mn, a1); mx = fmaxf(mx, a1); }
            }
            v[m] = use ? make_float2(a0, a1) : make_float2(0.f, 0.f);
        }
        team_fft_reg<N, -1>(v, ex, tw, lane);
        // half spectra k in [0, N/2) of both rows; bin 0 carries (DC, Nyquist),
        // both real for a real row
#pragma unroll
        for (int m = 0; m < PER; m++) ex[fft_pad(lane + T * m)] = v[m];
        __syncwarp();
        float2 *s0 = P.rc_spec + ((size_t)c * RPC + tm) * NH;
        float2 *s1 = P.rc_spec + ((size_t)c * RPC + TPW + tm) * NH;
        const float2 xn = ex[fft_pad(N / 2)];
#pragma unroll
        for (int m = 0; m < PER / 2; m++) {
            const int k = lane + T * m;
            const float2 z1 = v[m];
            if (RPT == 2) {
                float2 A, B;
                if (k == 0) {
                    A = make_float2(z1.x, xn.x);
                    B = make_float2(z1.y, xn.y);
                } else {
                    const float2 z2 = ex[fft_pad(N - k)];
                    A = make_float2(0.5f * (z1.x + z2.x), 0.5f * (z1.y - z2.y));
                    B = make_float2(0.5f * (z1.y + z2.y), -0.5f * (z1.x - z2.x));
                }
                s0[k] = A;
                s1[k] = B;
            } else {
                s0[k] = (k == 0) ? make_float2(z1.x, xn.x) : z1;
            }
        }
        __syncwarp();
        oob = __ballot_sync(0xffffffffu, oob) != 0u;
        // remaining tree levels, strides ACC/2 .. 1 (as k_rows)
        {
            float a[ACC / 32];
#pragma unroll
            for (int qq = 0; qq < ACC / 32; qq++) a[qq] = acc[l32 + 32 * qq + (32 * qq / N) * GOFF];
#pragma unroll
            for (int s = ACC / 64; s >= 1; s >>= 1)
#pragma unroll
                for (int qq = 0; qq < s; qq++) a[qq] = a[qq] + a[qq + s];
            float x = a[0];
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) x = x + __shfl_xor_sync(0xffffffffu, x, o);
            if (l32 == 0) P.rc_part[c] = x;
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            mn = fminf(mn, __shfl_xor_sync(0xffffffffu, mn, o));
            mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
        }
        if (l32 == 0) {
            P.rc_minmax[c] = make_float2(mn, mx);
            P.rc_oob[c] = oob ? 1 : 0;
        }
        __syncwarp();        // acc and rb are reused by the warp's next chunk
    }
}

// ------------------------------------------------------------------ column stage

// k_cols on the cached half spectra: team kx transforms the master's and the
// masked slave's column kx (rows of the window's chunks); kx = 0 holds the
// packed (DC, Nyquist) columns, separated by Hermitian symmetry in ky.  The
// product, demean/mask corrections (conv_ampl_demean.cu:111-139, applied by
// linearity), (-1)^(kx+ky) shift and inverse column FFT of the surface rows
// are k_cols' (do_freq_xcorr.cu:32-64, 106-114).
template <int M, int THR>
__global__ void __launch_bounds__(THR, ColsGeom<M, THR>::BLOCKS) k_cols_rc(Plan P) {
    using G = ColsGeom<M, THR>;
    constexpr int T = G::T, CS = G::CS, CP = G::CP, TWL = G::TWL;
    constexpr int PER = M / T;
    static_assert((CP & (CP - 1)) == 0 && T % 2 == 0, "columns per CTA: a power of two");
    static_assert(THR == 128, "four warps: two partial chunk sums per patch");

    extern __shared__ float4 smem_raw[];
    float2 *tw = reinterpret_cast<float2 *>(smem_raw);
    float2 *cols = tw + TWL;                   // [2*CP + 1][CS]: master, slave, kx = N/2 product
    float2 *boxy = cols + (2 * CP + 1) * CS;    // [M] DFT of the row mask
    float2 *boxx = boxy + M;                    // [CP + 1] DFT of the column mask at this CTA's kx, then N/2
    double *dsum = reinterpret_cast<double *>(boxx + CP + 1);   // [4] per-warp partial chunk sums

    const int w = blockIdx.y, b = blockIdx.x;
    const int N = P.npx, NH = N / 2;
    const int kx0 = b * CP;
    const int warp = threadIdx.x >> 5, l32 = threadIdx.x & 31;
    const int lane = l32 % T;
    const int team = warp * (32 / T) + l32 / T;
    const int2 wc = P.rc_wch[w];
    const float2 *ms = P.rc_spec + (size_t)wc.x * P.rpc * NH;   // window's master rows, stride NH
    const float2 *ss = P.rc_spec + (size_t)wc.y * P.rpc * NH;   // window's slave rows

    for (int i = threadIdx.x; i < TWL; i += blockDim.x) tw[i] = P.tw_col[i];
    {   // thread t stages slot t % CP for rows t / CP + k * THR/CP: the slave's
        // mask rows [M/4, 3M/4) first (zeros elsewhere), then the master
        constexpr int RSTEP = THR / CP;
        constexpr int NLD = M / RSTEP;
        const int sl = threadIdx.x % CP, row0 = threadIdx.x / CP;
        float2 *sslot = cols + (CP + sl) * CS, *mslot = cols + sl * CS;
#pragma unroll 8
        for (int k = 0; k < NLD; k++) {
            const int r = row0 + k * RSTEP;
            if (r >= M / 4 && r < 3 * M / 4) cp_async8(sslot + fft_pad(r), ss + (size_t)r * NH + kx0 + sl);
            else sslot[fft_pad(r)] = make_float2(0.f, 0.f);
        }
        cp_async_commit();
#pragma unroll 8
        for (int k = 0; k < NLD; k++) {
            const int r = row0 + k * RSTEP;
            cp_async8(mslot + fft_pad(r), ms + (size_t)r * NH + kx0 + sl);
        }
        cp_async_commit();
    }
    // the mask spectra this CTA uses, staged once (per-element reads missed
    // the L1 left beside the column slots)
    for (int i = threadIdx.x; i < M; i += THR) boxy[i] = __ldg(P.box_y + i);
    if (threadIdx.x <= CP) boxx[threadIdx.x] = __ldg(P.box_x + (threadIdx.x < CP ? kx0 + threadIdx.x : NH));
    {
        // patch means (conv_ampl_demean.cu:719-724) from the chunk sums,
        // warps 0-1 the master's, 2-3 the slave's: the FP32 chunk sums of a
        // patch are exact in double, so any order gives the reference's bits
        const int nch = P.nchunks;
        const int base = (warp < 2) ? wc.x : wc.y;
        double sp = 0.0;
        for (int i = (warp & 1) * 32 + l32; i < nch; i += 64) sp += (double)P.rc_part[base + i];
        sp = warp_sum_f64(sp);
        if (l32 == 0) dsum[warp] = sp;
    }
    cp_async_wait<1>();                          // slave columns in (this thread's copies)
    __syncthreads();                             // ... and everyone's
    float dc1, m2;
    {
        const double inv = pow2_inv(N * M);
        const double s1 = (dsum[0] + dsum[1]) * inv, s2 = (dsum[2] + dsum[3]) * inv;
        dc1 = (float)(s1 * (double)N * (double)M);   // the master's DC term, m1 N M
        m2 = (float)s2;
        if (b == 0 && threadIdx.x == 0) { P.means[2 * w] = s1; P.means[2 * w + 1] = s2; }
    }

    const int kx = kx0 + team;
    float2 *a = cols + team * CS;               // master column, later the result
    float2 *pa = cols + (CP + team) * CS;       // slave column
    float2 z[PER];
#pragma unroll
    for (int m = 0; m < PER; m++) z[m] = pa[fft_pad(lane + T * m)];
    __syncwarp();
    team_fft_reg_mid<M, -1>(z, pa, tw, lane);    // zero outside the mask rows
#pragma unroll
    for (int m = 0; m < PER; m++) pa[fft_pad(lane + T * m)] = z[m];
    cp_async_wait<0>();                          // master columns in
    __syncthreads();
#pragma unroll
    for (int m = 0; m < PER; m++) z[m] = a[fft_pad(lane + T * m)];
    __syncwarp();
    team_fft_reg<M, -1>(z, a, tw, lane);
#pragma unroll
    for (int m = 0; m < PER; m++) a[fft_pad(lane + T * m)] = z[m];
    __syncwarp();

    // the kx = 0 team also emits column N/2 (its product goes through the
    // extra slot first); the trip count stays warp-uniform because
    // team_fft_reg synchronises the whole warp
    const bool dc = (kx == 0);
    const int nout = __any_sync(0xffffffffu, dc) ? 2 : 1;
    float2 *xs = cols + 2 * CP * CS;
    auto product = [&](int kxx, float2 A1, float2 A2, int ky) {
        if (kxx == 0 && ky == 0) A1.x -= dc1;
        const float2 bm = cmulf(boxx[kxx == NH ? CP : kxx - kx0], boxy[ky]);
        A2.x -= m2 * bm.x;
        A2.y -= m2 * bm.y;
        float2 pr = cmulf_conj(A1, A2);
        if ((kxx + ky) & 1) { pr.x = -pr.x; pr.y = -pr.y; }
        return pr;
    };
#pragma unroll 1
    for (int o = 0; o < nout; o++) {
        if (o == 0) {
#pragma unroll
            for (int m = 0; m < PER; m++) {
                const int ky = lane + T * m;
                const float2 zm = a[fft_pad(ky)], zs = pa[fft_pad(ky)];
                if (!dc) {
                    z[m] = product(kx, zm, zs, ky);
                } else {
                    // columns kx = 0 and N/2 from the packed (DC, Nyquist) column
                    const int kyn = (M - ky) & (M - 1);
                    const float2 wm = a[fft_pad(kyn)], ws = pa[fft_pad(kyn)];
                    const float2 D1 = make_float2(0.5f * (zm.x + wm.x), 0.5f * (zm.y - wm.y));
                    const float2 D2 = make_float2(0.5f * (zs.x + ws.x), 0.5f * (zs.y - ws.y));
                    const float2 Q1 = make_float2(0.5f * (zm.y + wm.y), -0.5f * (zm.x - wm.x));
                    const float2 Q2 = make_float2(0.5f * (zs.y + ws.y), -0.5f * (zs.x - ws.x));
                    z[m] = product(0, D1, D2, ky);
                    xs[fft_pad(ky)] = product(NH, Q1, Q2, ky);
                }
            }
        } else {
#pragma unroll
            for (int m = 0; m < PER; m++) z[m] = xs[fft_pad(lane + T * m)];
        }
        float2 *dst = (o == 0) ? a : pa;
        __syncwarp();                            // every lane has read a, pa and xs before dst is reused
        team_fft_reg<M, +1>(z, dst, tw, lane);
#pragma unroll
        for (int m = PER / 4; m < 3 * PER / 4; m++) dst[fft_pad(lane + T * m)] = z[m];
        __syncwarp();
    }
    __syncthreads();
    // rows y in [ysearch, ysearch + nyc) of the half spectrum, kx <= N/2
    {
        constexpr int RS = THR / CP;
        float2 *qw = P.qspec + (size_t)w * P.nyc * P.qpitch;
        const int s = threadIdx.x % CP, y0 = threadIdx.x / CP;
        float2 *dstq = qw + (size_t)y0 * P.qpitch + kx0 + s;
        const float2 *srcc = cols + s * CS;
        for (int k = 0; k < (M / 2) / RS; k++) {
            const int sy = (RS % 16 == 0) ? fft_pad(y0 + M / 4) + k * (RS + RS / 16) : fft_pad(y0 + M / 4 + k * RS);
            dstq[(size_t)k * RS * P.qpitch] = srcc[sy];
        }
        if (b == 0)                                // column N/2: the kx = 0 team's slave slot
            for (int yq = threadIdx.x; yq < M / 2; yq += blockDim.x)
                qw[(size_t)yq * P.qpitch + NH] = cols[CP * CS + fft_pad(yq + M / 4)];
    }
}

// The column stage as a persistent, software-pipelined kernel (the default;
// k_cols_rc above is one CTA per tile).  A tile is (window, group of CP
// columns); CTAs take tiles a quarter window at a time from a counter, so a
// CTA's consecutive tiles are mostly the next column groups of one window:
// the twiddles and the row mask's spectrum are staged once per CTA and the
// patch means once per run of a window's tiles.  Per tile: the slave's mask
// rows (staged during the previous tile's inverse transform) are
// transformed first, then the master's (staged during the previous tile's
// copy-out and the slave transform); the master's spectrum stays in
// registers for the product, after which the slave slots are free and the
// next tile's slave rows are requested.  Rows outside the slave's mask are
// zero in registers, never staged, and the slave's first FFT pass skips
// their butterflies.  The arithmetic is k_cols_rc's, operation for
// operation, so the results are the same bits.  Tiles of column group 0 (the
// packed DC/Nyquist column, whose second output goes through the slave slot)
// request the next tile's slave rows only after their copy-out.
// KEEP: the slave's column spectrum stays in registers for the product
// (one CTA per SM fewer; the default form up to 256-point columns).
template <int M, int THR, bool KEEP>
__global__ void __launch_bounds__(THR, KEEP ? ColsGeom<M, THR>::BLOCKS - 1 : ColsGeom<M, THR>::BLOCKS)
k_cols_rcp(Plan P) {
    using G = ColsGeom<M, THR>;
    constexpr int T = G::T, CS = G::CS, CP = G::CP, TWL = G::TWL;
    constexpr int PER = M / T;
    constexpr int RSTEP = THR / CP;            // rows a staging pass covers
    static_assert((CP & (CP - 1)) == 0 && T % 2 == 0, "columns per CTA: a power of two");
    static_assert(THR == 128, "four warps: two partial chunk sums per patch");
    static_assert(PER % 4 == 0 && (M / 2) % RSTEP == 0, "mask rows: whole registers and staging passes");

    extern __shared__ float4 smem_raw[];
    float2 *tw = reinterpret_cast<float2 *>(smem_raw);
    float2 *cols = tw + TWL;                   // [2*CP + 1][CS]: master, slave, kx = N/2 product
    float2 *boxy = cols + (2 * CP + 1) * CS;    // [M] DFT of the row mask
    float2 *boxx = boxy + M;                    // [CP + 1] DFT of the column mask at this tile's kx, then N/2
    double *dsum = reinterpret_cast<double *>(boxx + CP + 1);   // [4] per-warp partial chunk sums
    int *grab = reinterpret_cast<int *>(dsum + 4);              // [1] the next chunk of tiles (thread 0's grab)

    const int N = P.npx, NH = N / 2;
    const int NG = NH / CP;                     // column groups per window
    const int ntiles = P.nwin * NG;
    // Tiles come in chunks of a quarter window from a counter the planner
    // zeroed (a CTA that starts late, behind the other batch's kernels, takes
    // fewer), or, without the counter, as one contiguous range per CTA.
    const bool dyn = (P.rc_tile_next != nullptr);
    const int K = (NG >= 4) ? NG / 4 : 1;
    int t, tend;                                // the current chunk [t, tend)
    if (dyn) {
        if (threadIdx.x == 0) *grab = atomicAdd(P.rc_tile_next, K);
        __syncthreads();
        t = *grab;
        __syncthreads();                        // every thread has read it before the next grab
    } else {
        t = (int)((long long)ntiles * blockIdx.x / gridDim.x);
        tend = (int)((long long)ntiles * (blockIdx.x + 1) / gridDim.x);
        if (t >= tend) return;
    }
    if (dyn) {
        if (t >= ntiles) return;
        tend = min(t + K, ntiles);
    }
    const int warp = threadIdx.x >> 5, l32 = threadIdx.x & 31;
    const int lane = l32 % T;
    const int team = warp * (32 / T) + l32 / T;
    const int sl = threadIdx.x % CP, row0 = threadIdx.x / CP;   // staging: slot, first row
    // tile t: window t / NG, column group t % NG (a CTA's consecutive tiles
    // are the next column groups of one window; taking the next windows at
    // one column group instead, so that windows sharing row chunks read them
    // at about the same time, was 29% slower: the means on every tile)
    auto tile = [&](int t, int &w, int &b) { w = t / NG; b = t - w * NG; };

    // tile t's slave mask rows [M/4, 3M/4) / master rows, into the slots (one commit group each)
    auto stage_slave = [&](int t) {
        int w, b;
        tile(t, w, b);
        const int kx0 = b * CP;
        const float2 *src = P.rc_spec + (size_t)P.rc_wch[w].y * P.rpc * NH + kx0 + sl;
        float2 *slot = cols + (CP + sl) * CS;
#pragma unroll 8
        for (int k = 0; k < (M / 2) / RSTEP; k++) {
            const int r = M / 4 + row0 + k * RSTEP;
            cp_async8(slot + fft_pad(r), src + (size_t)r * NH);
        }
        cp_async_commit();
    };
    auto stage_master = [&](int t) {
        int w, b;
        tile(t, w, b);
        const int kx0 = b * CP;
        const float2 *src = P.rc_spec + (size_t)P.rc_wch[w].x * P.rpc * NH + kx0 + sl;
        float2 *slot = cols + sl * CS;
#pragma unroll 8
        for (int k = 0; k < M / RSTEP; k++) {
            const int r = row0 + k * RSTEP;
            cp_async8(slot + fft_pad(r), src + (size_t)r * NH);
        }
        cp_async_commit();
    };

    stage_slave(t);
    stage_master(t);
    for (int i = threadIdx.x; i < TWL; i += THR) tw[i] = P.tw_col[i];
    for (int i = threadIdx.x; i < M; i += THR) boxy[i] = __ldg(P.box_y + i);

    int cur_w = -1;
    float dc1 = 0.f, m2 = 0.f;
    for (;;) {
        int w, b;
        tile(t, w, b);
        // the last tile of a chunk: the next chunk, read after the barrier below
        if (dyn && t + 1 == tend && threadIdx.x == 0) *grab = atomicAdd(P.rc_tile_next, K);
        const int kx0 = b * CP;
        const bool neww = (w != cur_w);
        // (the previous tile's last barrier ordered every read of boxx and dsum before these writes)
        if (threadIdx.x <= CP) boxx[threadIdx.x] = __ldg(P.box_x + (threadIdx.x < CP ? kx0 + threadIdx.x : NH));
        if (neww) {
            // patch means from the chunk sums (conv_ampl_demean.cu:719-724),
            // warps 0-1 the master's, 2-3 the slave's (exact in double: any order)
            const int2 wc = P.rc_wch[w];
            const int base = (warp < 2) ? wc.x : wc.y;
            double sp = 0.0;
            for (int i = (warp & 1) * 32 + l32; i < P.nchunks; i += 64) sp += (double)P.rc_part[base + i];
            sp = warp_sum_f64(sp);
            if (l32 == 0) dsum[warp] = sp;
        }
        cp_async_wait<1>();                      // this tile's slave rows in (this thread's copies)
        __syncthreads();                         // ... and everyone's; boxx, dsum, tw, boxy, grab written
        int tn = -1;                             // the next tile, none: -1
        if (t + 1 < tend) tn = t + 1;
        else if (dyn && *grab < ntiles) tn = *grab;
        if (neww) {
            const double inv = pow2_inv(N * M);
            const double s1 = (dsum[0] + dsum[1]) * inv, s2 = (dsum[2] + dsum[3]) * inv;
            dc1 = (float)(s1 * (double)N * (double)M);
            m2 = (float)s2;
            if (b == 0 && threadIdx.x == 0) { P.means[2 * w] = s1; P.means[2 * w + 1] = s2; }
            cur_w = w;
        }

        const int kx = kx0 + team;
        float2 *a = cols + team * CS;            // master column, later the result
        float2 *pa = cols + (CP + team) * CS;    // slave column
        float2 z[PER];
#pragma unroll
        for (int m = 0; m < PER; m++)
            z[m] = (m >= PER / 4 && m < 3 * PER / 4) ? pa[fft_pad(lane + T * m)] : make_float2(0.f, 0.f);
        __syncwarp();
        team_fft_reg_mid<M, -1>(z, pa, tw, lane);    // zero outside the mask rows
        float2 zs[KEEP ? PER : 1];
        if constexpr (KEEP) {
#pragma unroll
            for (int m = 0; m < PER; m++) zs[m] = z[m];
        }
        if (!KEEP || b == 0) {                   // column group 0 splits the packed column from the slot
#pragma unroll
            for (int m = 0; m < PER; m++) pa[fft_pad(lane + T * m)] = z[m];
        }
        cp_async_wait<0>();                      // master rows in
        __syncthreads();
#pragma unroll
        for (int m = 0; m < PER; m++) z[m] = a[fft_pad(lane + T * m)];
        __syncwarp();
        team_fft_reg<M, -1>(z, a, tw, lane);

        auto product = [&](int kxx, float2 A1, float2 A2, int ky) {
            if (kxx == 0 && ky == 0) A1.x -= dc1;
            const float2 bm = cmulf(boxx[kxx == NH ? CP : kxx - kx0], boxy[ky]);
            A2.x -= m2 * bm.x;
            A2.y -= m2 * bm.y;
            float2 pr = cmulf_conj(A1, A2);
            if ((kxx + ky) & 1) { pr.x = -pr.x; pr.y = -pr.y; }
            return pr;
        };
        // the product of column kx: from the master spectrum in registers, or
        // in column group 0 (CTA-uniform) through the master slot, where the
        // kx = 0 team splits the packed (DC, Nyquist) column and puts column
        // N/2's product in the extra slot
        const bool dc = (kx == 0);
        const int nout = (b == 0 && __any_sync(0xffffffffu, dc)) ? 2 : 1;    // warp-uniform
        float2 *xs = cols + 2 * CP * CS;
        if (b != 0) {
#pragma unroll
            for (int m = 0; m < PER; m++) {
                const int ky = lane + T * m;
                if constexpr (KEEP) z[m] = product(kx, z[m], zs[m], ky);
                else z[m] = product(kx, z[m], pa[fft_pad(ky)], ky);
            }
        } else {
#pragma unroll
            for (int m = 0; m < PER; m++) a[fft_pad(lane + T * m)] = z[m];
            __syncwarp();
#pragma unroll
            for (int m = 0; m < PER; m++) {
                const int ky = lane + T * m;
                const float2 zm = a[fft_pad(ky)], zs = pa[fft_pad(ky)];
                if (!dc) {
                    z[m] = product(kx, zm, zs, ky);
                } else {
                    const int kyn = (M - ky) & (M - 1);
                    const float2 wm = a[fft_pad(kyn)], ws = pa[fft_pad(kyn)];
                    const float2 D1 = make_float2(0.5f * (zm.x + wm.x), 0.5f * (zm.y - wm.y));
                    const float2 D2 = make_float2(0.5f * (zs.x + ws.x), 0.5f * (zs.y - ws.y));
                    const float2 Q1 = make_float2(0.5f * (zm.y + wm.y), -0.5f * (zm.x - wm.x));
                    const float2 Q2 = make_float2(0.5f * (zs.y + ws.y), -0.5f * (zs.x - ws.x));
                    z[m] = product(0, D1, D2, ky);
                    xs[fft_pad(ky)] = product(NH, Q1, Q2, ky);
                }
            }
        }
        __syncthreads();                         // every team has read its slave column
        // outside column group 0 the slave slots are free: the next tile's slave rows
        if (b != 0 && tn >= 0) stage_slave(tn);
        // inverse of column kx into its master slot; in column group 0 the
        // kx = 0 team's second output, column N/2, into its slave slot (one
        // call site of the transform for both cases)
#pragma unroll 1
        for (int o = 0; o < nout; o++) {
            if (o == 1) {
#pragma unroll
                for (int m = 0; m < PER; m++) z[m] = xs[fft_pad(lane + T * m)];
            }
            float2 *dst = (o == 0) ? a : pa;
            __syncwarp();
            team_fft_reg<M, +1>(z, dst, tw, lane);
#pragma unroll
            for (int m = PER / 4; m < 3 * PER / 4; m++) dst[fft_pad(lane + T * m)] = z[m];
            __syncwarp();
        }
        __syncthreads();
        {   // rows y in [ysearch, ysearch + nyc) of the half spectrum, kx <= N/2
            constexpr int RS = THR / CP;
            float2 *qw = P.qspec + (size_t)w * P.nyc * P.qpitch;
            float2 *dstq = qw + (size_t)row0 * P.qpitch + kx0 + sl;
            const float2 *srcc = cols + sl * CS;
            for (int k = 0; k < (M / 2) / RS; k++) {
                const int sy = (RS % 16 == 0) ? fft_pad(row0 + M / 4) + k * (RS + RS / 16)
                                              : fft_pad(row0 + M / 4 + k * RS);
                dstq[(size_t)k * RS * P.qpitch] = srcc[sy];
            }
            if (b == 0)
                for (int yq = threadIdx.x; yq < M / 2; yq += THR)
                    qw[(size_t)yq * P.qpitch + NH] = cols[CP * CS + fft_pad(yq + M / 4)];
        }
        __syncthreads();                         // the slots are read: the next tile's rows may land
        if (tn < 0) break;
        if (b == 0) stage_slave(tn);
        stage_master(tn);
        if (tn != t + 1) tend = min(tn + K, ntiles);
        t = tn;
    }
}

// ------------------------------------------------------------------ launchers

static size_t rc_plan_smem_bytes() {
    return (size_t)RC_ENTRIES * (sizeof(unsigned long long) + 5 * sizeof(int)) + 72 * sizeof(int);
}
template <int N>
static size_t segrows_smem() {
    constexpr int T = fft_lanes(N);
    constexpr int ACC = (N >= 1024) ? 1024 : 512;
    const int teams = 128 / T;
    return fft_twiddle_len(N) * (N <= 512 ? 2 : 1) * sizeof(float2) +
           (size_t)teams * (fft_padded_len(N) * sizeof(float2) + (2 * N + 32) * sizeof(float)) +
           (size_t)(128 / 32) * (ACC + 32) * sizeof(float);
}
template <int M>
static size_t cols_rc_smem() {
    using G = ColsGeom<M, 128>;
    return G::TWL * sizeof(float2) + (size_t)(2 * G::CP + 1) * G::CS * sizeof(float2) +
           (size_t)(M + G::CP + 1) * sizeof(float2) + 4 * sizeof(double) + 16;
}

template <int N>
static cudaError_t setup_segrows_t() {
    cudaError_t e = cudaSuccess;
    auto set = [&](auto kern) {
        if (e == cudaSuccess) e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)segrows_smem<N>());
    };
    set(k_segrows<N, 0>); set(k_segrows<N, 1>); set(k_segrows<N, 2>); set(k_segrows<N, 3>);
    return e;
}
template <int M>
static cudaError_t setup_cols_rc_t() {
    cudaError_t e = cudaFuncSetAttribute(k_cols_rc<M, 128>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)cols_rc_smem<M>());
    if (e) return e;
    e = cudaFuncSetAttribute(k_cols_rcp<M, 128, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)cols_rc_smem<M>());
    if (e) return e;
    return cudaFuncSetAttribute(k_cols_rcp<M, 128, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)cols_rc_smem<M>());
}

cudaError_t segrows_setup(const Plan &P) {
    cudaError_t e = cudaFuncSetAttribute(k_rc_plan, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)rc_plan_smem_bytes());
    if (e) return e;
    switch (P.npx) {
        case 64: e = setup_segrows_t<64>(); break;
        case 128: e = setup_segrows_t<128>(); break;
        case 256: e = setup_segrows_t<256>(); break;
        case 512: e = setup_segrows_t<512>(); break;
        case 1024: e = setup_segrows_t<1024>(); break;
        default: return cudaErrorInvalidValue;
    }
    if (e) return e;
    switch (P.npy) {
        case 64: return setup_cols_rc_t<64>();
        case 128: return setup_cols_rc_t<128>();
        case 256: return setup_cols_rc_t<256>();
        case 512: return setup_cols_rc_t<512>();
        case 1024: return setup_cols_rc_t<1024>();
    }
    return cudaErrorInvalidValue;
}

size_t rc_max_chunks(int npx, int npy, int nwin) {
    const int rpc = npx >= 1024 ? 1 : 1024 / npx;
    return (size_t)2 * nwin * (size_t)(npy / rpc);
}

void launch_rc_plan(const Plan &P, cudaStream_t s) {
    // one CTA per image unless the host entry wants the chunks listed by row band
    k_rc_plan<<<P.rc_nbands > 0 ? 1 : 2, PLAN_THREADS, rc_plan_smem_bytes(), s>>>(P);
}

template <int N>
static void launch_segrows_t(const Plan &P, cudaStream_t s) {
    // a grid-stride walk over the planned chunks, four per CTA; the grid is
    // sized for the chunks the batch would have without sharing, capped at
    // the CTAs that fit the GPU at once several times over
    int dev = 0, sms = 148;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const size_t maxq = (rc_max_chunks(P.npx, P.npy, P.nwin) + 3) / 4;
    const int per_sm = (N >= 1024) ? 2 : (N >= 512 ? 3 : 4);
    // a band's launch takes a share of the chunks: a smaller grid
    const size_t cap = (size_t)sms * per_sm * (P.rc_nbands > 0 ? 2 : 8);
    const int grid = (int)((maxq < cap) ? maxq : cap);
    switch (P.log2ri) {
        case 0: k_segrows<N, 0><<<grid, 128, segrows_smem<N>(), s>>>(P); break;
        case 1: k_segrows<N, 1><<<grid, 128, segrows_smem<N>(), s>>>(P); break;
        case 2: k_segrows<N, 2><<<grid, 128, segrows_smem<N>(), s>>>(P); break;
        default: k_segrows<N, 3><<<grid, 128, segrows_smem<N>(), s>>>(P); break;
    }
}
void launch_segrows(const Plan &P, cudaStream_t s) {
    switch (P.npx) {
        case 64: launch_segrows_t<64>(P, s); break;
        case 128: launch_segrows_t<128>(P, s); break;
        case 256: launch_segrows_t<256>(P, s); break;
        case 512: launch_segrows_t<512>(P, s); break;
        case 1024: launch_segrows_t<1024>(P, s); break;
    }
}

template <int M>
static void launch_cols_rc_t(const Plan &P, cudaStream_t s) {
    using G = ColsGeom<M, 128>;
    const int ntiles = ((P.npx / 2) / G::CP) * P.nwin;
    if (P.cols_cfg == 1) {                       // one CTA per tile
        dim3 grid((P.npx / 2) / G::CP, P.nwin);
        k_cols_rc<M, 128><<<grid, 128, cols_rc_smem<M>(), s>>>(P);
        return;
    }
    // persistent: one CTA per resident slot, tiles split into contiguous
    // ranges (leaving one slot per SM to the other batch's kernels measured
    // the same on the device entry and slower on the host entry)
    int dev = 0, sms = 148;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    // the slave spectrum kept in registers (one CTA per SM fewer): the
    // default up to 256 points (0.454 against 0.481 ms per 1000 windows of
    // 128 x 128), not beyond (full frame 72.4 against 69.5 ms); launch
    // shape 2 takes the other form
    const bool keep = (P.cols_cfg == 2) != (M <= 256);
    if (keep && G::BLOCKS > 1) {
        const int grid = std::min(ntiles, sms * (G::BLOCKS - 1));
        k_cols_rcp<M, 128, true><<<grid, 128, cols_rc_smem<M>(), s>>>(P);
        return;
    }
    const int grid = std::min(ntiles, sms * G::BLOCKS);
    k_cols_rcp<M, 128, false><<<grid, 128, cols_rc_smem<M>(), s>>>(P);
}
void launch_cols_rc(const Plan &P, cudaStream_t s) {
    switch (P.npy) {
        case 64: launch_cols_rc_t<64>(P, s); break;
        case 128: launch_cols_rc_t<128>(P, s); break;
        case 256: launch_cols_rc_t<256>(P, s); break;
        case 512: launch_cols_rc_t<512>(P, s); break;
        case 1024: launch_cols_rc_t<1024>(P, s); break;
    }
}

}  // namespace xcg
