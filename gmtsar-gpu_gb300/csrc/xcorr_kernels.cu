// The four kernels of the xcorr frequency-domain path on sm_103a.
//
//   k_rows   per 1024-sample chunk of rows: patch staging from the SLC
//            images (int16 I/Q or float32), range interpolation, amplitude,
//            the reference's FP32 chunk sums, and the forward row FFT of the
//            packed real pair a1 + i*a2*mask.
//   k_cols   per group of column pairs (kx, N-kx): forward column FFTs,
//            Hermitian split into the two patch spectra, mean correction,
//            conjugate product with the (-1)^(kx+ky) shift, inverse column FFT
//            of the half spectrum kx <= N/2 for the surface rows only.
//   k_peak   per window: inverse row FFTs (two real rows per complex FFT),
//            |.| surface, integer argmax with the reference's tie rules,
//            surface means, the int64 time-domain correlation at the peak,
//            normalisation and the 8x8 neighbourhood ^0.25.
//   k_subpix per window: separable zero-pad interpolation of the 8x8 block
//            as two small dense operators and the argmax of the real part.
//
// Every kernel cites the reference stages it replaces.
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include <type_traits>

#include "kernel_util.cuh"
#include "team_fft.cuh"
#include "xcorr_kernels.cuh"


namespace xcg {


// ---------------------------------------------------------------- helpers

__device__ __forceinline__ unsigned bitrev11(unsigned e) { return __brev(e) >> 21; }

// Sortable argmax key with the reference's tie rules (reduce6b / reduce6bC,
// conv_ampl_demean.cu:227-346,434-554, host finish :655-673,739-754): a
// thread starts from value 0 at the first element of its pair and takes a
// later element only if strictly greater; tree levels keep the lower thread
// on ties; the host keeps the earliest block.  Net effect: the winner has the
// largest effective value, ties to the smallest (block, bit-reversed local
// index); an element that is not > 0 counts as 0 in the first half of its
// 2048-element block and never wins in the second half.
__device__ __forceinline__ unsigned long long argmax_key(float v, unsigned e) {
    const unsigned local = e & 2047u;
    unsigned ord;
    if (v > 0.f) ord = __float_as_uint(v) + 1u;
    else ord = (local < 1024u) ? 1u : 0u;          // 0.0f -> 1, "never" -> 0
    const unsigned key = ((e >> 11) << 11) | bitrev11(local);
    return ((unsigned long long)ord << 32) | (0xffffffffu - key);
}
__device__ __forceinline__ unsigned argmax_index(unsigned long long k) {
    const unsigned key = 0xffffffffu - (unsigned)(k & 0xffffffffu);
    return ((key >> 11) << 11) | bitrev11(key & 2047u);
}
__device__ __forceinline__ float argmax_value(unsigned long long k) {
    const unsigned ord = (unsigned)(k >> 32);
    return ord <= 1u ? 0.f : __uint_as_float(ord - 1u);
}

// best = max(best, argmax_key(v, e)), the key built only where it can win.
// Keys order by their value word first, and every positive value's word
// (its bits + 1) is above the words of zero, negative and NaN values (0 or 1),
// so once best holds a positive value, a value below it cannot win; bestv is
// that value, or -inf while best holds none (then every key is built).
__device__ __forceinline__ void argmax_update(unsigned long long &best, float &bestv, float v, unsigned e) {
    if (!(v < bestv)) {
        const unsigned long long k = argmax_key(v, e);
        if (k > best) {
            best = k;
            bestv = ((unsigned)(k >> 32) >= 2u) ? argmax_value(k) : -INFINITY;
        }
    }
}

__device__ __forceinline__ unsigned long long warp_max_u64(unsigned long long v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        unsigned long long u = __shfl_xor_sync(0xffffffffu, v, o);
        v = u > v ? u : v;
    }
    return v;
}
__device__ __forceinline__ long long warp_sum_i64(long long v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

__device__ __forceinline__ float2 load_sample(const Plan &P, const void *img, int nx, int ny, int x, int y, bool &oob) {
    if (x < 0 || y < 0 || x >= nx || y >= ny) { oob = true; return make_float2(0.f, 0.f); }
    const size_t i = (size_t)y * (size_t)nx + (size_t)x;
    if (P.format == 0) {
        const short2 s = __ldg(reinterpret_cast<const short2 *>(img) + i);
        return make_float2((float)s.x, (float)s.y);
    }
    return make_float2(__ldg(reinterpret_cast<const float *>(img) + i), 0.f);
}


// ---------------------------------------------------------------- k_rows
// Replaces read_xcorr_data + the H2D patch cut (xcorr.cu:326-338), range
// interpolation (xcorr.cu:237-250, fft_interpolate_routines.cu:76-113),
// d_conv_ampl_strip (conv_ampl_demean.cu:98-108), h_reduceFD_strip (:703-726),
// the demean/mask of d_mean_mask_strip (:111-139, applied in k_cols by
// linearity) and the row half of the forward 2-D FFT (do_freq_xcorr.cu:99-101).
//
// Range interpolation: the reference pads the N-point spectrum to M = ri*N and
// keeps fine samples m in [N/2, 3N/2).  Fine sample m = ri*q + p equals the
// N-point inverse FFT of X[f]*exp(2 pi i f' p / M) / N at q (f' = f or f-N);
// for p = 0 that is the input sample x[q] itself.  So one forward FFT and
// ri-1 inverse FFTs of length N give every kept sample.
//
// A warp owns one 1024-sample chunk (1024/N rows) of one window; its teams of
// T lanes take the chunk's rows in turn, so the two rows that the reference's
// first reduction level adds (t and t+512) go through the same team and their
// sum is the only chunk-sum state kept in shared memory.  Rows live in
// registers in the team layout (lane l: samples l + T*m); the next row's
// samples are loaded while the current one is transformed.
template <int N, int LG>
__global__ void __launch_bounds__(128, (N >= 1024) ? 2 : (N >= 512 ? 3 : 4)) k_rows(Plan P) {
    constexpr int T = fft_lanes(N);
    constexpr int TPW = 32 / T;
    constexpr int PADN = fft_padded_len(N);
    constexpr int RPC = (N >= 1024) ? 1 : 1024 / N;     // rows per 1024-sample chunk
    constexpr int RPT = (N >= 1024) ? 1 : 2;            // rows per team: t and t+512
    static_assert(RPT * TPW == RPC, "chunk rows");
    constexpr int ACC = (N >= 1024) ? 1024 : 512;       // first-level sums per patch
    constexpr int TWL = fft_twiddle_len(N);
    constexpr int PER = N / T;

    // ri = 2 rows of up to 256 points: the phase of the interpolation rides
    // on a second twiddle table (team_ifft_half_shift)
    constexpr bool HSHIFT = (LG == 1) && (N <= 512);
    constexpr int TWS = (N <= 512) ? 2 * TWL : TWL;     // twiddle entries in shared memory

    extern __shared__ float4 smem_raw[];
    float2 *tw = reinterpret_cast<float2 *>(smem_raw);
    const int warp = threadIdx.x >> 5, l32 = threadIdx.x & 31;
    const int lane = l32 % T;
    const int tm = l32 / T;                             // team within the warp
    const int team = warp * TPW + tm;
    // The teams of a warp touch their amplitude rows and first-level sums
    // with the same instruction; team tm's copies sit GOFF*tm words further
    // on, and its amplitude rows are stored with index bit 0 flipped when tm
    // is odd, so both the stride-2 interleaved stores of the interpolation
    // and the lane-order loads hit distinct banks across the warp.
    constexpr int RBP = 32;                             // padding words per team / per patch
    constexpr int GOFF = 32 / TPW;
    char *tbase = reinterpret_cast<char *>(tw + TWS) + (size_t)team * (PADN * sizeof(float2) + (2 * N + RBP) * sizeof(float));
    float2 *ex = reinterpret_cast<float2 *>(tbase);
    float *rb = reinterpret_cast<float *>(ex + PADN) + tm * GOFF;    // [2][N] amplitudes, index i at i ^ (tm & 1)
    // i ^ (tm & 1) is i + 1 or i - 1 by the parity of i: one base pointer per
    // parity keeps the offsets of the unrolled accesses immediate
    const int rbx = tm & 1;
    float *const rbE = rb + rbx, *const rbO = rb - rbx;   // even / odd indices
    float *const rbL = (lane & 1) ? rbO : rbE;            // indices lane + T*m (T even)
    float *acc = reinterpret_cast<float *>(reinterpret_cast<char *>(tw + TWS) +
                                           (size_t)(blockDim.x / T) * (PADN * sizeof(float2) + (2 * N + RBP) * sizeof(float))) +
                 (size_t)warp * 2 * (ACC + RBP);         // [2][ACC + RBP] first-level sums of the warp's chunk

    for (int i = threadIdx.x; i < TWL; i += blockDim.x) tw[i] = P.tw_row[i];
    if constexpr (HSHIFT)
        for (int i = threadIdx.x; i < TWL; i += blockDim.x) tw[TWL + i] = P.phase[i];
    __syncthreads();

    const int w = blockIdx.y;
    const int c = blockIdx.x * (blockDim.x >> 5) + warp;  // chunk (always < nchunks, see launcher)
    const xcg_loc loc = P.locs[w];
    int local, pidx;
    const PairDev pd = pair_of(P, w, local, pidx);
    const int npy = P.npy;
    const int mx0 = loc.x - N / 2, my0 = loc.y - npy / 2;
    const int sx0 = loc.x + pd.x_offset - N / 2;
    const int sy0 = loc.y + pd.y_offset + slave_row_shift(pd, loc.y) - npy / 2;
    bool oob = false;
    constexpr int ri = 1 << LG;
    // kept fine samples k = ri*q + p - N/2 in [0, N) are q in [N/(2ri), 3N/(2ri)):
    // with q = lane + T*m that is m in [KM0, KM1) for every lane and phase
    constexpr int KM0 = (LG == 0) ? 0 : PER / (2 * ri), KM1 = (LG == 0) ? PER : 3 * PER / (2 * ri);
    float mn1 = INFINITY, mx1 = -INFINITY, mn2 = INFINITY, mx2 = -INFINITY;

    // raw samples of one patch row, team layout; 32-bit words (int16 pair or float)
    auto load_row = [&](int pt, int r, uint32_t *raw) {
        // image fields re-read per row (parameter space or L1) instead of held in registers
        const PairDev *q = P.pairs ? P.pairs + pidx : nullptr;
        const void *img = q ? (pt ? q->slave : q->master) : (pt ? P.single.slave : P.single.master);
        const int nx = q ? (pt ? q->s_nx : q->m_nx) : (pt ? P.single.s_nx : P.single.m_nx);
        const int ny = q ? (pt ? q->s_ny : q->m_ny) : (pt ? P.single.s_ny : P.single.m_ny);
        const int x0 = pt ? sx0 : mx0, y = (pt ? sy0 : my0) + r;
        const bool rowok = (y >= 0 && y < ny);
        const uint32_t *row = reinterpret_cast<const uint32_t *>(img) + (size_t)(rowok ? y : 0) * (size_t)nx;
        if (rowok && x0 >= 0 && x0 + N <= nx) {          // the usual case: the whole row segment is inside
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
    const bool iq16 = (P.format == 0);
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

    // amplitudes of one patch row into rb (natural order of the kept fine samples)
    auto amp_row = [&](int pt, int r, const uint32_t *raw) {
        float *const rowE = rbE + pt * N, *const rowO = rbO + pt * N;
        float2 v[PER];
        to_complex(raw, v);
        if (LG == 0) {
            float *const rowL = rbL + pt * N;
#pragma unroll
            for (int m = 0; m < PER; m++) rowL[lane + T * m] = hypotf(v[m].x, v[m].y);
            return;
        }
        // interpolated rows differ from the reference's cuFFT rows by rounding
        // anyway, so their amplitudes use the cheaper amp_of; hypotf is kept
        // where the samples are the input itself (ri == 1, bit-exact)
#pragma unroll
        for (int m = KM0; m < KM1; m++) {        // phase-0 samples are the input
            const int k = ((lane + T * m) << LG) - N / 2;     // even
            rowE[k] = amp_of(v[m]);
        }
#pragma unroll 1
        for (int p = 1; p < ri; p++) {
            if (p > 1) {                             // ri > 2: reread the row (L2) instead of keeping it live
                uint32_t again[PER];
                load_row(pt, r, again);
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

    uint32_t rawm[PER], raws[PER];
    load_row(0, c * RPC + tm, rawm);
#pragma unroll 1
    for (int ir = 0; ir < RPT; ir++) {
        const int r = c * RPC + ir * TPW + tm;
#pragma unroll 1
        for (int pt = 0; pt < 2; pt++) {
            uint32_t cur[PER];
#pragma unroll
            for (int m = 0; m < PER; m++) cur[m] = pt ? raws[m] : rawm[m];
            if (pt == 0) load_row(1, r, raws);                   // in flight during the master row
            else if (ir + 1 < RPT) load_row(0, r + TPW, rawm);   // in flight during the slave row
            amp_row(pt, r, cur);
        }
        __syncwarp();
        // packed real pair and its row FFT; amplitudes for the time correlation
        const bool rin = (r >= P.ysearch) && (r < npy - P.ysearch);
        float *a1g = P.amp1 + ((size_t)w * npy + r) * N;
        const bool r2c = (r >= P.ysearch) && (r < P.ysearch + P.ny_corr);
        float *a2g = P.amp2c + ((size_t)w * P.ny_corr + (r - P.ysearch)) * P.nx_corr;
        float *acc1 = acc + tm * (N + GOFF), *acc2 = acc + (ACC + RBP) + tm * (N + GOFF);
        float2 v[PER];
        // the slave mask's columns [xsearch, N - xsearch) (xsearch = N/4) and
        // the time-correlation window's [xsearch, xsearch + nx_corr) are both
        // m in [PER/4, 3 PER/4) for every lane.  First reduction level in the
        // reference's order, x[t] + x[t+512]: rows ir = 0 and 1 of this team.
        auto packed = [&](auto first) {
#pragma unroll
            for (int m = 0; m < PER; m++) {
                const int e = lane + T * m;
                const float a1 = rbL[e], a2 = rbL[N + e];
                const bool cin = (m >= PER / 4) && (m < 3 * PER / 4);
                const bool in = rin && cin;
                v[m] = make_float2(a1, in ? a2 : 0.f);
                mn1 = fminf(mn1, a1); mx1 = fmaxf(mx1, a1);
                if (in) { mn2 = fminf(mn2, a2); mx2 = fmaxf(mx2, a2); }
                a1g[e] = a1;
                if (r2c && cin) a2g[e - N / 4] = a2;
                if constexpr (decltype(first)::value) { acc1[e] = a1; acc2[e] = a2; }
                else { acc1[e] = acc1[e] + a1; acc2[e] = acc2[e] + a2; }
            }
        };
        if (ir == 0) packed(std::true_type{});
        else packed(std::false_type{});
        // the precision form transforms the packed rows on the tensor cores
        if (!P.tc_form) team_fft_reg<N, -1>(v, ex, tw, lane);
        float2 *zg = P.zrow + ((size_t)w * npy + r) * N;
#pragma unroll
        for (int m = 0; m < PER; m++) zg[lane + T * m] = v[m];
        __syncwarp();
    }
    oob = __ballot_sync(0xffffffffu, oob) != 0u;      // any lane of the chunk's warp
    // remaining tree levels over the warp's ACC first-level sums, strides
    // ACC/2 .. 1: lane L holds t = L + 32*q, so strides >= 32 are
    // register-local and smaller ones are warp shuffles
#pragma unroll
    for (int pt = 0; pt < 2; pt++) {
        float a[ACC / 32];
#pragma unroll
        for (int q = 0; q < ACC / 32; q++) a[q] = acc[pt * (ACC + RBP) + l32 + 32 * q + (32 * q / N) * GOFF];
#pragma unroll
        for (int s = ACC / 64; s >= 1; s >>= 1)
#pragma unroll
            for (int q = 0; q < s; q++) a[q] = a[q] + a[q + s];
        float x = a[0];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) x = x + __shfl_xor_sync(0xffffffffu, x, o);
        if (l32 == 0) P.part[((size_t)w * 2 + pt) * P.nchunks + c] = x;
    }
    if (l32 == 0) P.oobmap[(size_t)w * P.nchunks + c] = oob ? 1 : 0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        mn1 = fminf(mn1, __shfl_xor_sync(0xffffffffu, mn1, o));
        mx1 = fmaxf(mx1, __shfl_xor_sync(0xffffffffu, mx1, o));
        mn2 = fminf(mn2, __shfl_xor_sync(0xffffffffu, mn2, o));
        mx2 = fmaxf(mx2, __shfl_xor_sync(0xffffffffu, mx2, o));
    }
    if (l32 == 0) {
        float *mm = P.minmax + (size_t)w * 4 * P.nchunks;
        mm[c] = mn1; mm[P.nchunks + c] = mx1; mm[2 * P.nchunks + c] = mn2; mm[3 * P.nchunks + c] = mx2;
    }
}


// ---------------------------------------------------------------- k_cols
// Replaces the column half of the forward FFTs, d_mulaconjb/d_Cmul
// (do_freq_xcorr.cu:32-64,106-109), the inverse FFT's column half and
// d_scaleFft2D (:113-114), plus the patch means of h_reduceFD_strip
// (conv_ampl_demean.cu:713-725) and the demean/mask of d_mean_mask_strip
// (:111-139), applied here in the frequency domain: the master loses
// m1*N*M at bin (0,0), the slave m2 times the DFT of its mask.
// One team per column pair (kx, N-kx); the CTA stages the pairs' columns in
// shared memory with coalesced row reads, each FFT uses its own column slot as
// the exchange buffer (the column is in registers meanwhile), and the half
// spectrum goes back row by row.

// DEPTH 2: partner and own columns staged as two cp.async groups, the partner
// transforms overlapping the own columns' arrival; DEPTH 1: one group.
template <int M, int THR, int DEPTH>
__global__ void __launch_bounds__(THR, ColsGeom<M, THR>::BLOCKS) k_cols(Plan P) {
    using G = ColsGeom<M, THR>;
    constexpr int T = G::T, CS = G::CS, CP = G::CP, TWL = G::TWL;
    constexpr int PER = M / T;
    static_assert((CP & (CP - 1)) == 0 && T % 2 == 0, "column pairs per CTA: a power of two");

    extern __shared__ float4 smem_raw[];
    float2 *tw = reinterpret_cast<float2 *>(smem_raw);
    float2 *cols = tw + TWL;                   // [2*CP][CS]
    float *shf = reinterpret_cast<float *>(cols + 2 * CP * CS);    // m1 N M and m2 as floats

    const int w = blockIdx.y, b = blockIdx.x;
    const int N = P.npx;
    const int kx0 = b * CP;
    const int warp = threadIdx.x >> 5, l32 = threadIdx.x & 31;
    const int lane = l32 % T;
    const int team = warp * (32 / T) + l32 / T;

    for (int i = threadIdx.x; i < TWL; i += blockDim.x) tw[i] = P.tw_col[i];
    {   // thread t stages column slot t % CP of both halves (partner slots CP.., then
        // own slots 0..) for rows t / CP + k * THREADS/CP, as two cp.async groups:
        // the partner columns land first and are transformed while the own
        // columns are still arriving
        constexpr int RSTEP = G::THREADS / CP;
        constexpr int NLD = M / RSTEP;
        const int sl = threadIdx.x % CP, row0 = threadIdx.x / CP;
        const int kxp = kx0 + sl;
        const int pcol = (kxp == 0) ? N / 2 : N - kxp;
        const float2 *base = P.zrow + (size_t)w * M * N;
#pragma unroll 8
        for (int k = 0; k < NLD; k++) {
            const int r = row0 + k * RSTEP;
            cp_async8(cols + (CP + sl) * CS + fft_pad(r), base + (size_t)r * N + pcol);
        }
        if constexpr (DEPTH == 2) cp_async_commit();
#pragma unroll 8
        for (int k = 0; k < NLD; k++) {
            const int r = row0 + k * RSTEP;
            cp_async8(cols + sl * CS + fft_pad(r), base + (size_t)r * N + kxp);
        }
        cp_async_commit();
    }
    if (warp == 0) {
        // patch means (:719-724): the reference adds the FP32 chunk sums in
        // double in index order; these partial sums are exact in double for
        // any realistic patch (chunk sums of one patch span far fewer than 29
        // binary orders), so a tree order gives the same bits
        const float *pb = P.part + (size_t)w * 2 * P.nchunks;
        double s1 = 0.0, s2 = 0.0;
        for (int i = l32; i < P.nchunks; i += 32) { s1 += (double)pb[i]; s2 += (double)pb[P.nchunks + i]; }
        s1 = warp_sum_f64(s1);
        s2 = warp_sum_f64(s2);
        if (l32 == 0) {
            // / (N M), a power of two: an exact scaling instead of an FP64 division
            const double inv = pow2_inv(N * M);
            s1 *= inv;
            s2 *= inv;
            shf[0] = (float)(s1 * (double)N * (double)M);   // the master's DC term, m1 N M
            shf[1] = (float)s2;
            if (b == 0) { P.means[2 * w] = s1; P.means[2 * w + 1] = s2; }
        }
    }
    if constexpr (DEPTH == 2) cp_async_wait<1>();   // partner columns in (this thread's copies)
    else cp_async_wait<0>();                        // all columns in
    __syncthreads();                                // ... and everyone's
    const float dc1 = shf[0];
    const float m2 = shf[1];

    const int kx = kx0 + team;
    float2 *a = cols + team * CS;
    float2 *pa = cols + (CP + team) * CS;
    float2 z[PER];
    // partner column first, back into its slot (read below at -ky)
#pragma unroll
    for (int m = 0; m < PER; m++) z[m] = pa[fft_pad(lane + T * m)];
    __syncwarp();
    team_fft_reg<M, -1>(z, pa, tw, lane);
#pragma unroll
    for (int m = 0; m < PER; m++) pa[fft_pad(lane + T * m)] = z[m];
    if constexpr (DEPTH == 2) {
        cp_async_wait<0>();                      // own columns in
        __syncthreads();
    }
#pragma unroll
    for (int m = 0; m < PER; m++) z[m] = a[fft_pad(lane + T * m)];
    __syncwarp();
    team_fft_reg<M, -1>(z, a, tw, lane);
#pragma unroll
    for (int m = 0; m < PER; m++) a[fft_pad(lane + T * m)] = z[m];
    __syncwarp();
    // the kx = 0 team also emits column N/2; the trip count stays warp-uniform
    // because team_fft_reg synchronises the whole warp
    const int nout = __any_sync(0xffffffffu, kx == 0) ? 2 : 1;
#pragma unroll 1
    for (int o = 0; o < nout; o++) {
        // o = 0: column kx with partner pa (itself for kx = 0); o = 1: column N/2, self-paired
        const float2 *zs = (o == 0) ? a : pa;
        const float2 *zp = (o == 0) ? ((kx == 0) ? a : pa) : pa;
        const int kxx = (o == 0) ? kx : N / 2;
        const float2 bx = __ldg(P.box_x + kxx);
        const bool flip = ((kxx + lane) & 1) != 0;   // (-1)^(kx+ky): ky = lane + T*m, T even
        // mirrored row M - ky: for m >= 1 it never wraps, and with T a multiple
        // of 16 its padded index falls by T + T/16 per m (immediate offsets)
        const float2 *zp1 = zp + fft_pad((M - lane - T) & (M - 1));
#pragma unroll
        for (int m = 0; m < PER; m++) {
            const int ky = lane + T * m;
            const float2 z1 = zs[fft_pad(ky)];
            float2 z2;
            if constexpr (T % 16 == 0) z2 = (m == 0) ? zp[fft_pad((M - lane) & (M - 1))] : zp1[-(m - 1) * (T + T / 16)];
            else z2 = zp[fft_pad((M - ky) & (M - 1))];
            // A1 = (z1 + conj z2)/2, A2 = (z1 - conj z2)/(2i)
            float2 A1 = make_float2(0.5f * (z1.x + z2.x), 0.5f * (z1.y - z2.y));
            float2 A2 = make_float2(0.5f * (z1.y + z2.y), -0.5f * (z1.x - z2.x));
            if (kxx == 0 && ky == 0) A1.x -= dc1;
            const float2 bm = cmulf(bx, __ldg(P.box_y + ky));
            A2.x -= m2 * bm.x;
            A2.y -= m2 * bm.y;
            float2 pr = cmulf_conj(A1, A2);
            if (flip) { pr.x = -pr.x; pr.y = -pr.y; }
            z[m] = pr;
        }
        float2 *dst = (o == 0) ? a : pa;
        __syncwarp();                            // every lane has read a and pa before dst is reused
        team_fft_reg<M, +1>(z, dst, tw, lane);
        // only the surface rows [ysearch, ysearch + nyc) = [M/4, 3M/4) go out
#pragma unroll
        for (int m = PER / 4; m < 3 * PER / 4; m++) dst[fft_pad(lane + T * m)] = z[m];
        __syncwarp();
    }
    __syncthreads();
    // write rows y in [ysearch, ysearch+nyc) of the half spectrum, kx <= N/2:
    // thread -> slot threadIdx % CP, rows threadIdx / CP + k * RS
    {
        constexpr int RS = G::THREADS / CP;        // = T
        float2 *qw = P.qspec + (size_t)w * P.nyc * P.qpitch;
        const int s = threadIdx.x % CP, y0 = threadIdx.x / CP;
        float2 *dstq = qw + (size_t)y0 * P.qpitch + kx0 + s;
        const float2 *srcc = cols + s * CS;
        for (int k = 0; k < (M / 2) / RS; k++) {
            // RS a multiple of 16: the padded row index steps by RS + RS/16
            const int sy = (RS % 16 == 0) ? fft_pad(y0 + M / 4) + k * (RS + RS / 16) : fft_pad(y0 + M / 4 + k * RS);
            dstq[(size_t)k * RS * P.qpitch] = srcc[sy];
        }
        if (b == 0)                                // column N/2, the kx = 0 team's partner slot
            for (int yq = threadIdx.x; yq < M / 2; yq += blockDim.x)
                qw[(size_t)yq * P.qpitch + N / 2] = cols[CP * CS + fft_pad(yq + M / 4)];
    }
}

// ---------------------------------------------------------------- k_peak
// Replaces the row half of the inverse FFT, d_fillcorrmat_strip/d_Cabs
// (do_freq_xcorr.cu:26-29,67-84,141-143), h_reduce_strip (conv_ampl_demean.cu:642-675),
// the per-window host loop of d_do_freq_corr_strip (do_freq_xcorr.cu:150-195),
// the time correlation d_calc_time_corr_strip (do_time_int_xcorr.cu:71-100),
// d_scaled_strip (conv_ampl_demean.cu:50-68) and d_cppow_strip (:75-95).
// row pairs of the largest surface (nyc = 512: windows of 512 rows)
constexpr int PEAK_MAX_ROW_PAIRS = 256;

template <int N, int MINB, int NT = 256>
__global__ void __launch_bounds__(NT, MINB) k_peak(Plan P) {
    constexpr int T = fft_lanes(N);
    constexpr int PADN = fft_padded_len(N);
    constexpr int TWL = fft_twiddle_len(N);
    constexpr int PER = N / T;
    constexpr int NW = NT / 32;

    extern __shared__ float4 smem_raw[];
    float2 *tw = reinterpret_cast<float2 *>(smem_raw);
    const int teams = NT / T;
    float2 *fb = tw + TWL;                                // [teams][PADN]
    unsigned long long *rk = reinterpret_cast<unsigned long long *>(fb + teams * PADN);  // [NW]
    double *rd = reinterpret_cast<double *>(rk + NW);     // [2][NW]
    long long *ri64 = reinterpret_cast<long long *>(rd + 2 * NW);   // [3][NW]
    double *bc = reinterpret_cast<double *>(ri64 + 3 * NW);   // broadcast [4]
    // [nyc / 2 <= 256] surface sum of each row pair, and its part in the reference's half blocks
    float *rowf = reinterpret_cast<float *>(bc + 4);
    float *rowh = rowf + PEAK_MAX_ROW_PAIRS;

    const int w = blockIdx.x;
    const int warp = threadIdx.x >> 5, l32 = threadIdx.x & 31;
    const int lane = l32 % T;
    const int team = warp * (32 / T) + l32 / T;
    float2 *ex = fb + team * PADN;
    const int M = P.npy, nxc = P.nxc, nyc = P.nyc;
    const float scale = 1.0f / ((float)N * (float)M);

    for (int i = threadIdx.x; i < TWL; i += NT) tw[i] = P.tw_row[i];
    // The reference's surface is exactly zero when either demeaned patch is
    // (its FFTs of zeros stay zeros); the packed transform here would leave
    // rounding residue of the other patch, so that case is set explicitly.
    if (warp == 0) {          // per-chunk extremes and out-of-image flags, reduced by one warp
        float a = INFINITY, b = -INFINITY, c2 = INFINITY, d = -INFINITY;
        int oobf = 0;
        if (P.rc) {
            // shared row segments: the window's chunks; the slave's extremes
            // over the chunks of its mask rows (a chunk's rows are all inside
            // or all outside: rows per chunk divide ysearch)
            const int2 wc = P.rc_wch[w];
            for (int i = l32; i < P.nchunks; i += 32) {
                const float2 m1 = P.rc_minmax[wc.x + i];
                a = fminf(a, m1.x); b = fmaxf(b, m1.y);
                const int r0 = i * P.rpc;
                if (r0 >= P.ysearch && r0 < M - P.ysearch) {
                    const float2 m2 = P.rc_minmax[wc.y + i];
                    c2 = fminf(c2, m2.x); d = fmaxf(d, m2.y);
                }
                oobf |= P.rc_oob[wc.x + i] | P.rc_oob[wc.y + i];
            }
        } else {
            const float *mm = P.minmax + (size_t)w * 4 * P.nchunks;
            for (int i = l32; i < P.nchunks; i += 32) {
                a = fminf(a, mm[i]); b = fmaxf(b, mm[P.nchunks + i]);
                c2 = fminf(c2, mm[2 * P.nchunks + i]); d = fmaxf(d, mm[3 * P.nchunks + i]);
                oobf |= P.oobmap[(size_t)w * P.nchunks + i];
            }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            a = fminf(a, __shfl_xor_sync(0xffffffffu, a, o));
            b = fmaxf(b, __shfl_xor_sync(0xffffffffu, b, o));
            c2 = fminf(c2, __shfl_xor_sync(0xffffffffu, c2, o));
            d = fmaxf(d, __shfl_xor_sync(0xffffffffu, d, o));
        }
        oobf = __any_sync(0xffffffffu, oobf != 0);
        if (l32 == 0) {
            const float m1f = (float)P.means[2 * w], m2f = (float)P.means[2 * w + 1];
            const bool z1 = (a == b) && (a - m1f == 0.f);
            const bool z2 = (c2 == d) && (c2 - m2f == 0.f);
            bc[2] = (z1 || z2) ? 0.0 : 1.0;
            bc[3] = oobf ? 1.0 : 0.0;
        }
    }
    __syncthreads();
    const float keep = (float)bc[2];
    unsigned long long best = 0ull;
    const float2 *q = P.qspec + (size_t)w * nyc * P.qpitch;
    float *surf = P.surf + (size_t)w * nyc * nxc;
    for (int pr = team; pr < nyc / 2; pr += teams) {
        const int y1 = 2 * pr, y2 = y1 + 1;
        // two real rows in one complex inverse FFT: S = Q1 + i Q2, Hermitian-extended
        float2 v[PER];
#pragma unroll
        for (int m = 0; m < PER; m++) {
            const int e = lane + T * m;
            const int kx = (e <= N / 2) ? e : N - e;
            float2 q1 = q[(size_t)y1 * P.qpitch + kx], q2 = q[(size_t)y2 * P.qpitch + kx];
            if (kx == 0 || kx == N / 2) { q1.y = 0.f; q2.y = 0.f; }
            v[m] = (e <= N / 2) ? make_float2(q1.x - q2.y, q1.y + q2.x) : make_float2(q1.x + q2.y, q2.x - q1.y);
        }
        team_fft_reg<N, +1>(v, ex, tw, lane);
        // surface sums: each row pair's in FP32 (the lane's values, then a
        // fixed tree over the team), then the row pairs in double in a fixed
        // order, so the sums do not depend on the launch shape (GB300's FP64
        // pipe is a small fraction of its FP32 rate; the FP32 rounding, about
        // 1e-7 relative, is far below what the statistics need)
        float fpart = 0.f, hpart = 0.f;
#pragma unroll
        for (int m = 0; m < PER; m++) {
            const int xq = lane + T * m - P.nx_corr / 2;
            if (xq < 0 || xq >= nxc) continue;
            const float c1 = fabsf(v[m].x * scale) * keep, c2 = fabsf(v[m].y * scale) * keep;
            surf[(size_t)y1 * nxc + xq] = c1;
            surf[(size_t)y2 * nxc + xq] = c2;
            const unsigned e1 = (unsigned)(y1 * nxc + xq), e2 = (unsigned)(y2 * nxc + xq);
            const unsigned long long k1 = argmax_key(c1, e1), k2 = argmax_key(c2, e2);
            best = k1 > best ? k1 : best;
            best = k2 > best ? k2 : best;
            fpart += c1 + c2;
            if (!(e1 & 512u)) hpart += c1;      // reduce6<double,1024> keeps local [0,512) and [1024,1536)
            if (!(e2 & 512u)) hpart += c2;
        }
#pragma unroll
        for (int o = T / 2; o > 0; o >>= 1) {            // within the team
            fpart += __shfl_xor_sync(0xffffffffu, fpart, o);
            hpart += __shfl_xor_sync(0xffffffffu, hpart, o);
        }
        if (lane == 0) { rowf[pr] = fpart; rowh[pr] = hpart; }
    }
    best = warp_max_u64(best);
    if (l32 == 0) rk[warp] = best;
    __syncthreads();
    if (warp == 0) {
        double hs = 0.0, fs = 0.0;
        for (int i = l32; i < nyc / 2; i += 32) { hs += (double)rowh[i]; fs += (double)rowf[i]; }
        hs = warp_sum_f64(hs);
        fs = warp_sum_f64(fs);
        if (l32 == 0) {
            unsigned long long bb = rk[0];
            for (int i = 1; i < NW; i++) bb = rk[i] > bb ? rk[i] : bb;
            rk[0] = bb; rd[0] = hs; rd[NW] = fs;
        }
    }
    __syncthreads();
    const unsigned pk = argmax_index(rk[0]);
    const int ip = (int)(pk / (unsigned)nxc), jp = (int)(pk % (unsigned)nxc);
    const double cmax = (double)argmax_value(rk[0]);
    const float jpeak = (float)jp - (float)nxc / 2.0f;     // do_freq_xcorr.cu:158-159
    const float ipeak = (float)ip - (float)nyc / 2.0f;

    // time-domain correlation at the integer peak on (int) demeaned amplitudes
    const float m1f = (float)P.means[2 * w], m2f = (float)P.means[2 * w + 1];
    // master patch rows (row stride N) and the slave's centre (row stride a2s):
    // per window, or rows of the window's chunks of shared row segments
    const float *a1, *a2;
    int a2s;
    if (P.rc) {
        const int2 wc = P.rc_wch[w];
        a1 = P.rc_amp + ((size_t)wc.x * P.rpc + P.ysearch + (int)ipeak) * N + (int)jpeak + P.xsearch;
        a2 = P.rc_amp + ((size_t)wc.y * P.rpc + P.ysearch) * N + P.xsearch;
        a2s = N;
    } else {
        a1 = P.amp1 + (size_t)w * M * N + (size_t)(P.ysearch + (int)ipeak) * N + (int)jpeak + P.xsearch;
        a2 = P.amp2c + (size_t)w * P.ny_corr * P.nx_corr;
        a2s = P.nx_corr;
    }
    long long sn = 0, s1 = 0, s2 = 0;
    constexpr int NXC = N / 2;          // nx_corr = 2 xsearch = npx / 2
    if constexpr (N <= 256) {
        // The rows are staged by cp.async in the transforms' exchange buffers,
        // free from here on: RRM rows of both operands per round, all of them
        // in flight at once without holding registers (the peak stage of
        // these sizes is latency-bound: 0.107 -> 0.098 ms per 1000 windows of
        // 128 x 128; the 512-point stage, at several waves, is faster with the
        // register loads below).  The sums are integers, so their order does
        // not change them.
        constexpr int FBF = (NT / T) * PADN * 2;        // floats of the exchange buffers
        constexpr int RRM = FBF / (2 * NXC);            // rows of both operands per round
        static_assert(RRM >= 1 && NXC % 4 == 0, "staging rows");
        float *sa = reinterpret_cast<float *>(fb), *sb = sa + RRM * NXC;
        for (int r0 = 0; r0 < P.ny_corr; r0 += RRM) {
            const int n = min(RRM, P.ny_corr - r0) * NXC;
            for (int i = threadIdx.x; i < n; i += NT) {      // master rows at the peak offset: any alignment
                const int r = i / NXC, cc = i - r * NXC;
                cp_async4(sa + i, a1 + (size_t)(r0 + r) * N + cc);
            }
            for (int i = threadIdx.x; i < n / 4; i += NT) {  // the slave's centre: 16-byte aligned rows
                const int e = 4 * i, r = e / NXC, cc = e - r * NXC;
                cp_async16(sb + e, a2 + (size_t)(r0 + r) * a2s + cc);
            }
            cp_async_commit();
            cp_async_wait<0>();
            __syncthreads();
            for (int i = threadIdx.x; i < n; i += NT) {
                const long long ia = (long long)(int)(sa[i] - m1f), ib = (long long)(int)(sb[i] - m2f);
                sn += ia * ib; s1 += ia * ia; s2 += ib * ib;
            }
            __syncthreads();             // read before the next round's copies land
        }
    } else {
        constexpr int GU = 8;            // loads in flight per thread and operand
        const int ntot = P.ny_corr * NXC;   // a multiple of NT * GU
        for (int i0 = threadIdx.x; i0 < ntot; i0 += NT * GU) {
            float va[GU], vb[GU];
#pragma unroll
            for (int u = 0; u < GU; u++) {
                const int i = i0 + u * NT;
                const int r = i / NXC, cc = i - r * NXC;
                va[u] = __ldg(a1 + (size_t)r * N + cc);
                vb[u] = __ldg(a2 + (size_t)r * a2s + cc);
            }
#pragma unroll
            for (int u = 0; u < GU; u++) {
                const long long ia = (long long)(int)(va[u] - m1f), ib = (long long)(int)(vb[u] - m2f);
                sn += ia * ib; s1 += ia * ia; s2 += ib * ib;
            }
        }
    }
    sn = warp_sum_i64(sn); s1 = warp_sum_i64(s1); s2 = warp_sum_i64(s2);
    if (l32 == 0) { ri64[warp] = sn; ri64[NW + warp] = s1; ri64[2 * NW + warp] = s2; }
    __syncthreads();
    if (threadIdx.x == 0) {
        long long tn = 0, t1 = 0, t2 = 0;
        for (int i = 0; i < NW; i++) { tn += ri64[i]; t1 += ri64[NW + i]; t2 += ri64[2 * NW + i]; }
        const double gd = sqrt(1.0 * (double)t1 * (double)t2);
        const double gamma = (gd == 0.0) ? 0.0 : 100.0 * fabs((double)tn / gd);
        const double msc = cmax / gamma;
        bc[0] = gamma;
        bc[1] = msc;
        const double c0n = (double)surf[0] / msc;
        P.corr0n[w] = c0n;
        int local, pidx;
        const PairDev pd = pair_of(P, w, local, pidx);
        xcg_result &o = pd.out[local];
        o.xoff = -1 * jpeak;
        o.yoff = -1 * ipeak;
        o.corr = (float)gamma;
        o.ip = ip; o.jp = jp;
        o.flags = (bc[3] != 0.0) ? XCG_FLAG_OOB : 0;
        // precision form: the tensor-core stages before this kernel raise the
        // flag when a bounded wait ran out and left part of a spectrum unwritten
        if (P.tc_form && P.tc_err && *reinterpret_cast<volatile const int *>(P.tc_err)) o.flags |= XCG_FLAG_STAGE_TIMEOUT;
        o.cmax = cmax;
        const double inv_ns = pow2_inv(nxc * nyc);      // exact: nxc * nyc is a power of two
        o.cave = rd[0] * inv_ns;
        o.cave_true = rd[NW] * inv_ns;
        o.gamma = gamma;
        o.mean1 = P.means[2 * w];
        o.mean2 = P.means[2 * w + 1];
        o.corr0n = c0n;
        o.fip = -1; o.fjp = -1; o.fmax = 0.f; o.xfrac = 0.f; o.yfrac = 0.f;
    }
    __syncthreads();
    // normalised 9x9 neighbourhood of the integer peak, for the subpixel refiner
    {
        int local, pidx;
        const PairDev pd = pair_of(P, w, local, pidx);
        if (pd.feat) {
            for (int t = threadIdx.x; t < 81; t += NT) {
                const int yy = ip - 4 + t / 9, xx = jp - 4 + t % 9;
                float v = 0.f;
                // cmax is a float value: the FP32 quotient is the correctly rounded
                // one, without the FP64 division (slow on GB300)
                if (cmax > 0.0 && yy >= 0 && yy < nyc && xx >= 0 && xx < nxc) v = surf[yy * nxc + xx] / (float)cmax;
                pd.feat[(size_t)local * 81 + t] = v;
            }
        }
    }
    // 8x8 neighbourhood with the reference's flat bounds test (conv_ampl_demean.cu:82-93)
    if (P.interp_flag) {
        const int n2 = P.n2x * P.n2y;
        const double msc = bc[1];
        const int jc = (nxc / 2) - P.n2x / 2 - (int)(-1 * jpeak);
        const int ic = (nyc / 2) - P.n2y / 2 - (int)(-1 * ipeak);
        const long long ns = (long long)nxc * nyc;
        for (int t = threadIdx.x; t < n2; t += NT) {
            const int iy = t / P.n2x, ix = t - iy * P.n2x;
            const long long k = (long long)(ic + iy) * nxc + (jc + ix);
            float v = 0.f;
            unsigned char nx = 0;
            if (k >= 0 && k < ns) v = powf((float)((double)surf[k] / msc), 0.25f);
            else if (k == ns) nx = 1;
            P.md[(size_t)w * n2 + t] = v;
            P.mdnext[(size_t)w * n2 + t] = nx;
        }
    }
}

// ---------------------------------------------------------------- k_subpix
// Replaces d_do_highres_corr (highres_corr.cu:23-79): the 2-D zero-pad
// interpolation d_fft_interpolate_2d_strip (fft_interpolate_routines.cu:118-147)
// as out = KY * md * KX^T with KX (nx2 x n2x) and KY (ny2 x n2y) the exact
// FFT-pad-IFFT-scale operators, then the argmax of the real part
// (h_reduceCr_strip, conv_ampl_demean.cu:730-756) and the fractions
// (highres_corr.cu:59-76).
__global__ void __launch_bounds__(256) k_subpix(Plan P) {
    extern __shared__ float4 smem_raw[];
    const int n2x = P.n2x, n2y = P.n2y, nx2 = P.nx2, ny2 = P.ny2;
    float *md = reinterpret_cast<float *>(smem_raw);                 // [n2y*n2x]
    float2 *tr = reinterpret_cast<float2 *>(md + 64);                // [n2y][nx2]
    float2 *kys = tr + n2y * nx2;                                    // [ny2][n2y]
    float2 *kxs = kys + ny2 * n2y;                                   // [n2x][nx2], transposed
    unsigned long long *rk = reinterpret_cast<unsigned long long *>(kxs + nx2 * n2x);
    int *fl = reinterpret_cast<int *>(rk + 8);

    const int w = blockIdx.x;
    if (P.skip && P.skip[w]) return;                  // the refiner answered for this window
    const int n2 = n2x * n2y;
    if (threadIdx.x == 0) *fl = 0;
    __syncthreads();
    for (int t = threadIdx.x; t < n2; t += blockDim.x) {
        float v = P.md[(size_t)w * n2 + t];
        if (P.mdnext[(size_t)w * n2 + t]) {
            // the reference reads the next window of its strip (conv_ampl_demean.cu:84-89)
            int local, pidx, nlocal = -1, npidx = -1;
            const PairDev pd = pair_of(P, w, local, pidx);
            if (w + 1 < P.nwin) {
                (void)pair_of(P, w + 1, nlocal, npidx);
                if (npidx != pidx) nlocal = -1;
            }
            const int g = local + 1;
            const bool same = pd.strip_len > 0 && g < pd.nlocs && (g % pd.strip_len) != 0 && nlocal == g;
            v = same ? powf((float)P.corr0n[w + 1], 0.25f) : 0.f;
            atomicOr(fl, XCG_FLAG_NEXTREAD);
        }
        md[t] = v;
    }
    for (int t = threadIdx.x; t < ny2 * n2y; t += blockDim.x) kys[t] = __ldg(P.ky + t);
    for (int t = threadIdx.x; t < nx2 * n2x; t += blockDim.x) {
        const int X = t / n2x, c = t - X * n2x;
        kxs[c * nx2 + X] = __ldg(P.kx + t);
    }
    __syncthreads();
    // row pass: tr[r][X] = sum_c md[r][c] * KX[X][c]
    for (int t = threadIdx.x; t < n2y * nx2; t += blockDim.x) {
        const int r = t / nx2, X = t - r * nx2;
        float2 s = make_float2(0.f, 0.f);
#pragma unroll
        for (int c = 0; c < 8; c++) {
            const float2 k = kxs[c * nx2 + X];
            const float m = md[r * 8 + c];
            s.x = fmaf(m, k.x, s.x);
            s.y = fmaf(m, k.y, s.y);
        }
        tr[t] = s;
    }
    __syncthreads();
    // column pass, real part only, and the argmax: a thread keeps two columns
    // (X and X + nx2/2) of the row-pass result in registers (2 x n2y values)
    // and walks the output rows Y, four at a time; a warp shares Y, so each
    // KY read is one broadcast that feeds both columns
    unsigned long long best = 0ull;
    float bestv = -INFINITY;
    const int half = nx2 / 2;
    const int tpr = half < (int)blockDim.x ? half : (int)blockDim.x;   // threads per output row
    const int rp = (int)blockDim.x / tpr;                               // rows in flight per pass
    const float4 *ky4 = reinterpret_cast<const float4 *>(kys);          // two KY entries per load
    for (int X = threadIdx.x % tpr; X < half; X += tpr) {
        float2 tc[2][8];
#pragma unroll
        for (int r = 0; r < 8; r++) { tc[0][r] = tr[r * nx2 + X]; tc[1][r] = tr[r * nx2 + X + half]; }
        for (int Y = threadIdx.x / tpr; Y < ny2; Y += 4 * rp) {
            float re[2][4] = {{0.f, 0.f, 0.f, 0.f}, {0.f, 0.f, 0.f, 0.f}};
#pragma unroll
            for (int j = 0; j < 4; j++) {
                const int yy = Y + j * rp;
                if (yy >= ny2) break;
#pragma unroll
                for (int r2 = 0; r2 < 4; r2++) {
                    const float4 k = ky4[yy * 4 + r2];
#pragma unroll
                    for (int h = 0; h < 2; h++) {
                        re[h][j] = fmaf(k.x, tc[h][2 * r2].x, re[h][j]);
                        re[h][j] = fmaf(-k.y, tc[h][2 * r2].y, re[h][j]);
                        re[h][j] = fmaf(k.z, tc[h][2 * r2 + 1].x, re[h][j]);
                        re[h][j] = fmaf(-k.w, tc[h][2 * r2 + 1].y, re[h][j]);
                    }
                }
            }
#pragma unroll
            for (int j = 0; j < 4; j++) {
                const int yy = Y + j * rp;
                if (yy >= ny2) break;
#pragma unroll
                for (int h = 0; h < 2; h++) {
                    argmax_update(best, bestv, re[h][j], (unsigned)(yy * nx2 + X + h * half));
                }
            }
        }
    }
    best = warp_max_u64(best);
    const int warp = threadIdx.x >> 5;
    if ((threadIdx.x & 31) == 0) rk[warp] = best;
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned long long bb = rk[0];
        for (int i = 1; i < (int)(blockDim.x >> 5); i++) bb = rk[i] > bb ? rk[i] : bb;
        const unsigned pk = argmax_index(bb);
        const int fip = (int)(pk / (unsigned)nx2), fjp = (int)(pk % (unsigned)nx2);
        int local, pidx;
        const PairDev pd = pair_of(P, w, local, pidx);
        xcg_result &o = pd.out[local];
        o.fip = fip;
        o.fjp = fjp;
        o.fmax = argmax_value(bb);
        const float jpeak = (float)fjp - (float)ny2 / 2.0f;    // ny2 for both axes (highres_corr.cu:61-62)
        const float ipeak = (float)fip - (float)ny2 / 2.0f;
        o.xfrac = jpeak / (float)P.ifc;
        o.yfrac = ipeak / (float)P.ifc;
        o.flags |= *fl;
    }
}

// ---------------------------------------------------------------- launchers

int put_row_phase(float2 *dst, int n, int ri) {
    if (ri == 1) { dst[0] = make_float2(0.f, 0.f); return 1; }
    if (ri == 2 && n <= 512) {
        // [(r-1)*16 + k] = exp(-2 pi i r (k + 1/2) / (16 r1)): the second
        // pass's twiddle with the lane factor of the half-sample shift folded
        // in; for n = 512 the third pass's [240 + k] = exp(-2 pi i (k + 1/2) / 512)
        const int r1 = n <= 256 ? n / 16 : 16;       // radix of the second pass
        int o = 0;
        for (int r = 1; r < r1; r++)
            for (int k = 0; k < 16; k++) {
                const double a = -2.0 * M_PI * r * (k + 0.5) / (16.0 * r1);
                dst[o++] = make_float2((float)cos(a), (float)sin(a));
            }
        if (n == 512)
            for (int k = 0; k < 256; k++) {
                const double a = -2.0 * M_PI * (k + 0.5) / 512.0;
                dst[o++] = make_float2((float)cos(a), (float)sin(a));
            }
        for (; o < n; o++) dst[o] = make_float2(0.f, 0.f);
        return n;
    }
    int o = 0;
    for (int q = 1; q < ri; q++)
        for (int f = 0; f < n; f++) {
            const int fp = (f < n / 2) ? f : f - n;
            const double a = 2.0 * M_PI * fp * q / ((double)ri * n);
            dst[o++] = make_float2((float)(cos(a) / n), (float)(sin(a) / n));
        }
    return o;
}

template <int N>
static size_t rows_smem() {
    constexpr int T = fft_lanes(N);
    constexpr int ACC = (N >= 1024) ? 1024 : 512;
    const int teams = 128 / T;
    return fft_twiddle_len(N) * (N <= 512 ? 2 : 1) * sizeof(float2) +
           (size_t)teams * (fft_padded_len(N) * sizeof(float2) + (2 * N + 32) * sizeof(float)) +
           (size_t)(128 / 32) * 2 * (ACC + 32) * sizeof(float);
}
template <int M, int THR = 128>
static size_t cols_smem(int) {
    using G = ColsGeom<M, THR>;
    return G::TWL * sizeof(float2) + (size_t)2 * G::CP * G::CS * sizeof(float2) + 2 * sizeof(double);
}
// resident k_peak CTAs per SM for configuration cfg
template <int N>
constexpr int peak_minb(int cfg) { return (N <= 256) ? (cfg == 1 ? 3 : 4) : (N <= 512 ? (cfg == 1 ? 2 : 3) : 1); }
template <int N, int NT = 256>
static size_t peak_smem() {
    constexpr int T = fft_lanes(N);
    constexpr int teams = NT / T, nw = NT / 32;
    return fft_twiddle_len(N) * sizeof(float2) + (size_t)teams * fft_padded_len(N) * sizeof(float2) +
           (size_t)nw * (sizeof(unsigned long long) + 2 * sizeof(double) + 3 * sizeof(long long)) + 4 * sizeof(double) +
           (size_t)2 * PEAK_MAX_ROW_PAIRS * sizeof(float);
}
// launch shape 2: 512 threads per window (twice the teams per window, the
// same warps per SM) for transforms up to 512 points
template <int N>
constexpr bool peak_wide_ok() { return N <= 512; }
template <int N>
constexpr int peak_wide_minb() { return N <= 256 ? 2 : 1; }
static size_t subpix_smem(const Plan &P) {
    return 64 * sizeof(float) + (size_t)P.n2y * P.nx2 * sizeof(float2) + (size_t)P.ny2 * P.n2y * sizeof(float2) +
           (size_t)P.nx2 * P.n2x * sizeof(float2) + 8 * sizeof(unsigned long long) + 16;
}

template <int N>
static cudaError_t setup_rows() {
    cudaError_t e = cudaSuccess;
    auto set = [&](auto kern) {
        if (e == cudaSuccess) e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)rows_smem<N>());
    };
    set(k_rows<N, 0>); set(k_rows<N, 1>); set(k_rows<N, 2>); set(k_rows<N, 3>);
    return e;
}
template <int M>
static cudaError_t setup_cols(int) {
    // the attribute is per kernel, shared by every context
    cudaError_t e = cudaFuncSetAttribute(k_cols<M, 128, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)cols_smem<M, 128>(M));
    if (!e) e = cudaFuncSetAttribute(k_cols<M, 256, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)cols_smem<M, 256>(M));
    if (!e) e = cudaFuncSetAttribute(k_cols<M, 128, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)cols_smem<M, 128>(M));
    return e;
}
template <int N>
static cudaError_t setup_peak() {
    cudaError_t e = cudaFuncSetAttribute(k_peak<N, peak_minb<N>(0)>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)peak_smem<N>());
    if (!e && peak_minb<N>(1) != peak_minb<N>(0))
        e = cudaFuncSetAttribute(k_peak<N, peak_minb<N>(1)>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)peak_smem<N>());
    if constexpr (peak_wide_ok<N>())
        if (!e)
            e = cudaFuncSetAttribute(k_peak<N, peak_wide_minb<N>(), 512>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)peak_smem<N, 512>());
    return e;
}

cudaError_t kernels_setup(const Plan &P) {
    cudaError_t e = cudaSuccess;
    switch (P.npx) {
        case 64: e = setup_rows<64>(); if (!e) e = setup_peak<64>(); break;
        case 128: e = setup_rows<128>(); if (!e) e = setup_peak<128>(); break;
        case 256: e = setup_rows<256>(); if (!e) e = setup_peak<256>(); break;
        case 512: e = setup_rows<512>(); if (!e) e = setup_peak<512>(); break;
        case 1024: e = setup_rows<1024>(); if (!e) e = setup_peak<1024>(); break;
        default: return cudaErrorInvalidValue;
    }
    if (e) return e;
    switch (P.npy) {
        case 64: e = setup_cols<64>(P.nchunks); break;
        case 128: e = setup_cols<128>(P.nchunks); break;
        case 256: e = setup_cols<256>(P.nchunks); break;
        case 512: e = setup_cols<512>(P.nchunks); break;
        case 1024: e = setup_cols<1024>(P.nchunks); break;
        default: return cudaErrorInvalidValue;
    }
    if (e) return e;
    Plan big = P;                      // the largest interpolated grid any context uses (factor 64)
    big.nx2 = big.n2x * 64;
    big.ny2 = big.n2y * 64;
    return cudaFuncSetAttribute(k_subpix, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)subpix_smem(big));
}

template <int N>
static void launch_rows_t(const Plan &P, cudaStream_t s) {
    dim3 grid(P.nchunks / 4, P.nwin);          // one chunk per warp, 4 warps per CTA
    switch (P.log2ri) {                        // range interpolation factor 1, 2, 4, 8
        case 0: k_rows<N, 0><<<grid, 128, rows_smem<N>(), s>>>(P); break;
        case 1: k_rows<N, 1><<<grid, 128, rows_smem<N>(), s>>>(P); break;
        case 2: k_rows<N, 2><<<grid, 128, rows_smem<N>(), s>>>(P); break;
        default: k_rows<N, 3><<<grid, 128, rows_smem<N>(), s>>>(P); break;
    }
}
template <int M>
static void launch_cols_t(const Plan &P, cudaStream_t s) {
    // 256-thread CTAs take twice the column pairs: only where that divides npx/2
    const bool wide = P.cols_cfg == 1 && ((P.npx / 2) % ColsGeom<M, 256>::CP) == 0;
    if (wide) {
        dim3 grid((P.npx / 2) / ColsGeom<M, 256>::CP, P.nwin);
        k_cols<M, 256, 2><<<grid, 256, cols_smem<M, 256>(P.nchunks), s>>>(P);
        return;
    }
    dim3 grid((P.npx / 2) / ColsGeom<M>::CP, P.nwin);
    if (P.cols_cfg == 2) k_cols<M, 128, 1><<<grid, 128, cols_smem<M>(P.nchunks), s>>>(P);
    else k_cols<M, 128, 2><<<grid, 128, cols_smem<M>(P.nchunks), s>>>(P);
}
template <int N>
static void launch_peak_t(const Plan &P, cudaStream_t s) {
    if constexpr (peak_wide_ok<N>()) {
        if (P.peak_cfg == 2) {
            k_peak<N, peak_wide_minb<N>(), 512><<<P.nwin, 512, peak_smem<N, 512>(), s>>>(P);
            return;
        }
    }
    if (P.peak_cfg == 1) k_peak<N, peak_minb<N>(1)><<<P.nwin, 256, peak_smem<N>(), s>>>(P);
    else k_peak<N, peak_minb<N>(0)><<<P.nwin, 256, peak_smem<N>(), s>>>(P);
}

void launch_rows(const Plan &P, cudaStream_t s) {
    switch (P.npx) {
        case 64: launch_rows_t<64>(P, s); break;
        case 128: launch_rows_t<128>(P, s); break;
        case 256: launch_rows_t<256>(P, s); break;
        case 512: launch_rows_t<512>(P, s); break;
        case 1024: launch_rows_t<1024>(P, s); break;
    }
}
void launch_cols(const Plan &P, cudaStream_t s) {
    switch (P.npy) {
        case 64: launch_cols_t<64>(P, s); break;
        case 128: launch_cols_t<128>(P, s); break;
        case 256: launch_cols_t<256>(P, s); break;
        case 512: launch_cols_t<512>(P, s); break;
        case 1024: launch_cols_t<1024>(P, s); break;
    }
}
void launch_peak(const Plan &P, cudaStream_t s) {
    switch (P.npx) {
        case 64: launch_peak_t<64>(P, s); break;
        case 128: launch_peak_t<128>(P, s); break;
        case 256: launch_peak_t<256>(P, s); break;
        case 512: launch_peak_t<512>(P, s); break;
        case 1024: launch_peak_t<1024>(P, s); break;
    }
}
void launch_subpix(const Plan &P, cudaStream_t s) {
    k_subpix<<<P.nwin, 256, subpix_smem(P), s>>>(P);
}

}  // namespace xcg
