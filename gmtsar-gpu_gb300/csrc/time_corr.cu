// The -time and -time4 modes: a full-search time-domain correlation surface
// in place of the FFT surface (do_time_corr, do_time_int_xcorr.cu:146-189).
// The reference's GPU build leaves these modes without data (its host ints
// are never filled, xcorr.cu:364-368 with :413-414); this restores what the
// CPU code computes: for every lag (ioff, joff) in [-ysearch, ysearch) x
// [-xsearch, xsearch), calc_time_corr (:30-68) or calc_time_corr_hat
// (:103-144) over the ny_corr x nx_corr window of (int) demeaned amplitudes,
// the peak rule of do_time_corr (|corr| above the float-rounded running
// maximum, scan order ioff then joff), and the same 8x8 neighbourhood and
// subpixel stage as the frequency path.
//
//   k_tcorr  per (lag tile, window): the master/slave ints are staged in
//            shared memory by bands of window rows; each thread keeps 2 x 4
//            lags in registers and slides along the window row, so one
//            shared load feeds 8 multiply-adds of the cross sum; the master
//            energy of every lag comes from sliding window sums.  Sums are
//            64-bit (time: exact; time4: modulo 2^64 like the reference's
//            long long).
//   k_tpeak  per window: the scan-order peak, outputs, 8x8 neighbourhood.
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include "time_corr.cuh"

namespace xcg {
namespace {

constexpr int TC_THREADS = 256;
constexpr int TI = 32;      // lag rows per tile (ioff)
constexpr int TJ = 64;      // lag columns per tile (joff)
constexpr int RI = 2, RJ = 4;

template <int MODE>
struct TcTraits;
template <>
struct TcTraits<0> {        // -time: a, b and sums of a*b, a*a
    using E = int32_t;
    using S = long long;
    static constexpr int YB = 32;
    __device__ static E elem(int v) { return v; }
    __device__ static S prod(E a, E b) { return (S)a * (S)b; }
};
template <>
struct TcTraits<1> {        // -time4: u = a^2, v = b^2 and sums of u*v, u*u, wrapping
    using E = unsigned long long;
    using S = unsigned long long;
    static constexpr int YB = 8;
    __device__ static E elem(int v) { return (E)((long long)v * (long long)v); }
    __device__ static S prod(E a, E b) { return a * b; }
};

template <int MODE>
__host__ __device__ constexpr int tc_aw(int nx_corr) { return nx_corr + TJ - 1; }

__host__ __device__ constexpr size_t align16(size_t b) { return (b + 15) & ~(size_t)15; }

// shared layout: A band [YB+TI-1][AW] | B band [YB][nx_corr] | 2 means | 16 reduction slots
template <int MODE>
__host__ __device__ size_t tc_off_b(int nx_corr) {
    using Tr = TcTraits<MODE>;
    return align16((size_t)(Tr::YB + TI - 1) * tc_aw<MODE>(nx_corr) * sizeof(typename Tr::E));
}
template <int MODE>
__host__ __device__ size_t tc_off_m(int nx_corr) {
    using Tr = TcTraits<MODE>;
    return tc_off_b<MODE>(nx_corr) + align16((size_t)Tr::YB * nx_corr * sizeof(typename Tr::E));
}
template <int MODE>
size_t tcorr_smem(int nx_corr) {
    return tc_off_m<MODE>(nx_corr) + 2 * sizeof(double) + 16 * sizeof(unsigned long long);
}

__device__ __forceinline__ double warp_sum_d(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// (int) of a demeaned amplitude, the expression of d_mean_mask_strip
// (conv_ampl_demean.cu:129-136) as the frequency path's gamma uses it
__device__ __forceinline__ int demeaned_int(float amp, float mean) {
    float v = amp - mean;
    v = v * 1.0f;
    return (int)v;
}

template <int MODE>
__global__ void __launch_bounds__(TC_THREADS) k_tcorr(Plan P) {
    using Tr = TcTraits<MODE>;
    using E = typename Tr::E;
    using S = typename Tr::S;
    constexpr int YB = Tr::YB;
    extern __shared__ float4 smem_raw[];
    const int nx_corr = P.nx_corr, ny_corr = P.ny_corr;
    const int AW = tc_aw<MODE>(nx_corr);
    char *sb = reinterpret_cast<char *>(smem_raw);
    E *As = reinterpret_cast<E *>(sb);                                          // [YB+TI-1][AW]
    E *Bs = reinterpret_cast<E *>(sb + tc_off_b<MODE>(nx_corr));                // [YB][nx_corr]
    double *mean_sh = reinterpret_cast<double *>(sb + tc_off_m<MODE>(nx_corr));
    unsigned long long *red = reinterpret_cast<unsigned long long *>(mean_sh + 2);

    const int w = blockIdx.y;
    const int tiles_j = P.nxc / TJ;
    const int i0 = (blockIdx.x / tiles_j) * TI - P.ysearch;         // first ioff of the tile
    const int j0 = (blockIdx.x % tiles_j) * TJ - P.xsearch;         // first joff
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    const int N = P.npx;
    const int l32 = threadIdx.x & 31, warp = threadIdx.x >> 5;

    if (warp == 0) {   // patch means, as the frequency path forms them
        const float *pb = P.part + (size_t)w * 2 * P.nchunks;
        double s1 = 0.0, s2 = 0.0;
        for (int i = l32; i < P.nchunks; i += 32) { s1 += (double)pb[i]; s2 += (double)pb[P.nchunks + i]; }
        s1 = warp_sum_d(s1);
        s2 = warp_sum_d(s2);
        if (l32 == 0) {
            const double inv = __longlong_as_double((long long)(1023 - (31 - __clz(N * P.npy))) << 52);   // 1/(N npy), a power of two
            s1 *= inv;
            s2 *= inv;
            mean_sh[0] = s1; mean_sh[1] = s2;
            if (blockIdx.x == 0) { P.means[2 * w] = s1; P.means[2 * w + 1] = s2; }
        }
    }
    __syncthreads();
    const float m1f = (float)mean_sh[0], m2f = (float)mean_sh[1];
    const float *amp1 = P.amp1 + (size_t)w * P.npy * N;
    const float *amp2 = P.amp2c + (size_t)w * ny_corr * nx_corr;

    S sab[RI][RJ], saa[RI][RJ];
#pragma unroll
    for (int a = 0; a < RI; a++)
#pragma unroll
        for (int b = 0; b < RJ; b++) sab[a][b] = 0;
    S sbb = 0;

#pragma unroll 1
    for (int y0 = 0; y0 < ny_corr; y0 += YB) {
        // master rows ysearch + y0 + i0 + [0, YB+TI-1), columns xsearch + j0 + [0, AW)
        const int ar0 = P.ysearch + y0 + i0, ac0 = P.xsearch + j0;
        for (int t = threadIdx.x; t < (YB + TI - 1) * AW; t += TC_THREADS) {
            const int r = t / AW, cc = t - r * AW;
            As[t] = Tr::elem(demeaned_int(amp1[(size_t)(ar0 + r) * N + ac0 + cc], m1f));
        }
        for (int t = threadIdx.x; t < YB * nx_corr; t += TC_THREADS) {
            const E v = Tr::elem(demeaned_int(amp2[(size_t)y0 * nx_corr + t], m2f));
            Bs[t] = v;
            sbb += Tr::prod(v, v);
        }
        __syncthreads();
#pragma unroll 1
        for (int yy = 0; yy < YB; yy++) {
            const E *brow = Bs + (size_t)yy * nx_corr;
            const E *arow0 = As + (size_t)(yy + RI * ty) * AW + RJ * tx;
            const E *arow1 = arow0 + AW;
            E wa[RI][RJ];
#pragma unroll
            for (int b = 0; b < RJ - 1; b++) { wa[0][b + 1] = arow0[b]; wa[1][b + 1] = arow1[b]; }
#pragma unroll 4
            for (int x = 0; x < nx_corr; x++) {
#pragma unroll
                for (int b = 0; b < RJ - 1; b++) { wa[0][b] = wa[0][b + 1]; wa[1][b] = wa[1][b + 1]; }
                wa[0][RJ - 1] = arow0[x + RJ - 1];
                wa[1][RJ - 1] = arow1[x + RJ - 1];
                const E bv = brow[x];
#pragma unroll
                for (int a = 0; a < RI; a++)
#pragma unroll
                    for (int b = 0; b < RJ; b++) sab[a][b] += Tr::prod(wa[a][b], bv);
            }
        }
        __syncthreads();
    }
    // Sums of a*a (time4: u*u) over each lag's master window, from sliding
    // sums instead of a second multiply-add per lag and element (exact in
    // 64 bits, or modulo 2^64 like the main sums): D[i][x] = the column sum
    // over the window rows of lag row i, for the tile's AW columns, in the
    // shared memory the bands used (it fits: TI * AW * 8 bytes).
    {
        S *D = reinterpret_cast<S *>(sb);
        const int ar0 = P.ysearch + i0, ac0 = P.xsearch + j0;
        auto sq = [&](int r, int cc) -> S {
            const E e = Tr::elem(demeaned_int(amp1[(size_t)r * N + ac0 + cc], m1f));
            return Tr::prod(e, e);
        };
        for (int x = threadIdx.x; x < AW; x += TC_THREADS) {
            S d = 0;
            for (int y = 0; y < ny_corr; y++) d += sq(ar0 + y, x);
            D[x] = d;
            for (int i = 1; i < TI; i++) {
                d += sq(ar0 + i - 1 + ny_corr, x) - sq(ar0 + i - 1, x);
                D[(size_t)i * AW + x] = d;
            }
        }
        __syncthreads();
#pragma unroll
        for (int a = 0; a < RI; a++) {
            const S *drow = D + (size_t)(RI * ty + a) * AW + RJ * tx;
            S e = 0;
            for (int x = 0; x < nx_corr; x++) e += drow[x];
            saa[a][0] = e;
#pragma unroll
            for (int b = 1; b < RJ; b++) {
                e += drow[nx_corr + b - 1] - drow[b - 1];
                saa[a][b] = e;
            }
        }
        __syncthreads();
    }
    // sum of b*b (or b^4) over the window: every thread holds a share
    {
        unsigned long long v = (unsigned long long)sbb;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if (l32 == 0) red[warp] = v;
        __syncthreads();
        if (threadIdx.x == 0) {
            unsigned long long t = 0;
            for (int i = 0; i < TC_THREADS / 32; i++) t += red[i];
            red[8] = t;
        }
        __syncthreads();
    }
    const long long d2 = (long long)red[8];
    double *surf = reinterpret_cast<double *>(P.qspec) + (size_t)w * P.nyc * P.qpitch;
#pragma unroll
    for (int a = 0; a < RI; a++)
#pragma unroll
        for (int b = 0; b < RJ; b++) {
            const int ioff = i0 + RI * ty + a, joff = j0 + RJ * tx + b;
            const long long num = (long long)sab[a][b], d1 = (long long)saa[a][b];
            const double dd = 1.0 * (double)d1 * (double)d2;
            const double den = sqrt(dd);
            double g;
            if (MODE == 0) {
                g = (den == 0.0) ? 0.0 : 100.0 * fabs((double)num / den);
            } else {
                g = (den == 0.0) ? 0.0 : fabs((double)num / den);
                g = (g <= 0.5) ? 0.0 : 100.0 * sqrt((g * 2.0) - 1.0);
            }
            surf[(size_t)(ioff + P.ysearch) * P.qpitch + (joff + P.xsearch)] = g;
        }
}

// Scan-order peak of do_time_corr: with v* the largest |corr| and F = (float)v*,
// the running-maximum scan ends on the last element above F when F < v*, else
// on the first element that rounds to F.
__global__ void __launch_bounds__(TC_THREADS) k_tpeak(Plan P) {
    __shared__ double rd[8];
    __shared__ int ri_[8];
    __shared__ int oob_sh;
    __shared__ double bc[2];
    const int w = blockIdx.x;
    const int nxc = P.nxc, nyc = P.nyc, ns = nxc * nyc;
    const double *surf = reinterpret_cast<const double *>(P.qspec) + (size_t)w * nyc * P.qpitch;
    const int l32 = threadIdx.x & 31, warp = threadIdx.x >> 5;
    auto at = [&](int k) { return fabs(surf[(size_t)(k / nxc) * P.qpitch + (k % nxc)]); };

    double vmax = 0.0;
    for (int k = threadIdx.x; k < ns; k += TC_THREADS) vmax = fmax(vmax, at(k));
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) vmax = fmax(vmax, __shfl_xor_sync(0xffffffffu, vmax, o));
    if (l32 == 0) rd[warp] = vmax;
    __syncthreads();
    if (threadIdx.x == 0) {
        double v = rd[0];
        for (int i = 1; i < TC_THREADS / 32; i++) v = fmax(v, rd[i]);
        bc[0] = v;
    }
    __syncthreads();
    const double vstar = bc[0];
    const float F = (float)vstar;
    const bool down = (double)F < vstar;
    if (warp == 0) {          // any chunk that read outside an image, reduced by one warp
        int f = 0;
        for (int i = l32; i < P.nchunks; i += 32) f |= P.oobmap[(size_t)w * P.nchunks + i];
        f = __any_sync(0xffffffffu, f != 0);
        if (l32 == 0) oob_sh = f;
    }
    int pick = down ? -1 : ns;
    for (int k = threadIdx.x; k < ns; k += TC_THREADS) {
        const double v = at(k);
        if (down) { if (v > (double)F) pick = max(pick, k); }
        else if ((float)v == F) pick = min(pick, k);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const int u = __shfl_xor_sync(0xffffffffu, pick, o);
        pick = down ? max(pick, u) : min(pick, u);
    }
    if (l32 == 0) ri_[warp] = pick;
    __syncthreads();
    if (threadIdx.x == 0) {
        int pk = ri_[0];
        for (int i = 1; i < TC_THREADS / 32; i++) pk = down ? max(pk, ri_[i]) : min(pk, ri_[i]);
        if (pk < 0 || pk >= ns) pk = 0;     // not reached: some element attains v*
        ri_[0] = pk;
    }
    __syncthreads();
    const int pk = ri_[0];
    const int ip = pk / nxc, jp = pk % nxc;
    const float jpeak = (float)(jp - P.xsearch), ipeak = (float)(ip - P.ysearch);
    if (threadIdx.x == 0) {
        int local, pidx;
        const PairDev pd = pair_of(P, w, local, pidx);
        xcg_result &o = pd.out[local];
        o.xoff = -1 * jpeak;
        o.yoff = -1 * ipeak;
        o.corr = F;
        o.ip = ip; o.jp = jp;
        o.flags = oob_sh ? XCG_FLAG_OOB : 0;
        o.cmax = vstar;
        o.cave = 0.0;
        o.cave_true = 0.0;
        o.gamma = (double)F;
        o.mean1 = P.means[2 * w];
        o.mean2 = P.means[2 * w + 1];
        o.corr0n = surf[0];
        o.fip = -1; o.fjp = -1; o.fmax = 0.f; o.xfrac = 0.f; o.yfrac = 0.f;
        P.corr0n[w] = surf[0];
    }
    // 8x8 neighbourhood with the reference's flat bounds test (conv_ampl_demean.cu:82-93)
    if (P.interp_flag) {
        const int n2 = P.n2x * P.n2y;
        const int jc = (nxc / 2) - P.n2x / 2 - (int)(-1 * jpeak);
        const int ic = (nyc / 2) - P.n2y / 2 - (int)(-1 * ipeak);
        for (int t = threadIdx.x; t < n2; t += TC_THREADS) {
            const int iy = t / P.n2x, ix = t - iy * P.n2x;
            const long long k = (long long)(ic + iy) * nxc + (jc + ix);
            float v = 0.f;
            unsigned char nx = 0;
            if (k >= 0 && k < ns) v = powf((float)surf[(size_t)(k / nxc) * P.qpitch + (k % nxc)], 0.25f);
            else if (k == ns) nx = 1;
            P.md[(size_t)w * n2 + t] = v;
            P.mdnext[(size_t)w * n2 + t] = nx;
        }
    }
}

}  // namespace

cudaError_t time_setup(const Plan &P) {
    cudaError_t e = cudaFuncSetAttribute(k_tcorr<0>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)tcorr_smem<0>(P.nx_corr));
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_tcorr<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tcorr_smem<1>(P.nx_corr));
    return e;
}

size_t time_smem_needed(int nx_corr, int mode) {
    return mode == 0 ? tcorr_smem<0>(nx_corr) : tcorr_smem<1>(nx_corr);
}

void launch_tcorr(const Plan &P, cudaStream_t s) {
    dim3 grid((P.nyc / TI) * (P.nxc / TJ), P.nwin);
    if (P.corr_mode == 0) k_tcorr<0><<<grid, TC_THREADS, tcorr_smem<0>(P.nx_corr), s>>>(P);
    else k_tcorr<1><<<grid, TC_THREADS, tcorr_smem<1>(P.nx_corr), s>>>(P);
}

void launch_tpeak(const Plan &P, cudaStream_t s) { k_tpeak<<<P.nwin, TC_THREADS, 0, s>>>(P); }

}  // namespace xcg
