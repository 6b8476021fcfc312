// Affine fit of a pair's offsets on the device: the step GMTSAR runs after
// xcorr (fitoffset.csh, called out at xcorr.cu:52; the script is not part of
// the reference sources) to turn freq_xcorr.dat into the PRM resampling
// parameters rshift, sub_int_r, stretch_r, a_stretch_r and their azimuth
// counterparts.  It reads the correlation results where they already are (the
// device result array), so a correlate-then-fit pipeline never copies
// offsets to the host.
//
// Model per axis: o(x, y) = c0 + c1*x + c2*y (npar 3), c0 + c1*x (npar 2) or
// c0 (npar 1), over the locations whose correlation exceeds snr_min, with the
// offsets computed exactly as print_results.c:37-38 writes them (float
// arithmetic).  Coordinates are centred and scaled to [-1, 1] for the normal
// equations, which are accumulated in double with a fixed reduction order
// (deterministic).  robust_iters > 0 adds iteratively reweighted passes with
// Tukey's biweight (c = 4.685 times the weighted rms residual of the
// previous pass).
#include <cuda_runtime.h>
#include <math.h>

#include "xcorr_gb300.h"

namespace xcg {
void set_last_error(const char *msg);
}

namespace {

constexpr int FIT_THREADS = 512;
constexpr int NS = 10;     // per axis: w, wu, wv, wuu, wuv, wvv, wo, wuo, wvo, woo

struct AxisModel {
    double c[3];           // in normalised coordinates
    double scale;          // robust weight scale (0: unweighted pass)
};

__device__ __forceinline__ void offsets_of(const xcg_result &r, const xcg_loc &l, int ri, int x_offset, int y_offset,
                                           double astretcha, float &orng, float &oazi) {
    const int ishft = (int)((double)l.y * astretcha);
    orng = (r.xoff / (float)ri) - (r.xfrac / (float)ri) + (float)x_offset;
    oazi = r.yoff - r.yfrac + (float)y_offset + (float)ishft;
}

// block-wide sum of NV doubles per thread, fixed order; result valid in thread 0
template <int NV>
__device__ void block_sum(double *v, double *sh) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < NV; k++)
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v[k] += __shfl_down_sync(0xffffffffu, v[k], o);
    if (lane == 0)
#pragma unroll
        for (int k = 0; k < NV; k++) sh[warp * NV + k] = v[k];
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int k = 0; k < NV; k++) {
            double s = 0.0;
            for (int q = 0; q < FIT_THREADS / 32; q++) s += sh[q * NV + k];
            v[k] = s;
        }
    }
    __syncthreads();
}

// Solve the (npar x npar) normal equations by Gaussian elimination with
// partial pivoting; singular systems leave the higher coefficients at 0.
__device__ void solve(const double *S, int npar, double *c) {
    double A[3][4];
    const double M[3][3] = {{S[0], S[1], S[2]}, {S[1], S[3], S[4]}, {S[2], S[4], S[5]}};
    const double b[3] = {S[6], S[7], S[8]};
    for (int i = 0; i < npar; i++) {
        for (int j = 0; j < npar; j++) A[i][j] = M[i][j];
        A[i][3] = b[i];
    }
    for (int k = 0; k < 3; k++) c[k] = 0.0;
    int rank = npar;
    for (int k = 0; k < npar; k++) {
        int p = k;
        for (int i = k + 1; i < npar; i++)
            if (fabs(A[i][k]) > fabs(A[p][k])) p = i;
        if (!(fabs(A[p][k]) > 1e-300)) { rank = k; break; }
        if (p != k)
            for (int j = 0; j < 4; j++) { const double t = A[k][j]; A[k][j] = A[p][j]; A[p][j] = t; }
        for (int i = k + 1; i < npar; i++) {
            const double f = A[i][k] / A[k][k];
            for (int j = k; j < 4; j++) A[i][j] -= f * A[k][j];
        }
    }
    for (int k = rank - 1; k >= 0; k--) {
        double s = A[k][3];
        for (int j = k + 1; j < rank; j++) s -= A[k][j] * c[j];
        c[k] = s / A[k][k];
    }
}

__global__ void __launch_bounds__(FIT_THREADS) k_fit(const xcg_result *__restrict__ res, const xcg_loc *__restrict__ locs,
                                                     int n, int ri, int x_offset, int y_offset, double astretcha,
                                                     float snr_min, int npar_r, int npar_a, int robust_iters,
                                                     xcg_fit *out) {
    __shared__ double sh[(FIT_THREADS / 32) * 2 * NS];
    __shared__ double geo[4];          // cx, hx, cy, hy
    __shared__ AxisModel mod[2];
    __shared__ int ntot;

    // pass 0: extent of the used locations
    double ext[4] = {1e300, -1e300, 1e300, -1e300};
    int cnt = 0;
    for (int i = threadIdx.x; i < n; i += FIT_THREADS) {
        const xcg_result r = res[i];
        float o1, o2;
        offsets_of(r, locs[i], ri, x_offset, y_offset, astretcha, o1, o2);
        if (!(r.corr > snr_min) || !isfinite(o1) || !isfinite(o2)) continue;
        const double x = locs[i].x, y = locs[i].y;
        ext[0] = fmin(ext[0], x); ext[1] = fmax(ext[1], x);
        ext[2] = fmin(ext[2], y); ext[3] = fmax(ext[3], y);
        cnt++;
    }
    {
        const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
        for (int o = 16; o > 0; o >>= 1) {
            ext[0] = fmin(ext[0], __shfl_down_sync(0xffffffffu, ext[0], o));
            ext[1] = fmax(ext[1], __shfl_down_sync(0xffffffffu, ext[1], o));
            ext[2] = fmin(ext[2], __shfl_down_sync(0xffffffffu, ext[2], o));
            ext[3] = fmax(ext[3], __shfl_down_sync(0xffffffffu, ext[3], o));
            cnt += __shfl_down_sync(0xffffffffu, cnt, o);
        }
        if (lane == 0) {
            sh[warp * 5 + 0] = ext[0]; sh[warp * 5 + 1] = ext[1];
            sh[warp * 5 + 2] = ext[2]; sh[warp * 5 + 3] = ext[3];
            sh[warp * 5 + 4] = (double)cnt;
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            double e[4] = {1e300, -1e300, 1e300, -1e300}, c = 0.0;
            for (int q = 0; q < FIT_THREADS / 32; q++) {
                e[0] = fmin(e[0], sh[q * 5 + 0]); e[1] = fmax(e[1], sh[q * 5 + 1]);
                e[2] = fmin(e[2], sh[q * 5 + 2]); e[3] = fmax(e[3], sh[q * 5 + 3]);
                c += sh[q * 5 + 4];
            }
            if (c == 0.0) { e[0] = e[1] = e[2] = e[3] = 0.0; }
            ntot = (int)c;
            geo[0] = 0.5 * (e[0] + e[1]);
            geo[1] = (e[1] > e[0]) ? 0.5 * (e[1] - e[0]) : 1.0;
            geo[2] = 0.5 * (e[2] + e[3]);
            geo[3] = (e[3] > e[2]) ? 0.5 * (e[3] - e[2]) : 1.0;
            mod[0].scale = mod[1].scale = 0.0;
        }
        __syncthreads();
    }
    const double cx = geo[0], hx = geo[1], cy = geo[2], hy = geo[3];

    double S[2][NS];
    for (int pass = 0; pass <= robust_iters; pass++) {
        const AxisModel m0 = mod[0], m1 = mod[1];
        for (int a = 0; a < 2; a++)
            for (int k = 0; k < NS; k++) S[a][k] = 0.0;
        for (int i = threadIdx.x; i < n; i += FIT_THREADS) {
            const xcg_result r = res[i];
            float o1, o2;
            offsets_of(r, locs[i], ri, x_offset, y_offset, astretcha, o1, o2);
            if (!(r.corr > snr_min) || !isfinite(o1) || !isfinite(o2)) continue;
            const double u = ((double)locs[i].x - cx) / hx, v = ((double)locs[i].y - cy) / hy;
            const double o[2] = {(double)o1, (double)o2};
            const AxisModel *mm[2] = {&m0, &m1};
            for (int a = 0; a < 2; a++) {
                double w = 1.0;
                if (mm[a]->scale > 0.0) {
                    const double rr = (o[a] - (mm[a]->c[0] + mm[a]->c[1] * u + mm[a]->c[2] * v)) / (4.685 * mm[a]->scale);
                    w = fabs(rr) < 1.0 ? (1.0 - rr * rr) * (1.0 - rr * rr) : 0.0;
                }
                S[a][0] += w; S[a][1] += w * u; S[a][2] += w * v;
                S[a][3] += w * u * u; S[a][4] += w * u * v; S[a][5] += w * v * v;
                S[a][6] += w * o[a]; S[a][7] += w * u * o[a]; S[a][8] += w * v * o[a];
                S[a][9] += w * o[a] * o[a];
            }
        }
        block_sum<2 * NS>(&S[0][0], sh);
        if (threadIdx.x == 0) {
            for (int a = 0; a < 2; a++) {
                const int np = a == 0 ? npar_r : npar_a;
                double c[3];
                solve(S[a], np, c);
                // weighted residual sum of squares from the sums:
                // sum w (o - c.phi)^2 = woo - 2 c.(wo, wuo, wvo) + c^T M c
                const double *s = S[a];
                const double q = s[9] - 2.0 * (c[0] * s[6] + c[1] * s[7] + c[2] * s[8]) +
                                 c[0] * (c[0] * s[0] + c[1] * s[1] + c[2] * s[2]) +
                                 c[1] * (c[0] * s[1] + c[1] * s[3] + c[2] * s[4]) +
                                 c[2] * (c[0] * s[2] + c[1] * s[4] + c[2] * s[5]);
                mod[a].c[0] = c[0]; mod[a].c[1] = c[1]; mod[a].c[2] = c[2];
                // scale 0 (an exact fit) keeps the next pass unweighted
                mod[a].scale = s[0] > 0.0 ? sqrt(fmax(q, 0.0) / s[0]) : 0.0;
            }
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        for (int a = 0; a < 2; a++) {
            const AxisModel &m = mod[a];
            xcg_fit_axis f;
            // back to pixel coordinates: o = c0 + c1 (x - cx)/hx + c2 (y - cy)/hy
            f.stretch = m.c[1] / hx;
            f.a_stretch = m.c[2] / hy;
            f.shift = m.c[0] - f.stretch * cx - f.a_stretch * cy;
            f.ishift = (int32_t)f.shift;            // truncation, as (int) and awk int() do
            f.sub_int = f.shift - (double)f.ishift;
            f.weight = S[a][0];
            f.rms = m.scale;
            f.npts = ntot;
            if (a == 0) out->range = f; else out->azimuth = f;
        }
    }
}

}  // namespace

extern "C" xcg_status xcg_fit_offsets(const xcg_result *d_results, const xcg_loc *d_locs, int32_t nlocs, int32_t ri,
                                      int32_t x_offset, int32_t y_offset, double astretcha, float snr_min,
                                      int32_t npar_range, int32_t npar_azimuth, int32_t robust_iters, xcg_fit *d_out,
                                      void *stream) {
    if (!d_results || !d_locs || !d_out || nlocs < 0 || ri < 1 || npar_range < 1 || npar_range > 3 ||
        npar_azimuth < 1 || npar_azimuth > 3 || robust_iters < 0 || robust_iters > 100) {
        xcg::set_last_error("xcg_fit_offsets: invalid argument");
        return XCG_ERR_ARG;
    }
    k_fit<<<1, FIT_THREADS, 0, (cudaStream_t)stream>>>(d_results, d_locs, nlocs, ri, x_offset, y_offset, astretcha,
                                                        snr_min, npar_range, npar_azimuth, robust_iters, d_out);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        xcg::set_last_error(cudaGetErrorString(e));
        return XCG_ERR_CUDA;
    }
    return XCG_OK;
}
