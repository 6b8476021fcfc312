/* Per-precision body of the oracle (test infrastructure).  Included twice
 * by xcorr_oracle.c with R = float (XO_F32, the reference's float data path)
 * and R = double (XO_F64).  Each function cites the reference lines it
 * restates. */

#define XN(name) XCAT(name, SFX)

/* In-place complex FFT of length n (power of two), unnormalised, sign -1
 * forward (e^{-2 pi i nk/N}) and +1 inverse, the cuFFT conventions the
 * reference calls (fft_interpolate_routines.cu:89-105, do_freq_xcorr.cu:99-113).
 * Iterative radix-2 decimation in time. */
static void XN(fft)(R *x, int n, int sign)
{
    const xo_tab *t = tab_get(n);
    const R *wr = (const R *)XN(tab_cos)(t), *wi = (const R *)XN(tab_sin)(t);
    for (int i = 0; i < n; i++) {
        int j = t->rev[i];
        if (j > i) {
            R a = x[2 * i], b = x[2 * i + 1];
            x[2 * i] = x[2 * j]; x[2 * i + 1] = x[2 * j + 1];
            x[2 * j] = a; x[2 * j + 1] = b;
        }
    }
    for (int len = 2; len <= n; len <<= 1) {
        int half = len >> 1, step = n / len;
        for (int i = 0; i < n; i += len) {
            for (int k = 0; k < half; k++) {
                R c = wr[k * step];
                R s = sign < 0 ? wi[k * step] : -wi[k * step];   /* table holds -sin */
                R *a = x + 2 * (i + k), *b = x + 2 * (i + k + half);
                R tr = b[0] * c - b[1] * s;
                R ti = b[0] * s + b[1] * c;
                b[0] = a[0] - tr; b[1] = a[1] - ti;
                a[0] = a[0] + tr; a[1] = a[1] + ti;
            }
        }
    }
}

/* 1-D zero-pad interpolation of one row by ifactor
 * (d_fft_interpolate_1d_strip, fft_interpolate_routines.cu:76-113):
 * forward FFT of N, first N/2 bins to [0,N/2), last N/2 to [M-N/2,M),
 * inverse FFT of M = ifactor*N, scale by (float)(ifactor*2.0/(2M)).
 * in: N complex (overwritten by its spectrum), out: M complex. */
static void XN(interp1d)(R *in, int N, int ifactor, R *out)
{
    int M = ifactor * N, N2 = N / 2;
    XN(fft)(in, N, -1);
    memset(out, 0, sizeof(R) * 2 * (size_t)M);
    memcpy(out, in, sizeof(R) * 2 * (size_t)N2);
    memcpy(out + 2 * (size_t)(2 * ifactor - 1) * N2, in + 2 * (size_t)N2, sizeof(R) * 2 * (size_t)N2);
    XN(fft)(out, M, +1);
    R nm = (R)((double)ifactor * 2.0 / (2.0 * (double)M));
    for (int i = 0; i < 2 * M; i++) out[i] = out[i] * nm;
}

/* Range interpolation of one patch row (xcorr.cu:237-250): interpolate by ri
 * and keep fine samples [N/2, 3N/2). row: N complex in/out; work: ri*N complex. */
static void XN(range_row)(R *row, int N, int ri, R *work)
{
    XN(interp1d)(row, N, ri, work);
    memcpy(row, work + N, sizeof(R) * 2 * (size_t)N);    /* d_work + nx/2 complex */
}

/* Reference FP32 block sum over 1024 elements (reduce6<float,512>,
 * conv_ampl_demean.cu:350-429 launched by h_reduceFD_strip :703-726):
 * s[t] = x[t] + x[t+512], then pairs at strides 256,128,64,32,16,...,1. */
static float XN(block1024_sum_f32)(const R *x)
{
    float s[512];
    for (int t = 0; t < 512; t++) s[t] = (float)x[t] + (float)x[t + 512];
    for (int st = 256; st >= 1; st >>= 1)
        for (int t = 0; t < st; t++) s[t] = s[t] + s[t + st];
    return s[0];
}

/* Amplitude, mean, demean/mask, int copy of one patch (xcorr.cu:261-292;
 * d_conv_ampl_strip conv_ampl_demean.cu:98-108; h_reduceFD_strip :703-726;
 * d_mean_mask_strip :111-139; make_mask xcorr.cu:385-401).
 * c: npy*npx complex, in: range-interpolated patch, out: real part demeaned
 * (and masked for the slave), imag 0.  amp (optional) gets the amplitudes. */
static double XN(prep_patch)(const xo_params *p, R *c, int slave, int32_t *ints, float *amp)
{
    const int npx = p->npx, npy = p->npy, n = npx * npy;
    R *a = (R *)malloc(sizeof(R) * (size_t)n);
    for (int i = 0; i < n; i++) {
#if XO_IS_F32
        float v = hypotf((float)c[2 * i], (float)c[2 * i + 1]);
#else
        double v = hypot(c[2 * i], c[2 * i + 1]);
#endif
        a[i] = v;
        if (amp) amp[i] = (float)v;
    }
    double mean = 0.0;
#if XO_IS_F32
    for (int b = 0; b < n / 1024; b++) mean += (double)XN(block1024_sum_f32)(a + 1024 * b);
#else
    for (int i = 0; i < n; i++) mean += a[i];
#endif
    mean /= (double)n;
    const R m = (R)mean;
    for (int r = 0; r < npy; r++) {
        for (int col = 0; col < npx; col++) {
            int i = r * npx + col;
            R supp = 1;
            if (slave) {
                int in = !((r < p->ysearch) || (r >= npy - p->ysearch) ||
                           (col < p->xsearch) || (col >= npx - p->xsearch));
                supp = (R)in;
            }
            R v = a[i] - m;
            v = v * supp;
            c[2 * i] = v;
            c[2 * i + 1] = 0;
            ints[i] = (int32_t)v;
        }
    }
    free(a);
    return mean;
}

/* 2-D FFT of an ny x nx complex array, rows then columns. */
static void XN(fft2)(R *c, int nx, int ny, int sign, R *col)
{
    for (int r = 0; r < ny; r++) XN(fft)(c + 2 * (size_t)r * nx, nx, sign);
    for (int x = 0; x < nx; x++) {
        for (int r = 0; r < ny; r++) { col[2 * r] = c[2 * ((size_t)r * nx + x)]; col[2 * r + 1] = c[2 * ((size_t)r * nx + x) + 1]; }
        XN(fft)(col, ny, sign);
        for (int r = 0; r < ny; r++) { c[2 * ((size_t)r * nx + x)] = col[2 * r]; c[2 * ((size_t)r * nx + x) + 1] = col[2 * r + 1]; }
    }
}

/* Correlation surface of one window (d_fft_multiply_strip do_freq_xcorr.cu:90-117,
 * d_mulaconjb :46-64, d_Cmul :32-43, d_scaleFft2D fft_interpolate_routines.cu:59-70,
 * d_fillcorrmat_strip do_freq_xcorr.cu:67-84, d_Cabs :26-29).
 * c1, c2: prepared patches (overwritten).  corr: nyc x nxc doubles. */
static void XN(surface)(const xo_params *p, R *c1, R *c2, double *corr)
{
    const int N = p->npx, M = p->npy;
    R *col = (R *)malloc(sizeof(R) * 2 * (size_t)(M > N ? M : N));
    XN(fft2)(c1, N, M, -1, col);
    XN(fft2)(c2, N, M, -1, col);
    for (int iy = 0; iy < M; iy++) {
        for (int ix = 0; ix < N; ix++) {
            size_t i = (size_t)iy * N + ix;
            R ar = c1[2 * i], ai = c1[2 * i + 1];
            R br = c2[2 * i], bi = -c2[2 * i + 1];          /* cuConjf */
#if XO_IS_F32
            double zx = (double)(float)(ar * br), zy = (double)(float)(ai * bi);
            float zr = (float)(zx - zy);
            zx = (double)(float)(ai * br); zy = (double)(float)(ar * bi);
            float zi = (float)(zx + zy);
#else
            double zr = ar * br - ai * bi, zi = ai * br + ar * bi;
#endif
            R sgn = ((ix + iy) % 2 == 0) ? (R)1 : (R)-1;
            c1[2 * i] = zr * sgn;
            c1[2 * i + 1] = zi * sgn;
        }
    }
    XN(fft2)(c1, N, M, +1, col);
    const R nm = (R)(N * M);
    for (int y = 0; y < p->nyc; y++) {
        for (int x = 0; x < p->nxc; x++) {
            size_t ii = (size_t)(y + p->ny_corr / 2) * N + x + p->nx_corr / 2;
            R re = c1[2 * ii] / nm, im = c1[2 * ii + 1] / nm;
#if XO_IS_F32
            corr[(size_t)y * p->nxc + x] = (double)(float)hypot((double)re, (double)im);
#else
            corr[(size_t)y * p->nxc + x] = hypot(re, im);
#endif
        }
    }
    free(col);
}

/* 8x8 neighbourhood of the peak with the reference's flat bounds test
 * (d_cppow_strip, conv_ampl_demean.cu:75-95): md = corr^0.25 around
 * (xoff, yoff); next = 1 where it reads element nxc*nyc (the next window's
 * first value). */
static void XN(neighbourhood)(const xo_params *p, const double *corr, const xo_result *r, double *md,
                              unsigned char *next)
{
    const int64_t ns = (int64_t)p->nxc * p->nyc;
    int jc = (p->nxc / 2) - p->n2x / 2 - (int)r->xoff;
    int ic = (p->nyc / 2) - p->n2y / 2 - (int)r->yoff;
    for (int y = 0; y < p->n2y; y++) {
        for (int x = 0; x < p->n2x; x++) {
            int64_t k = (int64_t)(ic + y) * p->nxc + (jc + x);
            md[y * p->n2x + x] = 0.0;
            next[y * p->n2x + x] = 0;
            if (k < 0 || k > ns) continue;
            if (k == ns) { next[y * p->n2x + x] = 1; continue; }
#if XO_IS_F32
            md[y * p->n2x + x] = (double)powf((float)corr[k], 0.25f);
#else
            md[y * p->n2x + x] = pow(corr[k], 0.25);
#endif
        }
    }
}

/* Phase A of one window: everything up to the normalised surface and the
 * 8x8 neighbourhood (d_assign_values xcorr.cu:261-292, d_do_freq_corr_strip
 * do_freq_xcorr.cu:123-200, d_calc_time_corr_strip do_time_int_xcorr.cu:71-100,
 * d_scaled_strip conv_ampl_demean.cu:50-68, d_cppow_strip :75-95).
 * pm/ps: patches, npy*npx complex float.  md: n2y*n2x values; next: 1 where the
 * reference reads corr[nxc*nyc] (the following window's first element). */
static void XN(window_a)(const xo_params *p, const float *pm, const float *ps, xo_result *r,
                         double *md, unsigned char *next)
{
    const int N = p->npx, M = p->npy, n = N * M;
    R *c1 = (R *)malloc(sizeof(R) * 2 * (size_t)n);
    R *c2 = (R *)malloc(sizeof(R) * 2 * (size_t)n);
    R *work = (R *)malloc(sizeof(R) * 2 * (size_t)N * (p->ri > 1 ? p->ri : 1));
    int32_t *i1 = (int32_t *)malloc(sizeof(int32_t) * (size_t)n);
    int32_t *i2 = (int32_t *)malloc(sizeof(int32_t) * (size_t)n);
    double *corr = (double *)malloc(sizeof(double) * (size_t)p->nxc * p->nyc);
    for (int i = 0; i < 2 * n; i++) { c1[i] = (R)pm[i]; c2[i] = (R)ps[i]; }
    if (p->ri > 1) {
        for (int row = 0; row < M; row++) {
            XN(range_row)(c1 + 2 * (size_t)row * N, N, p->ri, work);
            XN(range_row)(c2 + 2 * (size_t)row * N, N, p->ri, work);
        }
    }
    r->mean1 = XN(prep_patch)(p, c1, 0, i1, NULL);
    r->mean2 = XN(prep_patch)(p, c2, 1, i2, NULL);
    const int64_t ns = (int64_t)p->nxc * p->nyc;
    if (p->corr_mode < 2) {
        /* -time / -time4: the full-search surface replaces the FFT surface and
         * feeds the same 8x8 neighbourhood (no normalisation) */
        time_surface(p, i1, i2, corr);
        time_peak(p, corr, r);
        XN(neighbourhood)(p, corr, r, md, next);
        free(c1); free(c2); free(work); free(i1); free(i2); free(corr);
        return;
    }
    XN(surface)(p, c1, c2, corr);

    double cmax;
    int64_t peak = xo_argmax_ref(corr, ns, &cmax);
    r->cmax = cmax;
    r->cave = xo_half_sum_ref(corr, ns) / (double)ns;
    double tot = 0.0;
    for (int64_t i = 0; i < ns; i++) tot += corr[i];
    r->cave_true = tot / (double)ns;
    r->ip = (int32_t)(peak / p->nxc);
    r->jp = (int32_t)(peak % p->nxc);
    float jpeak = (float)r->jp - (float)p->nxc / 2.0f;
    float ipeak = (float)r->ip - (float)p->nyc / 2.0f;
    r->xoff = -1 * jpeak;
    r->yoff = -1 * ipeak;

    /* time-domain correlation at the integer peak (do_freq_xcorr.cu:170-178) */
    int64_t num = 0, d1 = 0, d2 = 0;
    for (int y = 0; y < p->ny_corr; y++) {
        for (int x = 0; x < p->nx_corr; x++) {
            int64_t a = i1[(p->ysearch + (int)ipeak + y) * N + (int)jpeak + p->xsearch + x];
            int64_t b = i2[(p->ysearch + y) * N + p->xsearch + x];
            num += a * b; d1 += a * a; d2 += b * b;
        }
    }
    double gd = sqrt(1.0 * (double)d1 * (double)d2);
    double gamma = (gd == 0.0) ? 0.0 : 100.0 * fabs((double)num / gd);
    r->gamma = gamma;
    r->corr = (float)gamma;
    double msc = cmax / gamma;
    for (int64_t i = 0; i < ns; i++) corr[i] = corr[i] / msc;
    r->corr0n = corr[0];

    XN(neighbourhood)(p, corr, r, md, next);
    free(c1); free(c2); free(work); free(i1); free(i2); free(corr);
}

static double XN(pow_quarter)(double v)
{
#if XO_IS_F32
    return (double)powf((float)v, 0.25f);
#else
    return pow(v, 0.25);
#endif
}

/* Phase B: 2-D FFT zero-pad interpolation of the 8x8 block by ifc and the
 * argmax of the real part (d_do_highres_corr highres_corr.cu:23-79,
 * d_fft_interpolate_2d_strip fft_interpolate_routines.cu:118-147,
 * h_reduceCr_strip conv_ampl_demean.cu:730-756). */
static void XN(window_b)(const xo_params *p, const double *md, xo_result *r, double *re_out)
{
    const int nx = p->n2x, ny = p->n2y, ifc = p->ifc;
    const int nx2 = nx * ifc, ny2 = ny * ifc;
    R *rows = (R *)malloc(sizeof(R) * 2 * (size_t)ny * nx2);   /* ny rows of nx2 */
    R *in = (R *)malloc(sizeof(R) * 2 * (size_t)(nx > ny ? nx : ny));
    R *colo = (R *)malloc(sizeof(R) * 2 * (size_t)ny2);
    double *re = (double *)malloc(sizeof(double) * (size_t)nx2 * ny2);
    for (int y = 0; y < ny; y++) {
        for (int x = 0; x < nx; x++) { in[2 * x] = (R)md[y * nx + x]; in[2 * x + 1] = 0; }
        XN(interp1d)(in, nx, ifc, rows + 2 * (size_t)y * nx2);
    }
    for (int X = 0; X < nx2; X++) {
        for (int y = 0; y < ny; y++) { in[2 * y] = rows[2 * ((size_t)y * nx2 + X)]; in[2 * y + 1] = rows[2 * ((size_t)y * nx2 + X) + 1]; }
        XN(interp1d)(in, ny, ifc, colo);
        for (int Y = 0; Y < ny2; Y++) re[(size_t)Y * nx2 + X] = (double)colo[2 * Y];
    }
    if (re_out) memcpy(re_out, re, sizeof(double) * (size_t)nx2 * ny2);
    double vmax;
    int64_t pk = xo_argmax_ref(re, (int64_t)nx2 * ny2, &vmax);
    r->fip = (int32_t)(pk / nx2);
    r->fjp = (int32_t)(pk % nx2);
    r->fmax = (float)vmax;
    float jpeak = (float)r->fjp - (float)ny2 / 2.0f;     /* ny2 for both axes, highres_corr.cu:61-62 */
    float ipeak = (float)r->fip - (float)ny2 / 2.0f;
    r->xfrac = jpeak / (float)ifc;
    r->yfrac = ipeak / (float)ifc;
    free(rows); free(in); free(colo); free(re);
}

#undef XN
