// Team FFT: an N-point complex FFT computed by a team of T lanes of one warp
// in shared memory (Stockham auto-sort, radix-16 passes then one radix-8/4/2
// pass, natural order in and out, unnormalised; the conventions of the
// forward/inverse transforms the reference takes from cuFFT,
// fft_interpolate_routines.cu:89-105 and do_freq_xcorr.cu:99-113).
//
// Pass p with stride Ns and radix R: lane j (j < N/R, several per lane when
// N/R > T) loads x[j + r N/R] for r < R, multiplies by w_{Ns R}^{(j mod Ns) r},
// does an R-point DFT in registers and stores it to y[(j - j mod Ns) R + j mod Ns + r Ns].
// Shared-memory index i is padded to i + i/16, which makes every pass of
// N = 128..1024 conflict-free for 8-byte accesses.
// Pass twiddles live in a table laid out [pass][r-1][k] so that lanes with
// consecutive k read consecutive words; the host builds it in double.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace xcg {

__host__ __device__ constexpr int fft_pad(int i) { return i + (i >> 4); }
__host__ __device__ constexpr int fft_padded_len(int n) { return n + (n >> 4); }

// radix list: 16 while the remainder is >= 16, then the remainder
__host__ __device__ constexpr int fft_npasses(int n) {
    int p = 0;
    while (n >= 16) { n >>= 4; p++; }
    return p + (n > 1 ? 1 : 0);
}
__host__ __device__ constexpr int fft_radix(int n, int pass) {
    for (int p = 0; p < pass; p++) n = (n >= 16) ? (n >> 4) : 1;
    return n >= 16 ? 16 : n;
}
// number of twiddle entries of all passes (first pass needs none)
__host__ __device__ constexpr int fft_twiddle_len(int n) {
    int len = 0, ns = 1;
    for (int p = 0; p < fft_npasses(n); p++) {
        int r = fft_radix(n, p);
        if (p > 0) len += (r - 1) * ns;
        ns *= r;
    }
    return len;
}

// a + b and a * b + c on both components: sm_100's two-lane FP32 instructions,
// rounded per component as the scalar ones
__device__ __forceinline__ float2 fadd2(float2 a, float2 b) {
#if defined(__CUDA_ARCH__) && __CUDA_ARCH__ >= 1000
    return __fadd2_rn(a, b);
#else
    return make_float2(a.x + b.x, a.y + b.y);
#endif
}
__device__ __forceinline__ float2 ffma2(float2 a, float2 b, float2 c) {
#if defined(__CUDA_ARCH__) && __CUDA_ARCH__ >= 1000
    return __ffma2_rn(a, b, c);
#else
    return make_float2(fmaf(a.x, b.x, c.x), fmaf(a.y, b.y, c.y));
#endif
}

__device__ __forceinline__ float2 cmulf(float2 a, float2 b) {
    return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ float2 cmulf_conj(float2 a, float2 b) {   // a * conj(b)
    return make_float2(a.x * b.x + a.y * b.y, a.y * b.x - a.x * b.y);
}

// cos / sin of 2*pi*m/16
__device__ constexpr float kC1 = 0.923879532511286756128f;   // cos(pi/8)
__device__ constexpr float kS1 = 0.382683432365089771728f;   // sin(pi/8)
__device__ constexpr float kR2 = 0.707106781186547524401f;   // sqrt(2)/2

// b * exp(DIR * 2*pi*i * M16 / 16), with the trivial rotations written out
template <int M16, int DIR>
__device__ __forceinline__ float2 rot16(float2 b) {
    constexpr int m = ((M16 % 16) + 16) % 16;
    if constexpr (m == 0) {
        return b;
    } else if constexpr (m == 8) {
        return make_float2(-b.x, -b.y);
    } else if constexpr (m == 4) {      // exp(DIR i pi/2) = DIR * i
        return DIR < 0 ? make_float2(b.y, -b.x) : make_float2(-b.y, b.x);
    } else if constexpr (m == 12) {     // exp(DIR i 3pi/2) = -DIR * i
        return DIR < 0 ? make_float2(-b.y, b.x) : make_float2(b.y, -b.x);
    } else {
        constexpr int q = m & 3;        // angle within a quadrant: q * pi/8
        constexpr float cq = (q == 1) ? kC1 : (q == 2) ? kR2 : kS1;
        constexpr float sq = (q == 1) ? kS1 : (q == 2) ? kR2 : kC1;
        // rotate into quadrant m/4
        constexpr int quad = m >> 2;
        constexpr float c = (quad == 0) ? cq : (quad == 1) ? -sq : (quad == 2) ? -cq : sq;
        constexpr float s0 = (quad == 0) ? sq : (quad == 1) ? cq : (quad == 2) ? -sq : -cq;
        constexpr float s = DIR * s0;
        return make_float2(b.x * c - b.y * s, b.x * s + b.y * c);
    }
}

template <int R>
__host__ __device__ constexpr int bitrev_c(int i) {
    int r = 0;
    for (int b = 1, k = R >> 1; b < R; b <<= 1, k >>= 1)
        if (i & b) r |= k;
    return r;
}

// tan(pi/8) = sqrt(2) - 1
__device__ constexpr float kT1 = 0.414213562373095048802f;

// a +- b * exp(DIR * 2*pi*i * M16 / 16) for a rotation that is not a
// multiple of a quarter turn, factored as in the tangent (Linzer-Feig)
// butterfly: b * (c + i s) = f * (b + i r b) with f the larger of |c|, |s|
// (signed) and |r| <= 1, so the pair costs 2 + 4 fused operations instead of
// a 4-operation rotation and 4 additions.
template <int M16, int DIR>
__device__ __forceinline__ void tan_butterfly(float2 &a, float2 &b) {
    constexpr int m = ((M16 % 16) + 16) % 16;
    constexpr int q = m & 3;                      // angle within a quadrant: q * pi/8 (q != 0)
    constexpr int quad = m >> 2;
    // the rotation in quadrant 0 is (cq, sq); quadrant k multiplies by i^k
    constexpr float cq = (q == 1) ? kC1 : (q == 2) ? kR2 : kS1;
    constexpr float sq = (q == 1) ? kS1 : (q == 2) ? kR2 : kC1;
    constexpr float c = (quad == 0) ? cq : (quad == 1) ? -sq : (quad == 2) ? -cq : sq;
    constexpr float s = DIR * ((quad == 0) ? sq : (quad == 1) ? cq : (quad == 2) ? -sq : -cq);
    float2 u;
    float f;
    if constexpr (q == 2) {                       // |c| = |s|: r = s / c = +-1
        f = c;
        u = (s == c) ? make_float2(b.x - b.y, b.y + b.x) : make_float2(b.x + b.y, b.y - b.x);
    } else if constexpr ((q == 1) == (quad == 0 || quad == 2)) {   // |c| > |s|: factor c, r = s / c
        constexpr float r = ((s > 0.f) == (c > 0.f)) ? kT1 : -kT1;
        f = c;
        u = make_float2(fmaf(-r, b.y, b.x), fmaf(r, b.x, b.y));
    } else {                                      // |s| > |c|: factor s, b (c + i s) = s (r b + i b), r = c / s
        constexpr float r = ((s > 0.f) == (c > 0.f)) ? kT1 : -kT1;
        f = s;
        u = make_float2(fmaf(r, b.x, -b.y), fmaf(r, b.y, b.x));
    }
    const float2 a0 = a;
    a = make_float2(fmaf(f, u.x, a0.x), fmaf(f, u.y, a0.y));
    b = make_float2(fmaf(-f, u.x, a0.x), fmaf(-f, u.y, a0.y));
}

// One butterfly stage of length LEN inside an R-point register DFT.
template <int R, int LEN, int DIR, int K>
struct DftStage {
    static __device__ __forceinline__ void run(float2 *t, int i) {
        if constexpr (K < LEN / 2) {
            constexpr int M16 = K * (16 / LEN);
            if constexpr (M16 == 0) {             // no rotation: a +- b on both components at once
                // (a - b as b * -1 + a, rounded once: the scalar difference)
                const float2 a = t[i + K], b = t[i + K + LEN / 2];
                t[i + K] = fadd2(a, b);
                t[i + K + LEN / 2] = ffma2(b, make_float2(-1.f, -1.f), a);
            } else if constexpr ((M16 & 3) == 0) {   // quarter turns: exact swaps and signs
                float2 a = t[i + K];
                float2 b = rot16<M16, DIR>(t[i + K + LEN / 2]);
                t[i + K] = make_float2(a.x + b.x, a.y + b.y);
                t[i + K + LEN / 2] = make_float2(a.x - b.x, a.y - b.y);
            } else {
                float2 a = t[i + K], b = t[i + K + LEN / 2];
                tan_butterfly<M16, DIR>(a, b);
                t[i + K] = a;
                t[i + K + LEN / 2] = b;
            }
            DftStage<R, LEN, DIR, K + 1>::run(t, i);
        }
    }
};

template <int R, int LEN, int DIR>
__device__ __forceinline__ void dft_level(float2 *t) {
    if constexpr (LEN <= R) {
#pragma unroll
        for (int i = 0; i < R; i += LEN) DftStage<R, LEN, DIR, 0>::run(t, i);
        dft_level<R, LEN * 2, DIR>(t);
    }
}

// R-point DFT of v (R = 2, 4, 8, 16) in registers, natural order in and out.
template <int R, int DIR>
__device__ __forceinline__ void dft_reg(float2 *v) {
    float2 t[R];
#pragma unroll
    for (int i = 0; i < R; i++) t[i] = v[bitrev_c<R>(i)];
    dft_level<R, 2, DIR>(t);
#pragma unroll
    for (int i = 0; i < R; i++) v[i] = t[i];
}

// 16-point DFT of a sequence that is zero outside elements [4, 12), natural
// order in and out: the first butterfly level pairs element k with k + 8,
// one of which is zero, so that level is copies and negations.
template <int DIR>
__device__ __forceinline__ void dft16_mid(float2 *v) {
    float2 t[16];
#pragma unroll
    for (int i = 0; i < 16; i += 2) {
        const int k = bitrev_c<16>(i);           // 0..7
        if (k < 4) {                              // element k is zero
            const float2 b = v[k + 8];
            t[i] = b;
            t[i + 1] = make_float2(-b.x, -b.y);
        } else {                                  // element k + 8 is zero
            t[i] = v[k];
            t[i + 1] = v[k];
        }
    }
    dft_level<16, 4, DIR>(t);
#pragma unroll
    for (int i = 0; i < 16; i++) v[i] = t[i];
}

// One Stockham pass.  tw: this pass's twiddles [R-1][Ns] (forward sign).
template <int N, int R, int DIR>
__device__ __forceinline__ void stockham_pass(const float2 *__restrict__ src, float2 *__restrict__ dst,
                                              int Ns, const float2 *__restrict__ tw, int lane, int T) {
    constexpr int NR = N / R;
    for (int j = lane; j < NR; j += T) {
        float2 v[R];
        const int k = j & (Ns - 1);
#pragma unroll
        for (int r = 0; r < R; r++) v[r] = src[fft_pad(j + r * NR)];
        if (Ns > 1) {
#pragma unroll
            for (int r = 1; r < R; r++) {
                float2 w = tw[(r - 1) * Ns + k];
                v[r] = DIR < 0 ? cmulf(v[r], w) : cmulf_conj(v[r], w);
            }
        }
        dft_reg<R, DIR>(v);
        const int idxD = (j - k) * R + k;
#pragma unroll
        for (int r = 0; r < R; r++) dst[fft_pad(idxD + r * Ns)] = v[r];
    }
}

template <int N, int DIR, int PASS>
__device__ __forceinline__ float2 *team_fft_from(float2 *a, float2 *b, const float2 *tw, int Ns, int lane, int T) {
    if constexpr (PASS >= fft_npasses(N)) {
        return a;
    } else {
        constexpr int R = fft_radix(N, PASS);
        stockham_pass<N, R, DIR>(a, b, Ns, tw, lane, T);
        __syncwarp();
        const float2 *tw_next = (PASS == 0) ? tw : tw + (R - 1) * Ns;
        return team_fft_from<N, DIR, PASS + 1>(b, a, tw_next, Ns * R, lane, T);
    }
}

// N-point FFT of the padded sequence in a (scratch b, same size); returns the
// buffer holding the result.  tw: the size-N table (fft_twiddle_len(N) entries).
// Every lane of the warp must call it (it ends each pass with __syncwarp).
template <int N, int DIR>
__device__ __forceinline__ float2 *team_fft(float2 *a, float2 *b, const float2 *tw, int lane, int T) {
    return team_fft_from<N, DIR, 0>(a, b, tw, 1, lane, T);
}

}  // namespace xcg

namespace xcg {

// ---------------------------------------------------------------------------
// Register-resident team FFT.  The same Stockham passes, but the sequence
// lives in registers between passes: lane l of the team holds elements
// l + T*m (m < N/T) on entry and the transform's elements l + T*m on exit,
// and only the passes in between go through shared memory (one padded
// N-point exchange buffer per team, used in place: every pass reads all its
// inputs, syncs, then writes).  For N = 256 that is one exchange per FFT.
// Global loads and stores in the l + T*m layout are coalesced.

__host__ __device__ constexpr int fft_lanes(int n) { return (n / 16 < 32) ? n / 16 : 32; }

// cos(2 pi k / 32) and sin(2 pi k / 32), any integer k
__host__ __device__ constexpr float cos32_oct(int k) {      // k in 0..8
    return k == 0 ? 1.0f : k == 1 ? 0.980785280403230449126f : k == 2 ? 0.923879532511286756128f
         : k == 3 ? 0.831469612302545237079f : k == 4 ? 0.707106781186547524401f : k == 5 ? 0.555570233019602224743f
         : k == 6 ? 0.382683432365089771728f : k == 7 ? 0.195090322016128267848f : 0.0f;
}
__host__ __device__ constexpr float cos32(int k) {
    k = ((k % 32) + 32) % 32;
    return k <= 8 ? cos32_oct(k) : k <= 16 ? -cos32_oct(16 - k) : k <= 24 ? -cos32_oct(k - 16) : cos32_oct(32 - k);
}
__host__ __device__ constexpr float sin32(int k) { return cos32(k - 8); }

// HS (half-sample shift, inverse transforms of N = 128, 256 or 512): the
// input element f = lane + T*m is first multiplied by phi(f) = exp(i pi f'/N)
// / N (f' = f, or f - N for f >= N/2), which turns the inverse FFT into the
// half-sample shifted interpolation.  phi(f) = A(lane) * C(m): C(m) =
// exp(2 pi i m / 32) / N, negated for m >= 8, is a constant multiplied here;
// A(lane) = exp(i pi lane / N) rides on the later passes' twiddles.  For
// N <= 256 the pass-0 outputs of lane l are the next pass's inputs r = l, so
// that pass's table holds exp(-2 pi i r (k + 1/2) / N).  For N = 512 (T = 32,
// passes 16, 16, 2) pass 1's input r of lane j came from lane (j >> 4) + 2r:
// the factor exp(2 pi i r / 512) goes into pass 1's table, exp(-2 pi i r
// (k + 1/2) / 256), and the lane's common factor exp(i pi (j >> 4) / 512)
// reaches pass 2 as its input r = j >> 4, so pass 2's table holds
// exp(-2 pi i (k + 1/2) / 512) (put_row_phase builds these tables).
// ZMID: the sequence is zero outside registers [N/T/4, 3N/T/4), i.e. outside
// elements [N/4, 3N/4) (a masked column); the first pass then skips the
// butterflies with a zero input (its 16-point DFTs see elements [4, 12) only).
template <int N, int DIR, int PASS, bool HS = false, bool ZMID = false>
__device__ __forceinline__ void team_fft_reg_pass(float2 *v, float2 *ex, const float2 *tw, int Ns, int lane) {
    constexpr int T = fft_lanes(N);
    constexpr int NP = fft_npasses(N);
    constexpr int R = fft_radix(N, PASS);
    constexpr int NR = N / R;
    constexpr int IT = NR / T;                 // butterflies per lane in this pass
    static_assert(IT * R * T == N, "team layout");
    static_assert(!HS || (DIR > 0 && N / T == 16 && IT == 1 && (NP == 2 || N == 512)),
                  "half-sample shift: N = 128, 256 or 512");
    static_assert(!ZMID || (fft_radix(N, 0) == 16 && !HS), "zero outside the middle half: radix-16 first pass");
    if constexpr (PASS == 0) {
        // inputs from registers: element (lane + T*it) + NR*r = lane + T*(it + r*IT)
#pragma unroll
        for (int it = 0; it < IT; it++) {
            float2 u[R];
#pragma unroll
            for (int r = 0; r < R; r++) u[r] = v[it + r * IT];
            if constexpr (HS) {
#pragma unroll
                for (int r = 0; r < R; r++) {
                    const int k32 = r < 8 ? r : r + 16;          // m = r; the sign flip is +16/32 of a turn
                    const float c = cos32(k32) / (float)N, s = sin32(k32) / (float)N;
                    u[r] = make_float2(u[r].x * c - u[r].y * s, u[r].x * s + u[r].y * c);
                }
            }
            if constexpr (ZMID) dft16_mid<DIR>(u);
            else dft_reg<R, DIR>(u);
            const int j = lane + T * it;
#pragma unroll
            for (int r = 0; r < R; r++) ex[fft_pad(j * R + r)] = u[r];
        }
        __syncwarp();
        team_fft_reg_pass<N, DIR, 1>(v, ex, tw, R, lane);
    } else if constexpr (PASS < NP) {
        float2 u[IT][R];
#pragma unroll
        for (int it = 0; it < IT; it++) {
            const int j = lane + T * it;
            const int k = j & (Ns - 1);
#pragma unroll
            for (int r = 0; r < R; r++) u[it][r] = ex[fft_pad(j + r * NR)];
#pragma unroll
            for (int r = 1; r < R; r++) {
                const float2 w = tw[(r - 1) * Ns + k];
                u[it][r] = DIR < 0 ? cmulf(u[it][r], w) : cmulf_conj(u[it][r], w);
            }
        }
        if constexpr (PASS < NP - 1) __syncwarp();
#pragma unroll
        for (int it = 0; it < IT; it++) dft_reg<R, DIR>(u[it]);
        if constexpr (PASS == NP - 1) {
            // last pass: element j + Ns*r with j = lane + T*it and Ns = NR -> register it + r*IT
#pragma unroll
            for (int it = 0; it < IT; it++)
#pragma unroll
                for (int r = 0; r < R; r++) v[it + r * IT] = u[it][r];
            __syncwarp();     // the exchange buffer may be reused right after
        } else {
#pragma unroll
            for (int it = 0; it < IT; it++) {
                const int j = lane + T * it;
                const int k = j & (Ns - 1);
#pragma unroll
                for (int r = 0; r < R; r++) ex[fft_pad((j - k) * R + k + r * Ns)] = u[it][r];
            }
            __syncwarp();
            team_fft_reg_pass<N, DIR, PASS + 1>(v, ex, tw + (R - 1) * Ns, Ns * R, lane);
        }
    }
}

// In-register N-point FFT of the team's sequence v (N/T values per lane).
// ex: the team's exchange buffer, fft_padded_len(N) entries.  tw: the
// size-N pass twiddle table.  All lanes of the warp must call it.
template <int N, int DIR>
__device__ __forceinline__ void team_fft_reg(float2 *v, float2 *ex, const float2 *tw, int lane) {
    team_fft_reg_pass<N, DIR, 0>(v, ex, tw, 1, lane);
}

// The same for a sequence that is zero outside elements [N/4, 3N/4).
template <int N, int DIR>
__device__ __forceinline__ void team_fft_reg_mid(float2 *v, float2 *ex, const float2 *tw, int lane) {
    team_fft_reg_pass<N, DIR, 0, false, true>(v, ex, tw, 1, lane);
}

// Inverse FFT of X[f] * exp(i pi f' / N) / N (the odd samples of a 2x
// zero-pad interpolation) for N = 128, 256 or 512; twh: the tables put_row_phase builds.
template <int N>
__device__ __forceinline__ void team_ifft_half_shift(float2 *v, float2 *ex, const float2 *twh, int lane) {
    team_fft_reg_pass<N, +1, 0, true>(v, ex, twh, 1, lane);
}

}  // namespace xcg
