// Mixed-radix FFT for sizes that are not powers of two (sm_103a).
//
// The reference takes any NXMAX; its own configuration has NXMAX 125, so the
// fields are 250 x 250 and the Volkov mirror 500 x 500.  The warp-resident
// engine (fft_warp.cuh) needs N = T E with T lanes dividing the warp; these
// sizes do not factor that way, so they run on this engine: one warp per
// transform, the N points in shared memory, a Stockham autosort pass per
// radix (natural order in and out, two buffers used alternately,
// __syncwarp() between passes).  A pass of radix R and span S reads points
// b + k N/R (b < N/R, k < R), multiplies them by W_(S R)^((b mod S) k), runs
// an R-point DFT and writes point (b / S) S R + (b mod S) + m S.  The
// radices are the factors of N, 4 first, then 2, 3, 5 and 7.
//
// Twiddles come from a table of exp(-2 pi i k / Q) (k < Q) for a Q that N
// divides (the context keeps Q = 4F, which serves the F- and 2F-point
// transforms and the quarter-sample factors of the Volkov passes).  Sign
// conventions follow FFTW: DIR = -1 is exp(-2 pi i jk/N), DIR = +1 is
// exp(+2 pi i jk/N); neither is normalised.
#pragma once

#include "fft_core.cuh"

namespace tdm {

// The radix of the next pass for m points still to factor.
__host__ __device__ constexpr int gfft_radix(int m) {
    return m % 4 == 0 ? 4 : m % 2 == 0 ? 2 : m % 3 == 0 ? 3 : m % 5 == 0 ? 5 : m % 7 == 0 ? 7 : m;
}
__host__ __device__ constexpr int gfft_npasses(int n) {
    int k = 0;
    while (n > 1) {
        n /= gfft_radix(n);
        ++k;
    }
    return k;
}
// Whether N factors into the supported radices.
__host__ __device__ constexpr bool gfft_supported(int n) {
    while (n > 1) {
        const int r = gfft_radix(n);
        if (r > 7) return false;
        n /= r;
    }
    return true;
}

template <int DIR>
__device__ __forceinline__ void dft3(float2* x) {
    constexpr float h = 0.86602540378443864676f;  // sin(2 pi/3)
    const float2 s = c_add(x[1], x[2]), d = c_sub(x[1], x[2]);
    const float2 m = make_float2(x[0].x - 0.5f * s.x, x[0].y - 0.5f * s.y);
    const float2 t = mul_dir_i<DIR>(c_scale(d, h));
    x[0] = c_add(x[0], s);
    x[1] = c_add(m, t);
    x[2] = c_sub(m, t);
}

template <int DIR>
__device__ __forceinline__ void dft5(float2* x) {
    constexpr float c1 = 0.30901699437494742410f, c2 = -0.80901699437494742410f;  // cos(2 pi/5), cos(4 pi/5)
    constexpr float s1 = 0.95105651629515357212f, s2 = 0.58778525229247312917f;   // sin(2 pi/5), sin(4 pi/5)
    const float2 t1 = c_add(x[1], x[4]), t2 = c_add(x[2], x[3]);
    const float2 t3 = c_sub(x[1], x[4]), t4 = c_sub(x[2], x[3]);
    const float2 a1 = make_float2(x[0].x + c1 * t1.x + c2 * t2.x, x[0].y + c1 * t1.y + c2 * t2.y);
    const float2 a2 = make_float2(x[0].x + c2 * t1.x + c1 * t2.x, x[0].y + c2 * t1.y + c1 * t2.y);
    const float2 b1 = mul_dir_i<DIR>(make_float2(s1 * t3.x + s2 * t4.x, s1 * t3.y + s2 * t4.y));
    const float2 b2 = mul_dir_i<DIR>(make_float2(s2 * t3.x - s1 * t4.x, s2 * t3.y - s1 * t4.y));
    x[0] = c_add(x[0], c_add(t1, t2));
    x[1] = c_add(a1, b1);
    x[4] = c_sub(a1, b1);
    x[2] = c_add(a2, b2);
    x[3] = c_sub(a2, b2);
}

// R-point DFT by definition with twiddles from the table (radix 7).
template <int R, int DIR, int Q>
__device__ __forceinline__ void dft_table(float2* x, const float2* __restrict__ w) {
    float2 y[R];
#pragma unroll
    for (int m = 0; m < R; ++m) {
        float2 acc = x[0];
#pragma unroll
        for (int k = 1; k < R; ++k) {
            float2 t = __ldg(&w[((k * m) % R) * (Q / R)]);
            if constexpr (DIR > 0) t.y = -t.y;
            acc = c_add(acc, c_mul(x[k], t));
        }
        y[m] = acc;
    }
#pragma unroll
    for (int m = 0; m < R; ++m) x[m] = y[m];
}

template <int R, int DIR, int Q>
__device__ __forceinline__ void gdft(float2* x, const float2* __restrict__ w) {
    if constexpr (R == 2) dft2<DIR>(x[0], x[1]);
    else if constexpr (R == 3) dft3<DIR>(x);
    else if constexpr (R == 4) dft4<DIR>(x[0], x[1], x[2], x[3]);
    else if constexpr (R == 5) dft5<DIR>(x);
    else dft_table<R, DIR, Q>(x, w);
}

// One Stockham pass (radix R, span S) of an N-point transform, in -> out.
template <int N, int R, int S, int DIR, int Q>
__device__ __forceinline__ void gfft_pass(const float2* in, float2* out, const float2* __restrict__ w, int lane) {
    constexpr int NB = N / R;
#pragma unroll 2
    for (int b = lane; b < NB; b += 32) {
        const int p = b % S;
        float2 x[R];
#pragma unroll
        for (int k = 0; k < R; ++k) x[k] = in[b + k * NB];
        if constexpr (S > 1) {
#pragma unroll
            for (int k = 1; k < R; ++k) {
                float2 t = __ldg(&w[p * k * (Q / (S * R))]);
                if constexpr (DIR > 0) t.y = -t.y;
                x[k] = c_mul(x[k], t);
            }
        }
        gdft<R, DIR, Q>(x, w);
        const int base = (b / S) * S * R + p;
#pragma unroll
        for (int m = 0; m < R; ++m) out[base + m * S] = x[m];
    }
}

template <int N, int S, int DIR, int Q>
__device__ __forceinline__ void gfft_passes(float2*& a, float2*& b, const float2* __restrict__ w, int lane) {
    if constexpr (S < N) {
        constexpr int R = gfft_radix(N / S);
        gfft_pass<N, R, S, DIR, Q>(a, b, w, lane);
        __syncwarp();
        float2* t = a;
        a = b;
        b = t;
        gfft_passes<N, S * R, DIR, Q>(a, b, w, lane);
    }
}

// N-point transform of the warp's sequence in a, in place (natural order in
// and out); b is a second buffer of N points, overwritten.  Every lane of the
// warp must call it; the caller orders other accesses to a and b around it
// (a __syncwarp() before, when other lanes wrote a).  Ends with __syncwarp().
template <int N, int DIR, int Q>
__device__ __forceinline__ void gfft(float2* a, float2* b, const float2* __restrict__ w, int lane) {
    static_assert(gfft_supported(N) && Q % N == 0, "size");
    float2* x = a;
    float2* y = b;
    gfft_passes<N, 1, DIR, Q>(x, y, w, lane);
    if constexpr (gfft_npasses(N) & 1) {  // the result is in b
        for (int i = lane; i < N; i += 32) a[i] = x[i];
        __syncwarp();
    }
}

}  // namespace tdm
