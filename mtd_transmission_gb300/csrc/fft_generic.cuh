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
// radices are the factors of N: 10 while 10 divides what is left (a
// 2 x 5 DFT in registers, one shared-memory round trip where radices 2 and
// 5 took two), then 4, 2, 3, 5 and 7.  So 250 points take three passes
// (10, 5, 5) and 500 points three (10, 10, 5).
//
// Twiddles come from a table of exp(-2 pi i k / Q) (k < Q) for a Q that N
// divides (the context keeps Q = 4F, which serves the F- and 2F-point
// transforms and the quarter-sample factors of the Volkov passes).  A pass
// reads W^1 of its butterfly from the table and forms W^k, k > 1, as
// W^(k/2) W^(k - k/2): the L1/shared pipe, which these passes saturate, serves
// one table read where it served R - 1.  Sign
// conventions follow FFTW: DIR = -1 is exp(-2 pi i jk/N), DIR = +1 is
// exp(+2 pi i jk/N); neither is normalised.
#pragma once

#include <utility>

#include "fft_core.cuh"

namespace tdm {

// The radix of the next pass for m points still to factor.
__host__ __device__ constexpr int gfft_radix(int m) {
    return m % 10 == 0 ? 10 : m % 4 == 0 ? 4 : m % 2 == 0 ? 2 : m % 3 == 0 ? 3 : m % 5 == 0 ? 5 : m % 7 == 0 ? 7 : m;
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
        if (r > 7 && r != 10) return false;
        n /= r;
    }
    return true;
}

// cos and sin of 2 pi e / r at compile time (Taylor series in double on the
// angle reduced to [-pi, pi]), for the fixed twiddles inside composite radices.
__host__ __device__ constexpr double ct_angle(int e, int r) {
    const double pi = 3.14159265358979323846;
    const double t = 2.0 * pi * (double)(e % r) / (double)r;
    return t > pi ? t - 2.0 * pi : t;
}
__host__ __device__ constexpr double ct_sin(double x) {
    double term = x, sum = x;
    for (int n = 1; n < 24; ++n) {
        term *= -x * x / ((2.0 * n) * (2.0 * n + 1.0));
        sum += term;
    }
    return sum;
}
__host__ __device__ constexpr double ct_cos(double x) {
    double term = 1.0, sum = 1.0;
    for (int n = 1; n < 24; ++n) {
        term *= -x * x / ((2.0 * n - 1.0) * (2.0 * n));
        sum += term;
    }
    return sum;
}
// W_R^E in direction DIR: exp(DIR 2 pi i E / R)
template <int E, int R, int DIR>
__device__ __forceinline__ float2 ct_root() {
    constexpr float c = (float)ct_cos(ct_angle(E, R)), s = (float)ct_sin(ct_angle(E, R));
    return make_float2(c, DIR < 0 ? -s : s);
}

// f(integral_constant<int, 0>), ..., f(integral_constant<int, N - 1>)
template <class Fn, int... I>
__device__ __forceinline__ void static_for_seq(Fn&& f, std::integer_sequence<int, I...>) {
    (f(std::integral_constant<int, I>{}), ...);
}
template <int N, class Fn>
__device__ __forceinline__ void static_for(Fn&& f) {
    static_for_seq(f, std::make_integer_sequence<int, N>{});
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

// R1 R2-point DFT in registers (R1, R2 prime-radix sizes): with
// k = R2 k1 + k2 and m = m1 + R1 m2,
//     X[m1 + R1 m2] = sum_k2 W_R2^(k2 m2) W_R^(k2 m1) sum_k1 W_R1^(k1 m1) x[R2 k1 + k2],
// R1-point DFTs over k1, fixed twiddles W_R^(k2 m1), R2-point DFTs over k2.
template <int R1, int R2, int DIR, int Q>
__device__ __forceinline__ void dft_composite(float2* x, const float2* __restrict__ w);

template <int R, int DIR, int Q>
__device__ __forceinline__ void gdft(float2* x, const float2* __restrict__ w) {
    if constexpr (R == 2) dft2<DIR>(x[0], x[1]);
    else if constexpr (R == 3) dft3<DIR>(x);
    else if constexpr (R == 4) dft4<DIR>(x[0], x[1], x[2], x[3]);
    else if constexpr (R == 5) dft5<DIR>(x);
    else if constexpr (R == 10) dft_composite<2, 5, DIR, Q>(x, w);
    else dft_table<R, DIR, Q>(x, w);
}

template <int R1, int R2, int DIR, int Q>
__device__ __forceinline__ void dft_composite(float2* x, const float2* __restrict__ w) {
    constexpr int R = R1 * R2;
    float2 y[R];  // y[m1 R2 + k2]
    static_for<R2>([&](auto k2c) {
        constexpr int k2 = decltype(k2c)::value;
        float2 v[R1];
#pragma unroll
        for (int k1 = 0; k1 < R1; ++k1) v[k1] = x[R2 * k1 + k2];
        gdft<R1, DIR, Q>(v, w);
        static_for<R1>([&](auto m1c) {
            constexpr int m1 = decltype(m1c)::value;
            if constexpr ((k2 * m1) % R == 0) y[m1 * R2 + k2] = v[m1];
            else y[m1 * R2 + k2] = c_mul(v[m1], ct_root<(k2 * m1) % R, R, DIR>());
        });
    });
#pragma unroll
    for (int m1 = 0; m1 < R1; ++m1) {
        gdft<R2, DIR, Q>(y + m1 * R2, w);
#pragma unroll
        for (int m2 = 0; m2 < R2; ++m2) x[m1 + R1 * m2] = y[m1 * R2 + m2];
    }
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
            float2 t[R];
            t[1] = __ldg(&w[p * (Q / (S * R))]);
            if constexpr (DIR > 0) t[1].y = -t[1].y;
#pragma unroll
            for (int k = 2; k < R; ++k) t[k] = c_mul(t[k >> 1], t[k - (k >> 1)]);
#pragma unroll
            for (int k = 1; k < R; ++k) x[k] = c_mul(x[k], t[k]);
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
