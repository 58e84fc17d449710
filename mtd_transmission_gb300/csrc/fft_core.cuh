// Shared-memory Stockham FFT building blocks for sm_103a.
//
// A CTA holds B transforms of N points each in shared memory (complex64,
// padded layout).  Each transform is worked by T = N/8 threads that each keep
// 8 points in registers per stage: radix-8 stages, then one radix-4 or
// radix-2 stage for sizes that are not a power of 8.  Stage s with span Ns
// reads point b + k*N/R, twiddles it by W_{Ns*R}^{(b mod Ns) k}, runs an R-point
// DFT and writes point (b/Ns)*Ns*R + (b mod Ns) + m*Ns (autosort: natural
// order in, natural order out, no bit reversal).
//
// Layout: logical point i of a transform lives at pad_idx(i) = i + i/16, one
// spare complex every 16, which spreads the stride-R stores of the early
// stages over all banks; transforms are tstride(N) (odd) complexes apart.
//
// Sign conventions follow FFTW: DIR = -1 is exp(-2 pi i jk/N) (forward),
// DIR = +1 is exp(+2 pi i jk/N) (backward); neither is normalised.
#pragma once

#include <cuda_runtime.h>
#include <cstdint>

namespace tdm {

constexpr int kTwN = 4096;  // twiddle table size: exp(-2 pi i k / 4096)

// Points per lane of the warp-resident FFT of size n (fft_warp.cuh).
__host__ __device__ constexpr int warp_fft_e(int n) { return n >= 2048 ? 64 : n >= 512 ? 32 : n >= 128 ? 16 : 8; }
// Offset of the per-lane twiddle factors of the n-point warp FFT in the
// device twiddle table (after the kTwN-entry table): one n-entry block per
// size 64, 128, ..., 2048.
__host__ __device__ constexpr int twr_offset(int n) { return kTwN + n - 64; }
constexpr int kTwTotal = kTwN + 4096 - 64;

__host__ __device__ constexpr int pad_idx(int i) { return i + (i >> 4); }
__host__ __device__ constexpr int padded_len(int n) { return n + (n >> 4); }
// Distance between consecutive transforms of a CTA in shared memory: odd, so
// that B transforms read at the same logical index fall in distinct banks.
__host__ __device__ constexpr int tstride(int n) { return padded_len(n) + 1; }
__host__ __device__ constexpr int ilog2c(int n) { return n <= 1 ? 0 : 1 + ilog2c(n >> 1); }

__device__ __forceinline__ float2 c_add(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 c_sub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ float2 c_mul(float2 a, float2 b) {
    return make_float2(fmaf(a.x, b.x, -a.y * b.y), fmaf(a.x, b.y, a.y * b.x));
}
__device__ __forceinline__ float2 c_scale(float2 a, float s) { return make_float2(a.x * s, a.y * s); }
__device__ __forceinline__ float2 c_conj(float2 a) { return make_float2(a.x, -a.y); }

// a * (DIR * i)
template <int DIR>
__device__ __forceinline__ float2 mul_dir_i(float2 a) {
    return DIR < 0 ? make_float2(a.y, -a.x) : make_float2(-a.y, a.x);
}

template <int DIR>
__device__ __forceinline__ void dft2(float2& a0, float2& a1) {
    float2 t = a0;
    a0 = c_add(t, a1);
    a1 = c_sub(t, a1);
}

template <int DIR>
__device__ __forceinline__ void dft4(float2& a0, float2& a1, float2& a2, float2& a3) {
    float2 t0 = c_add(a0, a2), t1 = c_sub(a0, a2);
    float2 t2 = c_add(a1, a3), t3 = mul_dir_i<DIR>(c_sub(a1, a3));
    a0 = c_add(t0, t2);
    a2 = c_sub(t0, t2);
    a1 = c_add(t1, t3);
    a3 = c_sub(t1, t3);
}

template <int DIR>
__device__ __forceinline__ void dft8(float2* x) {
    float2 e0 = x[0], e1 = x[2], e2 = x[4], e3 = x[6];
    float2 o0 = x[1], o1 = x[3], o2 = x[5], o3 = x[7];
    dft4<DIR>(e0, e1, e2, e3);
    dft4<DIR>(o0, o1, o2, o3);
    const float r = 0.70710678118654752440f;
    // o1 *= exp(DIR i pi/4), o2 *= DIR i, o3 *= exp(DIR 3 i pi/4)
    o1 = make_float2(r * (o1.x - DIR * o1.y), r * (DIR * o1.x + o1.y));
    o2 = mul_dir_i<DIR>(o2);
    o3 = make_float2(-r * (o3.x + DIR * o3.y), r * (DIR * o3.x - o3.y));
    x[0] = c_add(e0, o0);
    x[4] = c_sub(e0, o0);
    x[1] = c_add(e1, o1);
    x[5] = c_sub(e1, o1);
    x[2] = c_add(e2, o2);
    x[6] = c_sub(e2, o2);
    x[3] = c_add(e3, o3);
    x[7] = c_sub(e3, o3);
}

// One Stockham stage on a transform held in shared memory (in place).
// Every thread of the CTA must call it (it contains __syncthreads()); threads
// with active == false only take part in the barriers.
template <int N, int R, int NS, int DIR>
__device__ __forceinline__ void fft_stage(float2* s, int j, const float2* __restrict__ tw, bool active) {
    constexpr int T = N / 8;
    constexpr int NB = 8 / R;
    float2 x[8];
    if (active) {
#pragma unroll
        for (int t = 0; t < NB; ++t) {
            const int b = j + t * T;
#pragma unroll
            for (int k = 0; k < R; ++k) x[t * R + k] = s[pad_idx(b + k * (N / R))];
        }
    }
    __syncthreads();
    if (active) {
#pragma unroll
        for (int t = 0; t < NB; ++t) {
            const int b = j + t * T;
            const int p = b % NS;
            if constexpr (NS > 1) {
#pragma unroll
                for (int k = 1; k < R; ++k) {
                    float2 w = __ldg(&tw[p * k * (kTwN / (NS * R))]);
                    if constexpr (DIR > 0) w.y = -w.y;
                    x[t * R + k] = c_mul(x[t * R + k], w);
                }
            }
            if constexpr (R == 8) dft8<DIR>(&x[t * R]);
            else if constexpr (R == 4) dft4<DIR>(x[t * R], x[t * R + 1], x[t * R + 2], x[t * R + 3]);
            else dft2<DIR>(x[t * R], x[t * R + 1]);
            const int base = (b / NS) * NS * R + p;
#pragma unroll
            for (int m = 0; m < R; ++m) s[pad_idx(base + m * NS)] = x[t * R + m];
        }
    }
    __syncthreads();
}

// Full N-point transform of the padded shared-memory array s, worked by
// thread j in [0, N/8) of the transform.  Input and output in natural order.
template <int N, int DIR>
__device__ __forceinline__ void fft_smem(float2* s, int j, const float2* __restrict__ tw, bool active = true) {
    static_assert(N >= 64 && N <= kTwN && (N & (N - 1)) == 0, "power-of-two size in [64, 4096]");
    constexpr int L2 = ilog2c(N);
    constexpr int n8 = L2 / 3;
    constexpr int rem = L2 % 3;
    fft_stage<N, 8, 1, DIR>(s, j, tw, active);
    fft_stage<N, 8, 8, DIR>(s, j, tw, active);
    if constexpr (n8 >= 3) fft_stage<N, 8, 64, DIR>(s, j, tw, active);
    if constexpr (n8 >= 4) fft_stage<N, 8, 512, DIR>(s, j, tw, active);
    constexpr int NSf = 1 << (3 * n8);
    if constexpr (rem == 1) fft_stage<N, 2, NSf, DIR>(s, j, tw, active);
    if constexpr (rem == 2) fft_stage<N, 4, NSf, DIR>(s, j, tw, active);
}

}  // namespace tdm
