// Warp-resident FFT for sm_103a.
//
// An N-point transform is held by T = N/E lanes of one warp, E points per
// lane, so a warp carries G = 32/T transforms side by side.  With
// n = j + T n1 (lane j, register n1) and k = k1 + E k2:
//
//     X[k1 + E k2] = sum_n2 W_T^(n2 k2) [ W_N^(n2 k1) sum_n1 x[n2 + T n1] W_E^(n1 k1) ]
//
// so each lane runs an E-point DFT on its own registers, multiplies by
// W_N^(j k1), the lanes exchange through shared memory (one write, one read,
// __syncwarp only), and each lane finishes with E/T DFTs of T points.  Lane j
// ends holding X[(j + q T) + E k2] in register q T + k2.  Input and output are
// therefore "lane-minor": consecutive lanes hold consecutive elements, which
// makes the global loads and stores around the transform coalesced.
//
// The exchange uses the transform's own shared-memory array, padded with one
// spare slot every T elements (pad(i) = i + i/T).  Both exchange patterns,
// and the natural-order loads and stores, then touch distinct banks for
// T >= 16; for T = 8 two transforms share a half-warp and may meet 2-way
// conflicts in the exchange.
//
// The register DFTs are split-radix-free Cooley-Tukey codelets (2, 4, 8, and
// 16 = 4 x 4, 32 = 8 x 4, 64 = 8 x 8) with compile-time twiddles; the
// inter-lane twiddles W_N^(j k1) come from a [k1][j] table (twr_offset) so
// that a warp's loads are contiguous.  Sign conventions follow FFTW: DIR = -1
// is exp(-2 pi i jk/N), DIR = +1 is exp(+2 pi i jk/N); neither is normalised.
#pragma once

#include <type_traits>

#include "fft_core.cuh"

namespace tdm {

// cos(pi a / 16), exact to double precision for every integer a.
constexpr double cospi16(int a) {
    const double t[9] = {1.0,
                         0.98078528040323044912618223613424,
                         0.92387953251128675612818318939679,
                         0.83146961230254523707878837761791,
                         0.70710678118654752440084436210485,
                         0.55557023301960222474283081394853,
                         0.38268343236508977172845998403040,
                         0.19509032201612826784828486847702,
                         0.0};
    a = ((a % 32) + 32) % 32;
    if (a > 16) a = 32 - a;
    return a > 8 ? -t[16 - a] : t[a];
}
constexpr double sinpi16(int a) { return cospi16(8 - a); }

template <int I, int End, class Fn>
__device__ __forceinline__ void static_for(Fn&& fn) {
    if constexpr (I < End) {
        fn(std::integral_constant<int, I>{});
        static_for<I + 1, End>(fn);
    }
}

// v * exp(DIR 2 pi i M / R), R dividing 32 (64: M even or handled by the 8 x 8 split's own table)
template <int R, int M, int DIR>
__device__ __forceinline__ float2 twc(float2 v) {
    static_assert(32 % R == 0 || R == 64, "codelet size");
    if constexpr (R == 64) {
        // angle 2 pi M / 64 = pi M / 32: halve through the pi/16 table when M is even,
        // otherwise use the half-angle values
        if constexpr (M % 2 == 0) {
            return twc<32, M / 2, DIR>(v);
        } else {
            constexpr double c64[17] = {1.0,
                                        0.99518472667219688624483695310948,
                                        0.98078528040323044912618223613424,
                                        0.95694033573220886493579788698027,
                                        0.92387953251128675612818318939679,
                                        0.88192126434835502971275686366039,
                                        0.83146961230254523707878837761791,
                                        0.77301045336273696081090660975847,
                                        0.70710678118654752440084436210485,
                                        0.63439328416364549821517161322549,
                                        0.55557023301960222474283081394853,
                                        0.47139673682599764855638762590525,
                                        0.38268343236508977172845998403040,
                                        0.29028467725446236763619237581740,
                                        0.19509032201612826784828486847702,
                                        0.09801714032956060199419556388864,
                                        0.0};
            // cos(pi m / 32) for m in [0, 64)
            constexpr int m = M % 64;
            constexpr int r = m > 32 ? 64 - m : m;          // cos symmetric about pi
            constexpr double cs = r > 16 ? -c64[32 - r] : c64[r];
            constexpr int ms = ((16 - m) % 64 + 64) % 64;   // sin(x) = cos(pi/2 - x)
            constexpr int rs = ms > 32 ? 64 - ms : ms;
            constexpr double sn = rs > 16 ? -c64[32 - rs] : c64[rs];
            constexpr float c = (float)cs, s = (float)(DIR * sn);
            return make_float2(fmaf(c, v.x, -s * v.y), fmaf(c, v.y, s * v.x));
        }
    } else {
        constexpr int a = ((32 / R) * M) % 32;
        if constexpr (a == 0) {
            return v;
        } else if constexpr (a == 8) {
            return mul_dir_i<DIR>(v);
        } else if constexpr (a == 16) {
            return make_float2(-v.x, -v.y);
        } else if constexpr (a == 24) {
            return mul_dir_i<-DIR>(v);
        } else if constexpr (a % 4 == 0) {  // odd multiples of pi/4: |cos| = |sin| = 1/sqrt 2
            constexpr float c = (float)cospi16(a), s = (float)(DIR * sinpi16(a));
            return c == s ? make_float2(c * (v.x - v.y), c * (v.y + v.x))
                          : make_float2(c * (v.x + v.y), c * (v.y - v.x));
        } else {
            constexpr float c = (float)cospi16(a), s = (float)(DIR * sinpi16(a));
            return make_float2(fmaf(c, v.x, -s * v.y), fmaf(c, v.y, s * v.x));
        }
    }
}

template <int R, int DIR>
__device__ __forceinline__ void dft(float2* x);

// R = N1 N2: N2 DFTs of N1 points on the stride-N2 subsequences, twiddles
// W_R^(n2 k1), N1 DFTs of N2 points; X[k1 + N1 k2].
template <int N1, int N2, int DIR>
__device__ __forceinline__ void dft_split(float2* x) {
    constexpr int R = N1 * N2;
    float2 y[R];
    static_for<0, N2>([&](auto n2c) {
        constexpr int n2 = decltype(n2c)::value;
        float2 t[N1];
#pragma unroll
        for (int n1 = 0; n1 < N1; ++n1) t[n1] = x[N2 * n1 + n2];
        dft<N1, DIR>(t);
        static_for<0, N1>([&](auto k1c) {
            constexpr int k1 = decltype(k1c)::value;
            y[n2 * N1 + k1] = twc<R, n2 * k1, DIR>(t[k1]);
        });
    });
#pragma unroll
    for (int k1 = 0; k1 < N1; ++k1) {
        float2 t[N2];
#pragma unroll
        for (int n2 = 0; n2 < N2; ++n2) t[n2] = y[n2 * N1 + k1];
        dft<N2, DIR>(t);
#pragma unroll
        for (int k2 = 0; k2 < N2; ++k2) x[k1 + N1 * k2] = t[k2];
    }
}

template <int R, int DIR>
__device__ __forceinline__ void dft(float2* x) {
    if constexpr (R == 2) dft2<DIR>(x[0], x[1]);
    else if constexpr (R == 4) dft4<DIR>(x[0], x[1], x[2], x[3]);
    else if constexpr (R == 8) dft8<DIR>(x);
    else if constexpr (R == 16) dft_split<4, 4, DIR>(x);
    else if constexpr (R == 32) dft_split<8, 4, DIR>(x);
    else if constexpr (R == 64) dft_split<8, 8, DIR>(x);
    else static_assert(R == 2, "unsupported codelet size");
}

template <int N>
struct WarpFFT {
    static_assert(N >= 64 && N <= 2048 && (N & (N - 1)) == 0, "power-of-two size in [64, 2048]");
    static constexpr int E = warp_fft_e(N);  // points per lane
    static constexpr int T = N / E;          // lanes per transform
    static constexpr int G = 32 / T;         // transforms per warp
    static constexpr int LOG_T = ilog2c(T);
    static constexpr int LEN = N + E;        // padded length
    // Distance between transforms in shared memory: odd, so that a CTA-wide
    // pass reading the same logical index of consecutive transforms (a
    // transposing load or store) touches distinct banks.
    static constexpr int STRIDE = LEN + 1;
    __host__ __device__ static constexpr int pad(int i) { return i + (i >> LOG_T); }
};

// x[k1] *= W_N^(DIR j k1), k1 = 1 .. E-1, from the [k1][j] table.  For
// E >= 16 only the factors of k1 = b (b < 8) and k1 = 8a are loaded and
// W^(j (8a + b)) = W^(8ja) W^(jb) is formed in registers: 7 + E/8 - 1 loads
// instead of E - 1 (the loads' L1 latency, not their arithmetic, bounded the
// FFT passes), at about one extra rounding per factor.
template <int N, int DIR>
__device__ __forceinline__ void twiddle_lane(float2 (&x)[WarpFFT<N>::E], const float2* __restrict__ twr, int j) {
    using W = WarpFFT<N>;
    constexpr int E = W::E, T = W::T;
    constexpr int R = E >= 16 ? 8 : E;  // k1 = R a + b
    float2 wb[R];
#pragma unroll
    for (int b = 1; b < R; ++b) {
        wb[b] = __ldg(&twr[b * T + j]);
        if constexpr (DIR > 0) wb[b].y = -wb[b].y;
        x[b] = c_mul(x[b], wb[b]);
    }
#pragma unroll
    for (int a = 1; a < E / R; ++a) {
        float2 wa = __ldg(&twr[R * a * T + j]);
        if constexpr (DIR > 0) wa.y = -wa.y;
        x[R * a] = c_mul(x[R * a], wa);
#pragma unroll
        for (int b = 1; b < R; ++b) x[R * a + b] = c_mul(x[R * a + b], c_mul(wa, wb[b]));
    }
}

// Register form.  On entry x[n1] holds element j + T n1 of the transform; on
// return x[q T + k2] holds element (j + q T) + E k2.  s is the transform's
// padded shared-memory array (WarpFFT<N>::LEN slots), used for the exchange.
// Every lane of the warp must call it together.
template <int N, int DIR>
__device__ __forceinline__ void fft_warp_regs(float2 (&x)[WarpFFT<N>::E], float2* s, int j,
                                              const float2* __restrict__ tw) {
    using W = WarpFFT<N>;
    constexpr int E = W::E, T = W::T;
    const float2* twr = tw + twr_offset(N);
    dft<E, DIR>(x);
    twiddle_lane<N, DIR>(x, twr, j);
    __syncwarp();  // earlier readers of s are done
#pragma unroll
    for (int k1 = 0; k1 < E; ++k1) s[k1 * (T + 1) + j] = x[k1];  // pad(k1 T + j)
    __syncwarp();
#pragma unroll
    for (int q = 0; q < E / T; ++q) {
#pragma unroll
        for (int n2 = 0; n2 < T; ++n2) x[q * T + n2] = s[(j + q * T) * (T + 1) + n2];  // pad((j + qT) T + n2)
    }
#pragma unroll
    for (int q = 0; q < E / T; ++q) dft<T, DIR>(&x[q * T]);
}

// fft_warp_regs with a smaller exchange buffer: the E/T output blocks are
// exchanged one at a time (block q reads the rows k1 in [qT, qT + T), which
// come from the same registers x[qT .. qT + T) of every lane), so s needs
// T (T + 1) slots instead of N + E (WarpFFT<N>::LEN).  Same values, in the
// same registers, as fft_warp_regs; one more __syncwarp pair per block.
template <int N, int DIR>
__device__ __forceinline__ void fft_warp_regs_lean(float2 (&x)[WarpFFT<N>::E], float2* s, int j,
                                                   const float2* __restrict__ tw) {
    using W = WarpFFT<N>;
    constexpr int E = W::E, T = W::T;
    const float2* twr = tw + twr_offset(N);
    dft<E, DIR>(x);
    twiddle_lane<N, DIR>(x, twr, j);
#pragma unroll
    for (int q = 0; q < E / T; ++q) {
        __syncwarp();  // earlier readers of s are done
#pragma unroll
        for (int kk = 0; kk < T; ++kk) s[kk * (T + 1) + j] = x[q * T + kk];
        __syncwarp();
#pragma unroll
        for (int n2 = 0; n2 < T; ++n2) x[q * T + n2] = s[j * (T + 1) + n2];
    }
#pragma unroll
    for (int q = 0; q < E / T; ++q) dft<T, DIR>(&x[q * T]);
}

// The same transform run from the other end: on entry x[q T + k2] holds
// element (j + q T) + E k2 (the order fft_warp_regs produces); on return x[n1]
// holds element j + T n1 of its DIR transform.  With k = k1 + E k2 and
// n = j' + T n1,
//     y[j' + T n1] = sum_k1 W_E^(n1 k1) W_N^(j' k1) [ sum_k2 W_T^(j' k2) Y[k1 + E k2] ]
// (all exponents with sign DIR): T-point DFTs first, the transposing
// exchange, the twiddles, then the E-point DFT.  A forward transform, a
// pointwise product in frequency and this inverse therefore never leave
// registers except for the two exchanges.
template <int N, int DIR>
__device__ __forceinline__ void fft_warp_regs_rev(float2 (&x)[WarpFFT<N>::E], float2* s, int j,
                                                  const float2* __restrict__ tw) {
    using W = WarpFFT<N>;
    constexpr int E = W::E, T = W::T;
    const float2* twr = tw + twr_offset(N);
#pragma unroll
    for (int q = 0; q < E / T; ++q) dft<T, DIR>(&x[q * T]);
    __syncwarp();  // earlier readers of s are done
#pragma unroll
    for (int q = 0; q < E / T; ++q) {
#pragma unroll
        for (int n2 = 0; n2 < T; ++n2) s[(j + q * T) * (T + 1) + n2] = x[q * T + n2];
    }
    __syncwarp();
#pragma unroll
    for (int k1 = 0; k1 < E; ++k1) x[k1] = s[k1 * (T + 1) + j];
    twiddle_lane<N, DIR>(x, twr, j);
    dft<E, DIR>(x);
}

// Forward transform with sign DIR, x[k] *= mul(k, x[k]) for every bin k, and
// the unnormalised transform with sign -DIR; x in the input order of
// fft_warp_regs on entry and on return.
template <int N, int DIR, class Mul>
__device__ __forceinline__ void fft_warp_filter(float2 (&x)[WarpFFT<N>::E], float2* s, int j,
                                                const float2* __restrict__ tw, Mul&& mul) {
    using W = WarpFFT<N>;
    constexpr int E = W::E, T = W::T;
    fft_warp_regs<N, DIR>(x, s, j, tw);
#pragma unroll
    for (int q = 0; q < E / T; ++q) {
#pragma unroll
        for (int k2 = 0; k2 < T; ++k2) x[q * T + k2] = mul(j + q * T + E * k2, x[q * T + k2]);
    }
    fft_warp_regs_rev<N, -DIR>(x, s, j, tw);
}

// Position in the padded array of element (j + q T) + E k2, the element held
// in register q T + k2 after fft_warp_regs.
template <int N>
__device__ __forceinline__ int warp_out_pos(int j, int q, int k2) {
    using W = WarpFFT<N>;
    return j + q * W::T + W::E * k2 + q + (W::E / W::T) * k2;
}

// Shared-memory form: transforms the padded array s in place (natural order
// in and out).  The caller orders other threads' accesses to s around it.
template <int N, int DIR>
__device__ __forceinline__ void fft_warp(float2* s, int j, const float2* __restrict__ tw) {
    using W = WarpFFT<N>;
    constexpr int E = W::E, T = W::T;
    float2 x[E];
#pragma unroll
    for (int n1 = 0; n1 < E; ++n1) x[n1] = s[j + n1 * (T + 1)];  // pad(j + T n1)
    fft_warp_regs<N, DIR>(x, s, j, tw);
    __syncwarp();
#pragma unroll
    for (int q = 0; q < E / T; ++q) {
#pragma unroll
        for (int k2 = 0; k2 < T; ++k2) s[warp_out_pos<N>(j, q, k2)] = x[q * T + k2];
    }
}

// Out-of-line copy of fft_warp: one body per (N, DIR) however many call
// sites a kernel has, which bounds the code size and the register count of
// kernels that chain several transforms.
template <int N, int DIR>
__device__ __noinline__ void fft_warp_call(float2* s, int j, const float2* __restrict__ tw) {
    fft_warp<N, DIR>(s, j, tw);
}

// Shared-memory filter on the out-of-line transforms: s (natural order) is
// replaced by FFT_{-DIR}(mul(k, FFT_DIR(s)[k])), unnormalised.
template <int N, int DIR, class Mul>
__device__ __forceinline__ void fft_warp_filter_call(float2* s, int j, const float2* __restrict__ tw, Mul&& mul) {
    using W = WarpFFT<N>;
    constexpr int E = W::E, T = W::T;
    fft_warp_call<N, DIR>(s, j, tw);
    __syncwarp();
#pragma unroll 8
    for (int n1 = 0; n1 < E; ++n1) {
        float2* p = &s[j + n1 * (T + 1)];  // pad(j + T n1)
        *p = mul(j + n1 * T, *p);
    }
    __syncwarp();
    fft_warp_call<N, -DIR>(s, j, tw);
}

}  // namespace tdm
