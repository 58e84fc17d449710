// Field formation: second loop of tomo_pretraitement
// (pretraitement_hors_axe_CPU/main.cpp:230-342) on chunks of angles.
//
//  argmax     coordSpec (fonctions.cpp:88-101), |z|^2 at index 0, |z| elsewhere,
//             first maximum wins.
//  field      calc_Uborn2 (fonctions.cpp:348-374): shift by -posSpec, unnormalised
//             inverse FFT, shift by (N, N) -- index remaps on load and store.
//  volkov     deroul_volkov4_total_sym_paire (src/deroulement_volkov4.cpp:14-92) on
//             the 2F x 2F even mirror.  A 2D spectral derivative along x is the
//             1D spectral derivative of each row (kappa depends on kx only), so
//             gradient_fft4 becomes a row pass and a column pass, each computed
//             from F-point transforms (the mirror's spectrum is a DCT of the row,
//             its derivative a DST: mirror_derivative).  The wrapped phase's own
//             gradient, which the reference subtracts from the phasor's before the
//             Poisson solve and whose solve it adds back, returns the phase less
//             its mean (the solve inverts the spectral gradient exactly, the mean
//             being the zero-frequency term it sets to 0), so the passes solve
//             for the phasor's gradient alone and add the mean of the wrapped
//             phase.  integ_grad4's Poisson
//             solve on the mirror is a DCT-II / DST-II of the quadrant's gx and
//             gy, a division by |kappa|^2 and an inverse DCT (DCT-III) back to
//             the quadrant, all from F-point transforms (k_volkov_integ_rows).
//             Literal kappa: the mirror's Nyquist bin of the derivatives is
//             zero, and the Nyquist row and column of the Poisson solve cancel
//             in the real part kept on the quadrant, so the -1/2 factor does
//             not enter; literal Re() projections, zero-frequency term 0.
//  fit/form   aberCorr2 / ampliCorr2 (Correction_aberration.cpp:166-217) and the
//             Born/Rytov formation (main.cpp:289-316).  The least-squares
//             projection onto degree-4 polynomials is computed in a basis that is
//             orthonormal over the sample points (same projection as the
//             reference's normal equations, better conditioned).
#include "tdm_internal.cuh"
#include "fft_warp.cuh"
#include "form.cuh"
#include "argmax.cuh"
#include "phase_mean.cuh"

namespace tdm {
namespace {

constexpr float kTwoPi = 6.283185307179586f;
constexpr float kInvTwoPi = 0.15915494309189535f;

template <class K>
cudaError_t allow_smem(K kernel, size_t bytes) {
    return max_dynamic_smem(reinterpret_cast<const void*>(kernel), bytes);
}


// ---------------------------------------------------------------- argmax
// coordSpec (fonctions.cpp:88-101) in two steps: partial winners over slices
// of each spectrum (k_argmax_part here, or the extraction column pass when
// the spectra come straight from the holograms), then argmax_final in
// k_field_rows, the first consumer.
__global__ void __launch_bounds__(256) k_argmax_part(const float2* __restrict__ spectra, int F,
                                                     float4* __restrict__ part) {
    const int a = blockIdx.y, sl = blockIdx.x;
    const int per = (F * F + kArgSlices - 1) / kArgSlices, i0 = sl * per, i1 = min(i0 + per, F * F);
    const float2* s = spectra + (size_t)a * F * F;
    float best = -1.0f, second = -1.0f;
    int bi = 0x7fffffff;
    for (int i = i0 + threadIdx.x; i < i1; i += blockDim.x) argmax_take(best, bi, second, s[i], i);
    argmax_block(best, bi, second);
    if (threadIdx.x == 0) part[(size_t)a * kArgSlices + sl] = argmax_record(best, bi, second);
}

// ---------------------------------------------------------------- field = shift(IFFT(shift(S)))
// All FFT passes below run on the warp-resident FFT (fft_warp.cuh).  A row
// pass loads and stores its lanes' elements directly (lane-minor order is
// contiguous along a row); a column pass stages B columns in shared memory
// with CTA-wide coalesced loads and stores around the transforms.
template <int F>
struct FieldCfg {
    using W = WarpFFT<F>;
    static constexpr int B = 8 * W::G;       // transforms per CTA
    static constexpr int NT = B * W::T;      // 256 threads
    static constexpr size_t SMEM = (size_t)B * W::STRIDE * sizeof(float2);
};

template <int F>
__global__ void __launch_bounds__(FieldCfg<F>::NT)
k_field_rows(const float2* __restrict__ spectra, const float4* __restrict__ argpart, int nparts,
             int2* __restrict__ posspec, float2* __restrict__ specval, int normalize, const float2* __restrict__ tw,
             float2* __restrict__ I1) {
    using C = FieldCfg<F>;
    using W = typename C::W;
    constexpr int T = W::T, E = W::E;
    extern __shared__ float2 sm[];
    const int tr = threadIdx.x / T, j = threadIdx.x % T;
    const int a = blockIdx.y, r = blockIdx.x * C::B + tr;
    const float2* spec = spectra + (size_t)a * F * F;
    const int bi = argmax_final(argpart + (size_t)a * nparts, nparts, spec, F * F);
    const int2 p = make_int2(bi % F, bi / F);
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        posspec[a] = p;
        specval[a] = spec[bi];
    }
    float2 nrm = make_float2(1.0f, 0.0f);
    if (normalize) {  // TF_UBorn * conj(spec) / |spec| (main.cpp:332-335)
        const float2 s0 = spec[bi];
        const float mod = sqrtf(s0.y * s0.y + s0.x * s0.x);
        nrm = make_float2(s0.x / mod, -s0.y / mod);
    }
    const float2* src = spectra + ((size_t)a * F + ((r + p.y) & (F - 1))) * F;
    float2 x[E];
#pragma unroll
    for (int n1 = 0; n1 < E; ++n1) {
        float2 v = src[(j + n1 * T + p.x) & (F - 1)];
        x[n1] = normalize ? c_mul(v, nrm) : v;
    }
    fft_warp_regs<F, +1>(x, sm + tr * W::STRIDE, j, tw);
    float2* dst = I1 + ((size_t)a * F + r) * F;
#pragma unroll
    for (int q = 0; q < E / T; ++q) {
#pragma unroll
        for (int k2 = 0; k2 < T; ++k2) dst[j + q * T + E * k2] = x[q * T + k2];
    }
}

// mode 1: phase/amplitude (C_ABER); mode 0: the field itself is the result.
// mode 1 also leaves the CTA's sum of the wrapped phase in
// psum[a * kPhaseParts + blockIdx.x] (FP32 per thread and warp, FP64 across
// the warps in a fixed order).
template <int F>
__global__ void __launch_bounds__(FieldCfg<F>::NT)
k_field_cols(const float2* __restrict__ I1, int mode, const float2* __restrict__ tw, float* __restrict__ phase,
             float* __restrict__ amp, float2* __restrict__ zph, float2* __restrict__ fields,
             double* __restrict__ psum) {
    using C = FieldCfg<F>;
    using W = typename C::W;
    constexpr int B = C::B, NT = C::NT;
    extern __shared__ float2 sm[];
    const int tr = threadIdx.x / W::T, j = threadIdx.x % W::T;
    const int a = blockIdx.y, x0 = blockIdx.x * B;
#pragma unroll  // every staging load in flight before the first store
    for (int r0 = 0; r0 < B * F / NT; ++r0) {
        const int i = threadIdx.x + r0 * NT, t = i % B, r = i / B;
        sm[t * W::STRIDE + W::pad(r)] = I1[((size_t)a * F + r) * F + x0 + t];
    }
    __syncthreads();
    fft_warp<F, +1>(sm + tr * W::STRIDE, j, tw);
    __syncthreads();
    float acc = 0.0f;
#pragma unroll 8
    for (int r0 = 0; r0 < B * F / NT; ++r0) {
        const int i = threadIdx.x + r0 * NT, t = i % B, y = i / B;
        const float2 u = sm[t * W::STRIDE + W::pad(y)];
        const int yo = (y + F / 2) & (F - 1), xo = (x0 + t + F / 2) & (F - 1);
        const size_t o = ((size_t)a * F + yo) * F + xo;
        if (mode) {
            const float m = hypotf(u.x, u.y);
            const float ph = atan2f(u.y, u.x);
            phase[o] = ph;
            acc += ph;
            amp[o] = m;
            // exp(i phase) without the round trip through the angle; atan2(0, 0) = 0
            zph[o] = m > 0.0f ? make_float2(u.x / m, u.y / m) : make_float2(1.0f, 0.0f);
        } else {
            fields[o] = u;
        }
    }
    if (mode) phase_sum_cta<NT>(acc, psum + (size_t)a * kPhaseParts + blockIdx.x);
}

// ---------------------------------------------------------------- Volkov unwrap
// Mirror derivative from F-point transforms.  A row z of F samples has the
// half-sample-symmetric 2F-point mirror m (m[F + x] = m[F - 1 - x] = z[x]),
// whose spectrum is a DCT-II of z; its spectral derivative (gradient_fft4 on
// the mirror: FFT, x i 2 pi kappa(k)/2F with kappa(k) = k/2F signed, inverse)
// is a DST of kappa times that DCT.  Both run as F-point transforms of the
// row permuted by mirror_pos (even samples, then odd samples reversed): with
// V that transform,
//     W[k] = (i pi / 2F) (e^{i pi k/F} V[F - k] - (1 - 2k/F) V[k]),  W[0] = 0,
// and the unnormalised inverse w of W is the derivative at X = F + x,
// x = mirror_pos(m): w[m] for m < F/2, -w[m] otherwise.  The mirror's Nyquist
// bin is zero, so the reference's Nyquist factor -1/2 does not enter.  This
// is the right half of the 2F-point filter (FFT of the mirror, x i 2 pi
// kappa(k)/2F, inverse), from two F-point transforms instead of two 2F-point ones.
__host__ __device__ constexpr int mirror_pos(int m, int F) { return m < F / 2 ? 2 * m : 2 * (F - 1 - m) + 1; }

// x[n1] holds row sample mirror_pos(j + T n1) on entry and the derivative at
// X = F + mirror_pos(j + T n1) on return; s is the transform's exchange array.
template <int F>
__device__ __forceinline__ void mirror_derivative(float2 (&x)[WarpFFT<F>::E], float2* s, int j,
                                                  const float2* __restrict__ tw) {
    using W = WarpFFT<F>;
    constexpr int E = W::E, T = W::T, L = 2 * F;
    fft_warp_regs<F, -1>(x, s, j, tw);
    // bin k = (j + qT) + E k2 is in x[qT + k2]; bin F - k is held by lane T - j of
    // the transform, register (E/T - 1 - q)T + (T - 1 - k2), and for lane 0 by
    // itself, register (T - k2) mod T when q = 0, (E/T - q)T + T - 1 - k2 otherwise
    const int src = ((threadIdx.x & 31) & ~(T - 1)) + ((T - j) & (T - 1));
    float2 el[E / T];  // e^{i pi (j + qT)/F}
#pragma unroll
    for (int q = 0; q < E / T; ++q) {
        const float2 t = __ldg(&tw[(j + q * T) * (kTwN / L)]);
        el[q] = make_float2(t.x, -t.y);
    }
    constexpr float c = 0.5f * kTwoPi / (float)L;  // pi / 2F
    float2 y[E];
    static_for<0, E / T>([&](auto qc) {
        constexpr int q = decltype(qc)::value;
        static_for<0, T>([&](auto kc) {
            constexpr int k2 = decltype(kc)::value;
            const float2 pv = x[(E / T - 1 - q) * T + (T - 1 - k2)];
            float2 vm = make_float2(__shfl_sync(0xffffffffu, pv.x, src), __shfl_sync(0xffffffffu, pv.y, src));
            if (j == 0) vm = x[q == 0 ? (T - k2) % T : (E / T - q) * T + (T - 1 - k2)];
            const int k = j + q * T + E * k2;
            const float2 e = twc<2 * T, k2, 1>(el[q]);  // e^{i pi k/F}
            const float2 t = c_sub(c_mul(e, vm), c_scale(x[q * T + k2], 1.0f - 2.0f * (float)k / (float)F));
            y[q * T + k2] = k == 0 ? make_float2(0.0f, 0.0f) : make_float2(-c * t.y, c * t.x);
        });
    });
    fft_warp_regs_rev<F, +1>(y, s, j, tw);
#pragma unroll
    for (int n1 = 0; n1 < E; ++n1) x[n1] = (j + n1 * T < F / 2) ? y[n1] : make_float2(-y[n1].x, -y[n1].y);
}

// The DCT-II along a column of gx and the DST-II of gy, for k in [0, F),
// from one F-point transform (Makhoul's algorithm, two real sequences in one
// complex transform):
//     DCT-II(a)[k] = sum_y a[y] cos(pi k (2y + 1)/2F),
//     DST-II(b)[k] = sum_y b[y] sin(pi k (2y + 1)/2F) = DCT-II((-1)^y b)[F - k].
// With V the transform of a + i (-1)^y b permuted by mirror_pos and
// w = e^{-i pi k/2F},
//     DCT-II(a)[k] = Re(w V[k] + conj(w) V[F-k]) / 2,
//     DST-II(b)[k] = Re(w V[k] - conj(w) V[F-k]) / 2.
// x holds a + i (-1)^y b permuted (x[n1] = element j + T n1) on entry;
// out(k, (DCT-II(a)[k], DST-II(b)[k])) receives every bin k in [0, F) once.
template <int F, class Out>
__device__ __forceinline__ void column_dct_dst(float2 (&x)[WarpFFT<F>::E], float2* s, int j,
                                               const float2* __restrict__ tw, Out&& out) {
    using W = WarpFFT<F>;
    constexpr int E = W::E, T = W::T, L = 2 * F;
    fft_warp_regs<F, -1>(x, s, j, tw);
    __syncwarp();  // the transform is done with s, which out() may overwrite
    const int src = ((threadIdx.x & 31) & ~(T - 1)) + ((T - j) & (T - 1));  // holder of bin F - k
    float2 wl[E / T];  // e^{-i pi (j + qT)/2F}
#pragma unroll
    for (int q = 0; q < E / T; ++q) wl[q] = __ldg(&tw[(j + q * T) * (kTwN / (2 * L))]);
    static_for<0, E / T>([&](auto qc) {
        constexpr int q = decltype(qc)::value;
        static_for<0, T>([&](auto kc) {
            constexpr int k2 = decltype(kc)::value;
            const float2 pv = x[(E / T - 1 - q) * T + (T - 1 - k2)];
            float2 vm = make_float2(__shfl_sync(0xffffffffu, pv.x, src), __shfl_sync(0xffffffffu, pv.y, src));
            if (j == 0) vm = x[q == 0 ? (T - k2) % T : (E / T - q) * T + (T - 1 - k2)];
            const float2 w = twc<4 * T, k2, -1>(wl[q]);  // e^{-i pi k/2F}
            const float2 a = c_mul(w, x[q * T + k2]), b = c_mul(c_conj(w), vm);
            out(j + q * T + E * k2, make_float2(0.5f * (a.x + b.x), 0.5f * (a.x - b.x)));
        });
    });
}

// Pass 1 in CTAs of 8 image rows: one F-point derivative transform of Z per
// row (mirror_derivative).
template <int F>
struct RCfg {
    using W = WarpFFT<F>;
    static constexpr int B = 8;                 // rows (transforms) per CTA
    static constexpr int NT = B * W::T;
    static_assert(B % W::G == 0, "whole warps");
    static constexpr size_t SMEM = (size_t)B * W::STRIDE * sizeof(float2);
};

// Pass 2 in CTAs of NC = 8 mirror columns: NC F-point derivative transforms
// of Z, then NC F-point transforms giving each column's DCT-II of gx and
// DST-II of gy (column_dct_dst), staged in its Q array.
template <int L>
struct VCfg {
    using WF = WarpFFT<L / 2>;
    static constexpr int NC = 8;                 // columns per CTA
    static constexpr int BF = NC;                // derivative transforms per CTA
    static_assert(NC % WF::G == 0, "whole warps");
    static constexpr int NT = BF * WF::T;
    // array stride 2 mod 16 float2 and at least F: a warp's 8 columns x 4 rows
    // of the staging loops land in distinct banks
    static constexpr int FS = WF::LEN + ((2 - WF::LEN % 16) + 16) % 16;
    static constexpr size_t SMEM_COLS = (size_t)(BF + NC) * FS * sizeof(float2);
    // CTAs per SM the registers are bounded for (up to L = 512; larger mirrors
    // need their registers)
    static constexpr int COLS_CTAS = L <= 512 ? 4 : 1;
};

// Pass 1: rows of the mirror.  Mirror rows Y and L-1-Y are the same image
// row, and only the right half of the phasor's gradient
// gx = Re(-i dZ/dx / Z) / 2pi is kept: gx[Y][X] = sign(X) gxh[m(Y)][m(X)].
// Each image row's x derivative on that half comes from F-point transforms
// (mirror_derivative).
template <int L>
__global__ void __launch_bounds__(RCfg<L / 2>::NT)
k_volkov_rows(const float2* __restrict__ zph, const float2* __restrict__ tw, float* __restrict__ gxh) {
    constexpr int F = L / 2;
    using C = RCfg<F>;
    using W = typename C::W;
    constexpr int T = W::T, E = W::E;
    extern __shared__ float2 sm[];
    const int tr = threadIdx.x / T, j = threadIdx.x % T;
    const int a = blockIdx.y, y = blockIdx.x * C::B + tr;
    float2* s = sm + tr * W::STRIDE;
    const size_t row = ((size_t)a * F + y) * F;
    const float2* zr = zph + row;
    float2 x[E];
#pragma unroll
    for (int n1 = 0; n1 < E; ++n1) x[n1] = zr[mirror_pos(j + n1 * T, F)];
    mirror_derivative<F>(x, s, j, tw);
    __syncwarp();  // the transform's exchanges are done with s
#pragma unroll
    for (int n1 = 0; n1 < E; ++n1) s[W::pad(mirror_pos(j + n1 * T, F))] = x[n1];
    __syncwarp();
    float* out = gxh + row;
#pragma unroll
    for (int n1 = 0; n1 < E; ++n1) {
        const int xx = j + n1 * T;
        const float2 z = zr[xx];
        const float2 g = s[W::pad(xx)];
        out[xx] = (g.y * z.x - g.x * z.y) / (z.x * z.x + z.y * z.y) * kInvTwoPi;  // Re(-i g / Z) / 2pi
    }
}

// Pass 2: columns X = F + x of the mirror (columns X and L-1-X are the same
// image column): gy = Re(-i dZ/dy / Z) / 2pi like gx, then the first half of the Poisson solve's
// transforms: along y, gx (even about the mirror's axis) is a DCT-II and gy
// (odd) a DST-II of the quadrant's column, c[ky][x] = (DCT-II_y gx,
// DST-II_y gy) for ky in [0, F) (column_dct_dst).  The derivatives come from
// F-point transforms on the half Y = F + y (mirror_derivative).  The loads and
// the gy epilogue run CTA-wide with the NC columns fastest (contiguous in
// global memory); the phasor and gx are read from L2 in the epilogue.
template <int L>
__global__ void __launch_bounds__(VCfg<L>::NT, VCfg<L>::COLS_CTAS)
k_volkov_cols(const float2* __restrict__ zph, const float* __restrict__ gxh, const float2* __restrict__ tw,
              float2* __restrict__ cdct) {
    using C = VCfg<L>;
    using WF = typename C::WF;
    constexpr int F = L / 2, NC = C::NC, NT = C::NT, FS = C::FS, T = WF::T, E = WF::E;
    extern __shared__ float2 sm[];
    float2* sq = sm + C::BF * FS;  // NC arrays: gx + i (-1)^y gy of each column (permuted), then c[.][x]
    const int a = blockIdx.y, x0 = blockIdx.x * NC;
    const int tr = threadIdx.x / T, j = threadIdx.x % T;
    auto src = [&](int y, int c) { return ((size_t)a * F + y) * F + x0 + c; };
    // image row y goes to element m of the permuted column, mirror_pos(m) = y
    auto slot = [&](int y) { return (y & 1) ? F - 1 - (y >> 1) : (y >> 1); };
#pragma unroll  // every staging load in flight before the first store
    for (int i = threadIdx.x; i < NC * F; i += NT) {
        const int c = i % NC, y = i / NC;
        const size_t o = src(y, c);
        sm[c * FS + WF::pad(slot(y))] = zph[o];
    }
    __syncthreads();
    {  // y derivatives of Z
        float2* s = sm + tr * FS;
        float2 x[E];
#pragma unroll
        for (int n1 = 0; n1 < E; ++n1) x[n1] = s[WF::pad(j + n1 * T)];
        mirror_derivative<F>(x, s, j, tw);
        __syncwarp();
#pragma unroll
        for (int n1 = 0; n1 < E; ++n1) s[WF::pad(mirror_pos(j + n1 * T, F))] = x[n1];
    }
    __syncthreads();
    // gy = Re(-i dZ/dy / Z) / 2pi at Y = F + y; the Q array takes
    // gx + i (-1)^y gy, permuted (column_dct_dst's input)
#pragma unroll 4
    for (int i = threadIdx.x; i < NC * F; i += NT) {
        const int c = i % NC, y = i / NC;
        const size_t o = src(y, c);
        const float2 z = zph[o];
        const float gx = gxh[o];
        const float2 g = sm[c * FS + WF::pad(y)];
        const float gy = (g.y * z.x - g.x * z.y) / (z.x * z.x + z.y * z.y) * kInvTwoPi;
        sq[c * FS + WF::pad(slot(y))] = make_float2(gx, (y & 1) ? -gy : gy);
    }
    __syncthreads();
    {
        float2* s = sq + tr * FS;
        float2 x[E];
#pragma unroll
        for (int n1 = 0; n1 < E; ++n1) x[n1] = s[WF::pad(j + n1 * T)];
        column_dct_dst<F>(x, s, j, tw, [&](int k, float2 v) { s[k] = v; });
    }
    __syncthreads();
#pragma unroll 4
    for (int i = threadIdx.x; i < NC * F; i += NT) {
        const int c = i % NC, ky = i / NC;
        cdct[((size_t)a * F + ky) * F + x0 + c] = sq[c * FS + ky];
    }
}

// Pass 3: rows ky of the Poisson solve: integ_grad4 on the mirror
// (src/deroulement_volkov4.cpp:162-191) followed by cut_quad4 (:247-276),
// reduced to the quadrant.  With kappa = k/2F (init_kvect_shift, FFT_fonctions.cpp:7-17, on
// the half k < F that the folding keeps), A = DST-II_x DCT-II_y gx and
// B = DCT-II_x DST-II_y gy (k in [0, F)^2),
//     P = -4/L^2 (kappa_x A + kappa_y B) / (kappa_x^2 + kappa_y^2),  P(0, 0) = 0,
//     2 pi IntM = DCT-III_y DCT-III_x P,  DCT-III(P)[n] = sum_k w_k P[k] cos(pi k (2n+1)/2F),
// w_0 = 1, w_k = 2: the 2F x 2F transforms of the reference, with the
// symmetric halves of the spectrum folded together (the Nyquist terms cancel).
// Along x, A and B come from one F-point transform of (-1)^x Re c + i Im c
// permuted by mirror_pos: with V that transform, w = e^{-i pi k/2F},
// qu = w (V[k] + conj V[F-k]) / 2 and qv = w (V[k] - conj V[F-k]) / 2i,
//     A[k] = -Im qu,  B[k] = Re qv.
// The DCT-III of two real rows is one inverse transform: with
// X = P_r1 + i P_r2 and X[F] = 0, the unnormalised inverse transform of
// conj(w) (X[k] - i X[F-k]) is U_r1 + i U_r2 permuted by mirror_pos.
template <int F>
struct ICfg {
    using W = WarpFFT<F>;
    static constexpr int NW = 4;                   // warps per CTA
    static constexpr int R = 2 * NW * W::G;        // rows (pass 3) or columns (pass 4) per CTA, two per transform
    static constexpr int NT = NW * 32;
    static constexpr size_t SMEM = (size_t)NW * W::G * W::STRIDE * sizeof(float2);
};

// P[k] of the lane's bins of one row from its transform x (bin (j + qT) + E k2
// in register qT + k2), src the holder of bin F - k.
template <int F>
__device__ __forceinline__ void poisson_row(const float2 (&x)[WarpFFT<F>::E], const float2 (&wl)[WarpFFT<F>::E / WarpFFT<F>::T],
                                            int j, int src, float kyv, float (&p)[WarpFFT<F>::E]) {
    using W = WarpFFT<F>;
    constexpr int E = W::E, T = W::T, L = 2 * F;
    constexpr float s = -4.0f / ((float)L * (float)L);
    static_for<0, E / T>([&](auto qc) {
        constexpr int q = decltype(qc)::value;
        static_for<0, T>([&](auto kc) {
            constexpr int k2 = decltype(kc)::value;
            const float2 pv = x[(E / T - 1 - q) * T + (T - 1 - k2)];
            float2 vm = make_float2(__shfl_sync(0xffffffffu, pv.x, src), __shfl_sync(0xffffffffu, pv.y, src));
            if (j == 0) vm = x[q == 0 ? (T - k2) % T : (E / T - q) * T + (T - 1 - k2)];
            const int k = j + q * T + E * k2;
            const float2 w = twc<4 * T, k2, -1>(wl[q]);  // e^{-i pi k/2F}
            const float2 v = x[q * T + k2];
            const float2 e = c_mul(w, make_float2(v.x + vm.x, v.y - vm.y));  // 2 qu
            const float2 d = c_mul(w, make_float2(v.x - vm.x, v.y + vm.y));  // 2i qv
            const float kx = (float)k / (float)L;
            const float den = kx * kx + kyv * kyv;
            // A = -Im qu = -e.y / 2, B = Re qv = d.y / 2
            p[q * T + k2] = den > 0.0f ? (0.5f * s) * (kyv * d.y - kx * e.y) / den : 0.0f;
        });
    });
}

// The DCT-III input of the lanes' bins: y = conj(w) (X[k] - i X[F-k]), X[F] = 0.
template <int F>
__device__ __forceinline__ void dct3_input(const float2 (&xv)[WarpFFT<F>::E], const float2 (&wl)[WarpFFT<F>::E / WarpFFT<F>::T],
                                           int j, int src, float2 (&y)[WarpFFT<F>::E]) {
    using W = WarpFFT<F>;
    constexpr int E = W::E, T = W::T;
    static_for<0, E / T>([&](auto qc) {
        constexpr int q = decltype(qc)::value;
        static_for<0, T>([&](auto kc) {
            constexpr int k2 = decltype(kc)::value;
            const float2 pv = xv[(E / T - 1 - q) * T + (T - 1 - k2)];
            float2 xm = make_float2(__shfl_sync(0xffffffffu, pv.x, src), __shfl_sync(0xffffffffu, pv.y, src));
            if (j == 0) xm = q == 0 && k2 == 0 ? make_float2(0.0f, 0.0f) : xv[q == 0 ? (T - k2) % T : (E / T - q) * T + (T - 1 - k2)];
            const float2 w = twc<4 * T, k2, -1>(wl[q]);  // e^{-i pi k/2F}
            const float2 xk = xv[q * T + k2];
            y[q * T + k2] = c_mul(c_conj(w), make_float2(xk.x + xm.y, xk.y - xm.x));
        });
    });
}

template <int F>
__global__ void __launch_bounds__(ICfg<F>::NT)
k_volkov_integ_rows(const float2* __restrict__ cdct, const float2* __restrict__ tw, float* __restrict__ urows) {
    using C = ICfg<F>;
    using W = typename C::W;
    constexpr int T = W::T, E = W::E, L = 2 * F;
    extern __shared__ float2 sm[];
    const int tr = threadIdx.x / T, j = threadIdx.x % T;
    const int a = blockIdx.y, r1 = blockIdx.x * C::R + 2 * tr;  // rows r1 and r1 + 1
    float2* s = sm + tr * W::STRIDE;
    const int src = ((threadIdx.x & 31) & ~(T - 1)) + ((T - j) & (T - 1));  // holder of bin F - k
    float2 wl[E / T];  // e^{-i pi (j + qT)/2F}
#pragma unroll
    for (int q = 0; q < E / T; ++q) wl[q] = __ldg(&tw[(j + q * T) * (kTwN / (2 * L))]);
    float p1[E], p2[E];
#pragma unroll
    for (int h = 0; h < 2; ++h) {
        const float2* row = cdct + ((size_t)a * F + r1 + h) * F;
        float2 x[E];
#pragma unroll
        for (int n1 = 0; n1 < E; ++n1) {  // element m = j + T n1 is column mirror_pos(m): even for m < F/2
            const int m = j + n1 * T;
            const float2 v = row[mirror_pos(m, F)];
            x[n1] = make_float2(m < F / 2 ? v.x : -v.x, v.y);
        }
        fft_warp_regs<F, -1>(x, s, j, tw);
        poisson_row<F>(x, wl, j, src, (float)(r1 + h) / (float)L, h ? p2 : p1);
    }
    float2 xv[E], y[E];
#pragma unroll
    for (int n = 0; n < E; ++n) xv[n] = make_float2(p1[n], p2[n]);
    dct3_input<F>(xv, wl, j, src, y);
    fft_warp_regs_rev<F, +1>(y, s, j, tw);
    float* u1 = urows + ((size_t)a * F + r1) * F;
#pragma unroll
    for (int n1 = 0; n1 < E; ++n1) {
        const int xx = mirror_pos(j + n1 * T, F);
        u1[xx] = y[n1].x;
        u1[F + xx] = y[n1].y;
    }
}

// Pass 4: columns of U, two per transform: the DCT-III along y (dct3_input
// and one inverse transform) gives the unwrapped phase less its mean, and the
// wrapped phase's mean (from the field column pass's nps sums) is added as
// the rows are stored, contiguous, through the transforms' arrays.
template <int F>
__global__ void __launch_bounds__(ICfg<F>::NT)
k_volkov_integ_cols(const float* __restrict__ urows, const double* __restrict__ psum, int nps,
                    const float2* __restrict__ tw, float* __restrict__ unwrapped) {
    using C = ICfg<F>;
    using W = typename C::W;
    constexpr int T = W::T, E = W::E, L = 2 * F, R = C::R, NT = C::NT;
    extern __shared__ float2 sm[];
    const int tr = threadIdx.x / T, j = threadIdx.x % T;
    const int a = blockIdx.y, c0 = blockIdx.x * R;
    float* smf = reinterpret_cast<float*>(sm);
    __shared__ float s_mean;
    if (threadIdx.x == 0) s_mean = phase_mean(psum + (size_t)a * kPhaseParts, nps, F);  // ordered by the barrier below
    // column c0 + t of U into float slot (t & 1) of transform t / 2's array, at row ky
#pragma unroll  // every staging load in flight before the first store
    for (int r = 0; r < R * F / NT; ++r) {
        const int i = threadIdx.x + r * NT, t = i % R, ky = i / R;
        smf[2 * ((t >> 1) * W::STRIDE + ky) + (t & 1)] = urows[((size_t)a * F + ky) * F + c0 + t];
    }
    __syncthreads();
    float2* s = sm + tr * W::STRIDE;
    const int src = ((threadIdx.x & 31) & ~(T - 1)) + ((T - j) & (T - 1));
    float2 wl[E / T];
#pragma unroll
    for (int q = 0; q < E / T; ++q) wl[q] = __ldg(&tw[(j + q * T) * (kTwN / (2 * L))]);
    float2 xv[E], y[E];
#pragma unroll
    for (int q = 0; q < E / T; ++q) {
#pragma unroll
        for (int k2 = 0; k2 < T; ++k2) xv[q * T + k2] = s[j + q * T + E * k2];
    }
    dct3_input<F>(xv, wl, j, src, y);
    fft_warp_regs_rev<F, +1>(y, s, j, tw);
    __syncwarp();  // the transform's exchange is done with s
#pragma unroll
    for (int n1 = 0; n1 < E; ++n1) s[mirror_pos(j + n1 * T, F)] = y[n1];
    __syncthreads();
    const float mean = s_mean;
#pragma unroll 8
    for (int r = 0; r < R * F / NT; ++r) {
        const int i = threadIdx.x + r * NT, t = i % R, yy = i / R;
        unwrapped[((size_t)a * F + yy) * F + c0 + t] = mean + smf[2 * ((t >> 1) * W::STRIDE + yy) + (t & 1)];
    }
}

// ---------------------------------------------------------------- aberration fit
// The least-squares projections c_k = sum_s q_k(s) b(s) of image b (0: the
// unwrapped phase, 1: the amplitude) onto the basis orthonormal over the
// background samples, then the monomial coefficients beta = Rinv c (scaled
// coordinates).  kFitSlices CTAs per (angle, image) each sum one slice of the
// samples in FP32 (per thread, then per warp); the last CTA of the group to
// finish adds the slices' partial sums in FP64 in slice order and forms beta,
// so the result does not depend on the CTAs' timing.  With |q_k(s)| of order
// nsamp^-1/2 the FP32 rounding is a few ulps of |b|.
constexpr int kFitThreads = 256;
constexpr int kFitSlices = 8;

__global__ void __launch_bounds__(kFitThreads) k_aber_fit(const float* __restrict__ unwrapped,
                                                          const float* __restrict__ amp,
                                                          const int* __restrict__ samp_idx,
                                                          const float* __restrict__ samp_q, int nsamp, int F,
                                                          const double* __restrict__ rinv, float* __restrict__ part,
                                                          unsigned* __restrict__ done, double* __restrict__ beta) {
    const int sl = blockIdx.x, im = blockIdx.y, a = blockIdx.z, g = a * 2 + im;
    const float* img = (im == 0 ? unwrapped : amp) + (size_t)a * F * F;
    const int per = (nsamp + kFitSlices - 1) / kFitSlices;
    const int s0 = sl * per, s1 = min(nsamp, s0 + per);
    float acc[kNC];
#pragma unroll
    for (int k = 0; k < kNC; ++k) acc[k] = 0.0f;
#pragma unroll 2
    for (int s = s0 + threadIdx.x; s < s1; s += kFitThreads) {
        const float v = img[samp_idx[s]];
        const float* q = samp_q + (size_t)s * kNC;
#pragma unroll
        for (int k = 0; k < kNC; ++k) acc[k] = fmaf(q[k], v, acc[k]);
    }
    constexpr int NW = kFitThreads / 32;
    __shared__ float red[NW][kNC];
    __shared__ double cf[kNC];
    __shared__ bool last;
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
#pragma unroll
    for (int k = 0; k < kNC; ++k) {
        float x = acc[k];
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) x += __shfl_down_sync(0xffffffffu, x, off);
        if (l == 0) red[w][k] = x;
    }
    __syncthreads();
    if (threadIdx.x < kNC) {
        float x = 0.0f;
        for (int i = 0; i < NW; ++i) x += red[i][threadIdx.x];
        part[((size_t)g * kFitSlices + sl) * kNC + threadIdx.x] = x;
        __threadfence();
    }
    __syncthreads();
    if (threadIdx.x == 0) last = atomicAdd(&done[g], 1u) == kFitSlices - 1;
    __syncthreads();
    if (!last) return;
    __threadfence();
    if (threadIdx.x < kNC) {
        double x = 0.0;
        for (int i = 0; i < kFitSlices; ++i) x += (double)__ldcg(&part[((size_t)g * kFitSlices + i) * kNC + threadIdx.x]);
        cf[threadIdx.x] = x;
    }
    __syncthreads();
    if (threadIdx.x < kNC) {
        const int k = threadIdx.x;
        double x = 0.0;
#pragma unroll
        for (int i = 0; i < kNC; ++i) x = fma(rinv[k * kNC + i], cf[i], x);
        beta[(size_t)g * kNC + k] = x;
    }
    if (threadIdx.x == 0) done[g] = 0;  // ready for the next chunk
}

// Evaluates the fits, corrects phase and amplitude and forms the Born or Rytov field.
__global__ void __launch_bounds__(256) k_form(const float* __restrict__ unwrapped, const float* __restrict__ amp,
                                              const double* __restrict__ beta, int F, int born,
                                              float2* __restrict__ fields) {
    const int a = blockIdx.y;
    __shared__ float bf[2 * kNC];
    if (threadIdx.x < 2 * kNC) bf[threadIdx.x] = (float)beta[(size_t)a * 2 * kNC + threadIdx.x];
    __syncthreads();
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= F * F) return;
    const int x = idx % F, y = idx / F;
    const size_t o = (size_t)a * F * F + idx;
    fields[o] = form_value(form_row(bf, y, F), x, F, unwrapped[o], amp[o], born);
}

template <int F>
int fields_impl(tdm_ctx* c, int a0, int n, float* dbg_phase, float* dbg_unwrapped, float* dbg_amp, int argparts,
                bool form) {
    constexpr int L = 2 * F;
    using FC = FieldCfg<F>;
    using VC = VCfg<L>;
    using IC = ICfg<F>;
    const Params& p = c->p;
    Buffers& b = c->b;
    const size_t FF = (size_t)F * F;
    static_assert(F / FC::B <= kPhaseParts, "phase sums per angle");
    using RC = RCfg<F>;
    const size_t sm_vrows = RC::SMEM;
    const size_t sm_vcols = VC::SMEM_COLS;
    if (allow_smem(k_field_rows<F>, FC::SMEM) || allow_smem(k_field_cols<F>, FC::SMEM) ||
        allow_smem(k_volkov_rows<L>, sm_vrows) || allow_smem(k_volkov_cols<L>, sm_vcols) ||
        allow_smem(k_volkov_integ_rows<F>, IC::SMEM) || allow_smem(k_volkov_integ_cols<F>, IC::SMEM))
        return TDM_ECUDA;
    for (int g0 = a0; g0 < a0 + n; g0 += c->chunk) {
        const int m = (a0 + n - g0) < c->chunk ? (a0 + n - g0) : c->chunk;
        const float2* spec = b.spectra + (size_t)g0 * FF;
        int nparts = argparts;
        if (!nparts) {
            Launch l(c, K_ARGMAX);
            k_argmax_part<<<dim3(kArgSlices, m), 256, 0, c->stream>>>(spec, F, b.argpart);
            nparts = kArgSlices;
        }
        {
            Launch l(c, K_FIELD_ROWS);
            k_field_rows<F><<<dim3(F / FC::B, m), FC::NT, FC::SMEM, c->stream>>>(
                spec, b.argpart, nparts, b.posspec + g0, b.specval + g0, p.c_aber ? 0 : 1, b.tw, b.I1);
        }
        {
            Launch l(c, K_FIELD_COLS);
            k_field_cols<F><<<dim3(F / FC::B, m), FC::NT, FC::SMEM, c->stream>>>(
                b.I1, p.c_aber, b.tw, b.phase, b.amp, b.zph, b.fields + (size_t)g0 * FF, b.phase_sum);
        }
        if (!p.c_aber) continue;
        const float* unw = b.phase;
        if (p.deroul && !p.volkov) {
            if (int rc = launch_herraez(c, g0, m)) return rc;
            unw = b.unwrapped;
        } else if (p.deroul) {
            {
                Launch l(c, K_VOLKOV_ROWS);
                k_volkov_rows<L><<<dim3(F / RC::B, m), RC::NT, sm_vrows, c->stream>>>(b.zph, b.tw, b.gx);
            }
            {
                Launch l(c, K_VOLKOV_COLS);
                k_volkov_cols<L><<<dim3(F / VC::NC, m), VC::NT, sm_vcols, c->stream>>>(b.zph, b.gx, b.tw, b.qc);
            }
            float* urows = reinterpret_cast<float*>(b.tq);
            {
                Launch l(c, K_VOLKOV_INTEG_ROWS);
                k_volkov_integ_rows<F><<<dim3(F / IC::R, m), IC::NT, IC::SMEM, c->stream>>>(b.qc, b.tw, urows);
            }
            {
                Launch l(c, K_VOLKOV_INTEG_COLS);
                k_volkov_integ_cols<F><<<dim3(F / IC::R, m), IC::NT, IC::SMEM, c->stream>>>(
                    urows, b.phase_sum, F / FC::B, b.tw, b.unwrapped);
            }
            unw = b.unwrapped;
        }
        {
            Launch l(c, K_ABER_FIT);
            k_aber_fit<<<dim3(kFitSlices, 2, m), kFitThreads, 0, c->stream>>>(
                unw, b.amp, b.samp_idx, b.samp_q, c->nsamp, F, b.rinv, b.fit_part, b.fit_done, b.beta);
        }
        if (form) {
            Launch l(c, K_FORM);
            k_form<<<dim3((unsigned)((FF + 255) / 256), m), 256, 0, c->stream>>>(unw, b.amp, b.beta, F, p.born,
                                                                                b.fields + (size_t)g0 * FF);
        }
        if (dbg_phase)
            cudaMemcpyAsync(dbg_phase + (g0 - a0) * FF, b.phase, m * FF * sizeof(float), cudaMemcpyDefault, c->stream);
        if (dbg_unwrapped)
            cudaMemcpyAsync(dbg_unwrapped + (g0 - a0) * FF, unw, m * FF * sizeof(float), cudaMemcpyDefault, c->stream);
        if (dbg_amp)
            cudaMemcpyAsync(dbg_amp + (g0 - a0) * FF, b.amp, m * FF * sizeof(float), cudaMemcpyDefault, c->stream);
    }
    return cudaGetLastError() == cudaSuccess ? TDM_OK : TDM_ECUDA;
}

}  // namespace

int launch_argmax_part(tdm_ctx* c, const float2* spec, int m) {
    Launch l(c, K_ARGMAX);
    k_argmax_part<<<dim3(kArgSlices, m), 256, 0, c->stream>>>(spec, c->p.F, c->b.argpart);
    return kArgSlices;
}

void launch_aber_fit(tdm_ctx* c, const float* unw, int m) {
    Launch l(c, K_ABER_FIT);
    k_aber_fit<<<dim3(kFitSlices, 2, m), kFitThreads, 0, c->stream>>>(unw, c->b.amp, c->b.samp_idx, c->b.samp_q,
                                                                      c->nsamp, c->p.F, c->b.rinv, c->b.fit_part,
                                                                      c->b.fit_done, c->b.beta);
}

void launch_form(tdm_ctx* c, const float* unw, int g0, int m) {
    const size_t FF = (size_t)c->p.F * c->p.F;
    Launch l(c, K_FORM);
    k_form<<<dim3((unsigned)((FF + 255) / 256), m), 256, 0, c->stream>>>(unw, c->b.amp, c->b.beta, c->p.F, c->p.born,
                                                                        c->b.fields + (size_t)g0 * FF);
}

int launch_fields(tdm_ctx* c, int a0, int n, float* dbg_phase, float* dbg_unwrapped, float* dbg_amp, int argparts,
                  bool form) {
    if (c->p.F & (c->p.F - 1)) return launch_fields_generic(c, a0, n, dbg_phase, dbg_unwrapped, dbg_amp, argparts, form);
    switch (c->p.F) {
        case 64: return fields_impl<64>(c, a0, n, dbg_phase, dbg_unwrapped, dbg_amp, argparts, form);
        case 128: return fields_impl<128>(c, a0, n, dbg_phase, dbg_unwrapped, dbg_amp, argparts, form);
        case 256: return fields_impl<256>(c, a0, n, dbg_phase, dbg_unwrapped, dbg_amp, argparts, form);
        case 512: return fields_impl<512>(c, a0, n, dbg_phase, dbg_unwrapped, dbg_amp, argparts, form);
        default: return TDM_EUNSUPPORTED;
    }
}

}  // namespace tdm
