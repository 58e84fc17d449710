// Field formation and cap mapping for field sizes that are not powers of two.
//
// The reference's own configuration has NXMAX 125: 250 x 250 fields and a
// 500 x 500 Volkov mirror (Tomo_config/config_manip.txt:16).  These passes
// compute what the warp-resident passes of k_fields.cu and k_recon.cu
// compute, on the same buffers and with the same algebra, but each transform
// runs on the mixed-radix engine of fft_generic.cuh: one warp per transform,
// its points in shared memory in natural order.  A row pass gives each warp
// one row (coalesced loads and stores); a column pass stages kCols columns
// CTA-wide and gives each warp one column.  The passes:
//
//  gk_field_rows / gk_field_cols   calc_Uborn2 (pretraitement_hors_axe_CPU/fonctions.cpp:348-374):
//                                  shift by -posSpec, inverse FFT, shift by (N, N);
//                                  phase, amplitude and phasor (fonctions.cpp:39-43)
//  gk_volkov_rows / gk_volkov_cols deroul_volkov4_total_sym_paire (src/deroulement_volkov4.cpp:14-92):
//                                  the mirror's derivatives from F-point transforms
//                                  (a DCT-II of the row, its derivative a DST), and
//                                  the DCT-II of gx and DST-II of gy along each column
//                                  from one F-point transform
//  gk_volkov_integ_rows / _cols    integ_grad4 (:162-191) and cut_quad4 (:247-276) as
//                                  k_fields.cu's Poisson passes compute them: along x
//                                  the second half of the forward transforms, the
//                                  division by |kappa|^2 and a DCT-III; along y a DCT-III
//  gk_cap_rows(_form) / gk_cap_cols per-field spectrum (Reconstruction/main.cpp:203-217)
//                                  and the cap records of retroPropag_Born
//                                  (Reconstruction/src/fonctions.cpp:875-935)
#include "tdm_internal.cuh"
#include "fft_generic.cuh"
#include "cap_geometry.cuh"
#include "form.cuh"
#include "argmax.cuh"
#include "phase_mean.cuh"

namespace tdm {
namespace {

constexpr float kTwoPiG = 6.283185307179586f;
constexpr float kInvTwoPiG = 0.15915494309189535f;
constexpr int kRows = 8;  // warps (rows) per CTA of a row pass
constexpr int kCols = 8;  // columns (warps) per CTA of a column pass

// Element-wise copy of COUNT items by NT threads, thread tid taking items
// tid, tid + NT, ...: the thread issues all of its loads before its first
// store, so they are in flight together rather than one at a time behind
// each store (the loop bounds are compile-time, the loops unrolled).
template <int COUNT, int NT, class Load, class Store>
__device__ __forceinline__ void staged_copy(int tid, Load&& load, Store&& store) {
    constexpr int IT = (COUNT + NT - 1) / NT;
    decltype(load(0)) v[IT];
#pragma unroll
    for (int k = 0; k < IT; ++k) {
        const int i = tid + k * NT;
        if (i < COUNT) v[k] = load(i);
    }
#pragma unroll
    for (int k = 0; k < IT; ++k) {
        const int i = tid + k * NT;
        if (i < COUNT) store(i, v[k]);
    }
}

template <class K>
cudaError_t allow_smem(K kernel, size_t bytes) {
    return max_dynamic_smem(reinterpret_cast<const void*>(kernel), bytes);
}

__host__ __device__ constexpr int gmirror_pos(int m, int F) { return m < F / 2 ? 2 * m : 2 * (F - 1 - m) + 1; }
// element m of the permuted sequence that holds row (or column) y: gmirror_pos(m) = y
__host__ __device__ constexpr int gslot(int y, int F) { return (y & 1) ? F - 1 - (y >> 1) : (y >> 1); }

// exp(s 2 pi i k / M) from the 4F-entry table (M divides 4F).
template <int Q, int M, int S>
__device__ __forceinline__ float2 groot(const float2* __restrict__ wq, int k) {
    float2 w = __ldg(&wq[(k % M) * (Q / M)]);
    if constexpr (S > 0) w.y = -w.y;
    return w;
}

// Mirror derivative from F-point transforms (the algebra of k_fields.cu's
// mirror_derivative): a holds the row permuted by gmirror_pos on entry; on
// return a[x] holds the derivative of the row's 2F-point even mirror at
// X = F + x.  b is scratch.
template <int F>
__device__ __forceinline__ void gmirror_derivative(float2* a, float2* b, const float2* __restrict__ wq, int lane) {
    constexpr int Q = 4 * F;
    constexpr float c = 0.5f * kTwoPiG / (float)(2 * F);  // pi / 2F
    gfft<F, -1, Q>(a, b, wq, lane);
    for (int k = lane; k < F; k += 32) {
        // W[k] = (i pi / 2F) (e^{i pi k/F} V[F-k] - (1 - 2k/F) V[k]), W[0] = 0
        const float2 vm = a[k ? F - k : 0];
        const float2 e = groot<Q, 2 * F, +1>(wq, k);
        const float2 t = c_sub(c_mul(e, vm), c_scale(a[k], 1.0f - 2.0f * (float)k / (float)F));
        b[k] = k == 0 ? make_float2(0.0f, 0.0f) : make_float2(-c * t.y, c * t.x);
    }
    __syncwarp();
    gfft<F, +1, Q>(b, a, wq, lane);
    for (int m = lane; m < F; m += 32) a[gmirror_pos(m, F)] = m < F / 2 ? b[m] : make_float2(-b[m].x, -b[m].y);
    __syncwarp();
}

// ---------------------------------------------------------------- field = shift(IFFT(shift(S)))
template <int F>
__global__ void __launch_bounds__(kRows * 32)
gk_field_rows(const float2* __restrict__ spectra, const float4* __restrict__ argpart, int nparts,
              int2* __restrict__ posspec, float2* __restrict__ specval, int normalize, const float2* __restrict__ wq,
              float2* __restrict__ I1) {
    extern __shared__ float2 sm[];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int a = blockIdx.y, r = blockIdx.x * kRows + w;
    const float2* spec = spectra + (size_t)a * F * F;
    const int bi = argmax_final(argpart + (size_t)a * nparts, nparts, spec, F * F);
    const int2 p = make_int2(bi % F, bi / F);
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        posspec[a] = p;
        specval[a] = spec[bi];
    }
    if (r >= F) return;  // warp-uniform, after the CTA-wide search
    float2 nrm = make_float2(1.0f, 0.0f);
    if (normalize) {  // TF_UBorn * conj(spec) / |spec| (main.cpp:332-335)
        const float2 s0 = spec[bi];
        const float mod = sqrtf(s0.y * s0.y + s0.x * s0.x);
        nrm = make_float2(s0.x / mod, -s0.y / mod);
    }
    float2* A = sm + w * 2 * F;
    float2* B = A + F;
    const float2* src = spec + (size_t)wrap_f(r + p.y, F) * F;
    staged_copy<F, 32>(
        lane, [&](int n) { return src[wrap_f(n + p.x, F)]; },
        [&](int n, float2 v) { A[n] = normalize ? c_mul(v, nrm) : v; });
    __syncwarp();
    gfft<F, +1, 4 * F>(A, B, wq, lane);
    float2* dst = I1 + ((size_t)a * F + r) * F;
    for (int k = lane; k < F; k += 32) dst[k] = A[k];
}

// mode 1: phase/amplitude/phasor (C_ABER) and the CTA's sum of the wrapped
// phase in psum[a * kPhaseParts + blockIdx.x]; mode 0: the field itself.
template <int F>
__global__ void __launch_bounds__(kCols * 32)
gk_field_cols(const float2* __restrict__ I1, int mode, const float2* __restrict__ wq, float* __restrict__ phase,
              float* __restrict__ amp, float2* __restrict__ zph, float2* __restrict__ fields,
              double* __restrict__ psum) {
    extern __shared__ float2 sm[];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int a = blockIdx.y, x0 = blockIdx.x * kCols;
    staged_copy<kCols * F, kCols * 32>(
        threadIdx.x,
        [&](int i) {
            const int t = i % kCols, r = i / kCols;
            return x0 + t < F ? I1[((size_t)a * F + r) * F + x0 + t] : make_float2(0.f, 0.f);
        },
        [&](int i, float2 v) {
            if (x0 + i % kCols < F) sm[(i % kCols) * 2 * F + i / kCols] = v;
        });
    __syncthreads();
    if (x0 + w < F) gfft<F, +1, 4 * F>(sm + w * 2 * F, sm + w * 2 * F + F, wq, lane);
    __syncthreads();
    float acc = 0.0f;
    for (int i = threadIdx.x; i < kCols * F; i += blockDim.x) {
        const int t = i % kCols, y = i / kCols;
        if (x0 + t >= F) continue;
        const float2 u = sm[t * 2 * F + y];
        const int yo = wrap_f(y + F / 2, F), xo = wrap_f(x0 + t + F / 2, F);
        const size_t o = ((size_t)a * F + yo) * F + xo;
        if (mode) {
            const float m = hypotf(u.x, u.y);
            const float ph = atan2f(u.y, u.x);
            phase[o] = ph;
            acc += ph;
            amp[o] = m;
            zph[o] = m > 0.0f ? make_float2(u.x / m, u.y / m) : make_float2(1.0f, 0.0f);
        } else {
            fields[o] = u;
        }
    }
    if (mode) phase_sum_cta<kCols * 32>(acc, psum + (size_t)a * kPhaseParts + blockIdx.x);
}

// ---------------------------------------------------------------- Volkov unwrap
// Pass 1: rows, one warp per image row: the x derivative of the phasor Z on
// the mirror's right half gives gx = Re(-i dZ/dx / Z) / 2pi (the wrapped
// phase's own gradient is not formed: k_fields.cu's Volkov notes).
constexpr int kVRows = 8;  // rows (warps) per CTA
template <int F>
__global__ void __launch_bounds__(kVRows * 32)
gk_volkov_rows(const float2* __restrict__ zph, const float2* __restrict__ wq, float* __restrict__ gxh) {
    extern __shared__ float2 sm[];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int a = blockIdx.y, y = blockIdx.x * kVRows + w;
    if (y >= F) return;  // warp-uniform; no CTA barrier below
    float2* A = sm + w * 2 * F;
    float2* B = A + F;
    const size_t row = ((size_t)a * F + y) * F;
    const float2* zr = zph + row;
    staged_copy<F, 32>(
        lane, [&](int m) { return zr[gmirror_pos(m, F)]; }, [&](int m, float2 v) { A[m] = v; });
    __syncwarp();
    gmirror_derivative<F>(A, B, wq, lane);
    float* out = gxh + row;
    staged_copy<F, 32>(
        lane, [&](int x) { return zr[x]; },
        [&](int x, float2 z) {
            const float2 g = A[x];
            out[x] = (g.y * z.x - g.x * z.y) / (z.x * z.x + z.y * z.y) * kInvTwoPiG;  // Re(-i g / Z) / 2pi
        });
}

// Pass 2: columns X = F + x of the mirror, kCols per CTA: the y derivatives
// of the kCols Z columns, gy = Re(-i dZ/dy / Z) / 2pi, then the column's
// DCT-II of gx and DST-II of gy from one F-point transform of
// gx + i (-1)^y gy permuted by gmirror_pos (k_fields.cu's column_dct_dst):
// with V that transform and w = e^{-i pi k/2F},
//     DCT-II(gx)[k] = Re(w V[k] + conj(w) V[F-k]) / 2,
//     DST-II(gy)[k] = Re(w V[k] - conj(w) V[F-k]) / 2,
// stored as cdct[ky][x] for ky in [0, F).
// Four CTAs per SM: registers capped at 64 (uncapped, 80 and three CTAs ran slower).
template <int F>
__global__ void __launch_bounds__(kCols * 32, 4)
gk_volkov_cols(const float2* __restrict__ zph, const float* __restrict__ gxh, const float2* __restrict__ wq,
               float2* __restrict__ cdct) {
    constexpr int L = 2 * F, Q4 = 4 * F;
    extern __shared__ float2 sm[];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int a = blockIdx.y, x0 = blockIdx.x * kCols;
    auto arr = [&](int t) { return sm + t * 2 * F; };  // warp t's pair of F-point arrays
    constexpr int NT = kCols * 32;
    staged_copy<kCols * F, NT>(
        threadIdx.x,
        [&](int i) {
            const size_t o = ((size_t)a * F + i / kCols) * F + x0 + i % kCols;
            return x0 + i % kCols < F ? zph[o] : make_float2(0.f, 0.f);
        },
        [&](int i, float2 v) {
            const int c = i % kCols;
            if (x0 + c < F) arr(c)[gslot(i / kCols, F)] = v;
        });
    __syncthreads();
    const bool live = x0 + w < F;  // warp-uniform
    if (live) gmirror_derivative<F>(arr(w), arr(w) + F, wq, lane);
    __syncthreads();
    staged_copy<kCols * F, NT>(
        threadIdx.x,
        [&](int i) {
            const size_t o = ((size_t)a * F + i / kCols) * F + x0 + i % kCols;
            if (x0 + i % kCols >= F) return make_float3(1.f, 0.f, 0.f);
            const float2 z = zph[o];
            return make_float3(z.x, z.y, gxh[o]);
        },
        [&](int i, float3 v) {
            const int c = i % kCols, y = i / kCols;
            if (x0 + c >= F) return;
            const float2 g = arr(c)[y];
            const float gy = (g.y * v.x - g.x * v.y) / (v.x * v.x + v.y * v.y) * kInvTwoPiG;
            arr(c)[F + gslot(y, F)] = make_float2(v.z, (y & 1) ? -gy : gy);
        });
    __syncthreads();
    if (w < kCols && x0 + w < F) {
        float2* V = arr(w) + F;
        float2* S = arr(w);
        gfft<F, -1, Q4>(V, S, wq, lane);
        for (int k = lane; k < F; k += 32) {  // S is free: gfft left the result in V
            const float2 wk = groot<Q4, 2 * L, -1>(wq, k);  // e^{-i pi k/2F}
            const float2 va = c_mul(wk, V[k]), vb = c_mul(c_conj(wk), V[k ? F - k : 0]);
            S[k] = make_float2(0.5f * (va.x + vb.x), 0.5f * (va.x - vb.x));
        }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < kCols * F; i += blockDim.x) {
        const int c = i % kCols, ky = i / kCols;
        if (x0 + c < F) cdct[((size_t)a * F + ky) * F + x0 + c] = arr(c)[ky];
    }
}

// Pass 3: row pairs of the Poisson solve (k_fields.cu's k_volkov_integ_rows):
// per row, one F-point transform of (-1)^x Re c + i Im c permuted by
// gmirror_pos gives A = DST-II_x and B = DCT-II_x of the row, and
// P = -4/L^2 (kappa_x A + kappa_y B) / (kappa_x^2 + kappa_y^2); the two rows'
// P = P_r1 + i P_r2 then take one inverse transform for their DCT-III along x.
// Three F-point arrays per warp: the transform, its scratch and P.
template <int F>
__global__ void __launch_bounds__(kRows * 32)
gk_volkov_integ_rows(const float2* __restrict__ cdct, const float2* __restrict__ wq, float* __restrict__ urows) {
    constexpr int L = 2 * F, Q4 = 4 * F;
    constexpr float sc = -4.0f / ((float)L * (float)L);
    extern __shared__ float2 sm[];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int a = blockIdx.y, r1 = 2 * (blockIdx.x * kRows + w);
    if (r1 >= F) return;  // warp-uniform; no CTA barrier below
    float2* A = sm + w * 3 * F;
    float2* B = A + F;
    float2* P = B + F;
#pragma unroll
    for (int h = 0; h < 2; ++h) {
        const float2* row = cdct + ((size_t)a * F + r1 + h) * F;
        staged_copy<F, 32>(
            lane, [&](int m) { return row[gmirror_pos(m, F)]; },
            [&](int m, float2 v) { A[m] = make_float2(m < F / 2 ? v.x : -v.x, v.y); });  // (-1)^x, x = gmirror_pos(m)
        __syncwarp();
        gfft<F, -1, Q4>(A, B, wq, lane);
        const float kyv = (float)(r1 + h) / (float)L;
        for (int k = lane; k < F; k += 32) {
            const float2 v = A[k], vm = A[k ? F - k : 0];
            const float2 wk = groot<Q4, 2 * L, -1>(wq, k);  // e^{-i pi k/2F}
            const float2 e = c_mul(wk, make_float2(v.x + vm.x, v.y - vm.y));  // 2 qu
            const float2 d = c_mul(wk, make_float2(v.x - vm.x, v.y + vm.y));  // 2i qv
            const float kx = (float)k / (float)L, den = kx * kx + kyv * kyv;
            const float pk = den > 0.0f ? (0.5f * sc) * (kyv * d.y - kx * e.y) / den : 0.0f;
            reinterpret_cast<float*>(&P[k])[h] = pk;
        }
        __syncwarp();  // every lane has read A before the next row overwrites it
    }
    for (int k = lane; k < F; k += 32) {  // DCT-III input conj(w) (X[k] - i X[F-k]), X[F] = 0
        const float2 x = P[k], xm = k ? P[F - k] : make_float2(0.0f, 0.0f);
        A[k] = c_mul(c_conj(groot<Q4, 2 * L, -1>(wq, k)), make_float2(x.x + xm.y, x.y - xm.x));
    }
    __syncwarp();
    gfft<F, +1, Q4>(A, B, wq, lane);
    float* u1 = urows + ((size_t)a * F + r1) * F;
    for (int m = lane; m < F; m += 32) {
        const int x = gmirror_pos(m, F);
        u1[x] = A[m].x;
        u1[F + x] = A[m].y;
    }
}

// Pass 4: column pairs: the DCT-III along y gives the unwrapped phase less
// its mean, and the wrapped phase's mean (from the field column pass's nps
// sums) is added as it is stored with the columns fastest.  Three F-point
// arrays per warp: the transform, its scratch and the column pair.
template <int F>
__global__ void __launch_bounds__(kCols * 32)
gk_volkov_integ_cols(const float* __restrict__ urows, const double* __restrict__ psum, int nps,
                     const float2* __restrict__ wq, float* __restrict__ unwrapped) {
    constexpr int L = 2 * F, Q4 = 4 * F, NC = 2 * kCols;
    extern __shared__ float2 sm[];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int a = blockIdx.y, c0 = blockIdx.x * NC;
    auto pair = [&](int t) { return sm + t * 3 * F + 2 * F; };  // warp t's column pair
    __shared__ float s_mean;
    if (threadIdx.x == 0) s_mean = phase_mean(psum + (size_t)a * kPhaseParts, nps, F);  // ordered by the barriers below
    staged_copy<NC * F, kCols * 32>(
        threadIdx.x,
        [&](int i) {
            const int t = i % NC, ky = i / NC;
            return c0 + t < F ? urows[((size_t)a * F + ky) * F + c0 + t] : 0.f;
        },
        [&](int i, float u) {
            const int t = i % NC, ky = i / NC;
            reinterpret_cast<float*>(&pair(t >> 1)[ky])[t & 1] = u;
        });
    __syncthreads();
    if (c0 + 2 * w < F) {  // warp-uniform; F is even, so both columns are in range
        float2* A = sm + w * 3 * F;
        float2* B = A + F;
        float2* X = pair(w);
        for (int k = lane; k < F; k += 32) {
            const float2 x = X[k], xm = k ? X[F - k] : make_float2(0.0f, 0.0f);
            A[k] = c_mul(c_conj(groot<Q4, 2 * L, -1>(wq, k)), make_float2(x.x + xm.y, x.y - xm.x));
        }
        __syncwarp();
        gfft<F, +1, Q4>(A, B, wq, lane);
        for (int m = lane; m < F; m += 32) X[gmirror_pos(m, F)] = A[m];
    }
    __syncthreads();
    const float mean = s_mean;
    for (int i = threadIdx.x; i < NC * F; i += kCols * 32) {
        const int t = i % NC, y = i / NC;
        if (c0 + t < F)
            unwrapped[((size_t)a * F + y) * F + c0 + t] = mean + reinterpret_cast<const float*>(&pair(t >> 1)[y])[t & 1];
    }
}

// ---------------------------------------------------------------- cap passes
// Row pass of the per-field spectrum: x Tukey(0.1) in x and y, forward FFT
// along x.  FORM: the field is formed on the fly from the chunk's unwrapped
// phase, amplitude and fits (k_form's arithmetic) and also stored.
template <int F, bool FORM>
__global__ void __launch_bounds__(kRows * 32)
gk_cap_rows(const float2* __restrict__ fields_in, const float* __restrict__ unwrapped, const float* __restrict__ amp,
            const double* __restrict__ beta, int born, const float* __restrict__ tuk, int2 flat,
            const float2* __restrict__ wq, float2* __restrict__ fields_out, float2* __restrict__ r1) {
    extern __shared__ float2 sm[];
    __shared__ float bf[2 * kNC];
    if (FORM) {
        if (threadIdx.x < 2 * kNC) bf[threadIdx.x] = (float)beta[(size_t)blockIdx.y * 2 * kNC + threadIdx.x];
        __syncthreads();
    }
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int a = blockIdx.y, y = blockIdx.x * kRows + w;
    if (y >= F) return;
    float2* A = sm + w * 2 * F;
    const float wy = tuk[y];
    const size_t row = ((size_t)a * F + y) * F;
    FormRow fr;
    if (FORM) fr = form_row(bf, y, F);
    for (int x = lane; x < F; x += 32) {
        float2 f;
        if (FORM) {
            f = form_value(fr, x, F, unwrapped[row + x], amp[row + x], born);
            fields_out[row + x] = f;
        } else {
            f = fields_in[row + x];
        }
        A[x] = c_scale(f, ((x >= flat.x && x <= flat.y) ? 1.0f : __ldg(&tuk[x])) * wy);
    }
    __syncwarp();
    gfft<F, -1, 4 * F>(A, A + F, wq, lane);
    for (int k = lane; k < F; k += 32) r1[row + k] = A[k];
}

// Column pass: forward FFT along y, then per bin the cap value (contribution
// on the cap cells, 0 elsewhere) and the cell's plane, as k_cap_cols writes them.
template <int F>
__global__ void __launch_bounds__(kCols * 32)
gk_cap_cols(const float2* __restrict__ r1, const int2* __restrict__ posspec, const double* __restrict__ s_tab,
            const float* __restrict__ s_tabf, Params p, const float2* __restrict__ wq, float2* __restrict__ rec,
            int16_t* __restrict__ recz, int* __restrict__ err) {
    extern __shared__ float2 sm[];
    __shared__ double s_fz;
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int a = blockIdx.y, kx0 = blockIdx.x * kCols;
    const int2 ps = posspec[a];
    if (threadIdx.x == 0) s_fz = cap_fzm0(p, ps);
    staged_copy<kCols * F, kCols * 32>(
        threadIdx.x,
        [&](int i) {
            const int t = i % kCols, ky = i / kCols;
            return kx0 + t < F ? r1[((size_t)a * F + ky) * F + kx0 + t] : make_float2(0.f, 0.f);
        },
        [&](int i, float2 v) {
            if (kx0 + i % kCols < F) sm[(i % kCols) * 2 * F + i / kCols] = v;
        });
    __syncthreads();
    if (kx0 + w < F) gfft<F, -1, 4 * F>(sm + w * 2 * F, sm + w * 2 * F + F, wq, lane);
    __syncthreads();
    const double fz = s_fz;
    const float fzf = (float)fz, ir = (float)p.inv_rayon;
    for (int i = threadIdx.x; i < kCols * F; i += blockDim.x) {
        const int t = i % kCols, ky = i / kCols, kx = kx0 + t;
        if (kx >= F) continue;
        const size_t o = ((size_t)a * F + ky) * F + kx;
        float sf = 0.f;
        const int z = cap_plane(p, ps, fz, fzf, kx, ky, s_tab, s_tabf, &sf, err);
        float2 val = make_float2(0.f, 0.f);
        if (z >= 0) {
            const float2 v = sm[t * 2 * F + ky];
            const float Bc = cap_weight(p, sf, ir, kx, ky);
            val = make_float2(-Bc * v.y, Bc * v.x);
        }
        rec[o] = val;
        recz[o] = (int16_t)z;
    }
}

constexpr size_t warp_arrays(int n, int warps) { return (size_t)warps * 2 * n * sizeof(float2); }

template <int F>
int gfields_impl(tdm_ctx* c, int a0, int n, float* dbg_phase, float* dbg_unwrapped, float* dbg_amp, int argparts,
                 bool form) {
    const Params& p = c->p;
    Buffers& b = c->b;
    const size_t FF = (size_t)F * F;
    const size_t sm_rows = warp_arrays(F, kRows), sm_cols = warp_arrays(F, kCols);
    const size_t sm_vrows = warp_arrays(F, kVRows), sm_vcols = warp_arrays(F, kCols);
    static_assert((F + kCols - 1) / kCols <= kPhaseParts, "phase sums per angle");
    const size_t sm_irows = (size_t)kRows * 3 * F * sizeof(float2), sm_icols = (size_t)kCols * 3 * F * sizeof(float2);
    if (allow_smem(gk_field_rows<F>, sm_rows) || allow_smem(gk_field_cols<F>, sm_cols) ||
        allow_smem(gk_volkov_rows<F>, sm_vrows) || allow_smem(gk_volkov_cols<F>, sm_vcols) ||
        allow_smem(gk_volkov_integ_rows<F>, sm_irows) || allow_smem(gk_volkov_integ_cols<F>, sm_icols))
        return TDM_ECUDA;
    const unsigned rows = (F + kRows - 1) / kRows, cols = (F + kCols - 1) / kCols;
    for (int g0 = a0; g0 < a0 + n; g0 += c->chunk) {
        const int m = (a0 + n - g0) < c->chunk ? (a0 + n - g0) : c->chunk;
        const float2* spec = b.spectra + (size_t)g0 * FF;
        const int nparts = argparts ? argparts : launch_argmax_part(c, spec, m);
        {
            Launch l(c, K_FIELD_ROWS);
            gk_field_rows<F><<<dim3(rows, m), kRows * 32, sm_rows, c->stream>>>(
                spec, b.argpart, nparts, b.posspec + g0, b.specval + g0, p.c_aber ? 0 : 1, b.wq, b.I1);
        }
        {
            Launch l(c, K_FIELD_COLS);
            gk_field_cols<F><<<dim3(cols, m), kCols * 32, sm_cols, c->stream>>>(
                b.I1, p.c_aber, b.wq, b.phase, b.amp, b.zph, b.fields + (size_t)g0 * FF, b.phase_sum);
        }
        if (!p.c_aber) continue;
        const float* unw = b.phase;
        if (p.deroul && !p.volkov) {
            if (int rc = launch_herraez(c, g0, m)) return rc;
            unw = b.unwrapped;
        } else if (p.deroul) {
            {
                Launch l(c, K_VOLKOV_ROWS);
                gk_volkov_rows<F><<<dim3((F + kVRows - 1) / kVRows, m), kVRows * 32, sm_vrows, c->stream>>>(
                    b.zph, b.wq, b.gx);
            }
            {
                Launch l(c, K_VOLKOV_COLS);
                gk_volkov_cols<F><<<dim3(cols, m), kCols * 32, sm_vcols, c->stream>>>(b.zph, b.gx, b.wq, b.qc);
            }
            float* urows = reinterpret_cast<float*>(b.tq);
            {
                Launch l(c, K_VOLKOV_INTEG_ROWS);
                gk_volkov_integ_rows<F><<<dim3((F / 2 + kRows - 1) / kRows, m), kRows * 32, sm_irows, c->stream>>>(
                    b.qc, b.wq, urows);
            }
            {
                Launch l(c, K_VOLKOV_INTEG_COLS);
                gk_volkov_integ_cols<F><<<dim3((F + 2 * kCols - 1) / (2 * kCols), m), kCols * 32, sm_icols,
                                          c->stream>>>(urows, b.phase_sum, (int)cols, b.wq, b.unwrapped);
            }
            unw = b.unwrapped;
        }
        launch_aber_fit(c, unw, m);
        if (form) launch_form(c, unw, g0, m);
        if (dbg_phase)
            cudaMemcpyAsync(dbg_phase + (g0 - a0) * FF, b.phase, m * FF * sizeof(float), cudaMemcpyDefault, c->stream);
        if (dbg_unwrapped)
            cudaMemcpyAsync(dbg_unwrapped + (g0 - a0) * FF, unw, m * FF * sizeof(float), cudaMemcpyDefault, c->stream);
        if (dbg_amp)
            cudaMemcpyAsync(dbg_amp + (g0 - a0) * FF, b.amp, m * FF * sizeof(float), cudaMemcpyDefault, c->stream);
    }
    return cudaGetLastError() == cudaSuccess ? TDM_OK : TDM_ECUDA;
}

template <int F>
int gcap_impl(tdm_ctx* c, int a0, int n, bool form) {
    Buffers& b = c->b;
    const size_t sm_rows = warp_arrays(F, kRows), sm_cols = warp_arrays(F, kCols);
    if (allow_smem(gk_cap_rows<F, false>, sm_rows) || allow_smem(gk_cap_rows<F, true>, sm_rows) ||
        allow_smem(gk_cap_cols<F>, sm_cols))
        return TDM_ECUDA;
    if (form && n > c->chunk) return TDM_EINVAL;  // the chunk buffers hold one chunk
    const size_t FF = (size_t)F * F;
    const unsigned rows = (F + kRows - 1) / kRows, cols = (F + kCols - 1) / kCols;
    for (int g0 = a0; g0 < a0 + n; g0 += c->chunk) {
        const int m = a0 + n - g0 < c->chunk ? a0 + n - g0 : c->chunk;
        {
            Launch l(c, K_CAP_ROWS);
            if (form)
                gk_cap_rows<F, true><<<dim3(rows, m), kRows * 32, sm_rows, c->stream>>>(
                    nullptr, c->p.deroul ? b.unwrapped : b.phase, b.amp, b.beta, c->p.born, b.tuk_f, c->tuk_f_flat,
                    b.wq, b.fields + g0 * FF, b.r1);
            else
                gk_cap_rows<F, false><<<dim3(rows, m), kRows * 32, sm_rows, c->stream>>>(
                    b.fields + g0 * FF, nullptr, nullptr, nullptr, 0, b.tuk_f, c->tuk_f_flat, b.wq, nullptr, b.r1);
        }
        {
            Launch l(c, K_CAP_COLS);
            gk_cap_cols<F><<<dim3(cols, m), kCols * 32, sm_cols, c->stream>>>(b.r1, b.posspec + g0, b.s_tab, b.s_tabf,
                                                                            c->p, b.wq, b.rec.val + g0 * FF,
                                                                            b.rec.z + g0 * FF, b.err);
        }
    }
    return cudaGetLastError() == cudaSuccess ? TDM_OK : TDM_ECUDA;
}

}  // namespace

// 2 NXMAX of the reference's own configuration (NXMAX 125); add a size here
// (and to generic_field_size) to compile the passes for it.
bool generic_field_size(int F) { return F == 250; }

int launch_fields_generic(tdm_ctx* c, int a0, int n, float* dbg_phase, float* dbg_unwrapped, float* dbg_amp,
                          int argparts, bool form) {
    switch (c->p.F) {
        case 250: return gfields_impl<250>(c, a0, n, dbg_phase, dbg_unwrapped, dbg_amp, argparts, form);
        default: return TDM_EUNSUPPORTED;
    }
}

int launch_cap_generic(tdm_ctx* c, int a0, int n, bool form) {
    switch (c->p.F) {
        case 250: return gcap_impl<250>(c, a0, n, form);
        default: return TDM_EUNSUPPORTED;
    }
}

}  // namespace tdm
