// Reconstruction (Reconstruction/main.cpp:203-352).
//
// Per field (main.cpp:207-217): x Tukey(0.1), shift by (N, N), forward FFT x dx^2,
// shift by posSpec.  With k the FFT bin, the value that retroPropag_Born reads
// at cap pixel fd = ((k + posSpec) mod F) - N is
//     (-1)^(kx+ky) dx^2 FFT2(field * tukey)[k],
// so the per-field kernels work on natural FFT bins and store, per bin, the
// cap contribution -2i k0 sdz value (cteUb2Pot*cteNorm*sdz, fonctions.cpp:902,927)
// and its volume plane z (-1 outside the NA disc).
//
// Mapping (retroPropag_Born, src/fonctions.cpp:875-935) as a gather: voxel
// column (X, Y) reads bin kx = (X - D/2) mod F for every angle whose cap window
// covers it; each angle hits a column at most once, so one thread per column
// walking the angles in order accumulates in the reference's order, without
// atomics, in FP64; hit counts are exact.  Accumulators live in a per-CTA
// scratch slab (L2-resident while the CTA runs).
//
// Volume: fftshift3D, backward 3D FFT x Delta_f^3, fftshift3D, x -1/(2 n0 kv^2)
// (main.cpp:282-352).  For even D the two shifts are sign modulations:
//     out[m] = (-1)^(mx+my+mz+3D/2) IFFT3((-1)^(kx+ky+kz) V)[m].
// The z transform is done by the gather CTA on its columns, then a y pass and
// an x pass that writes the index and absorption volumes.
#include "tdm_internal.cuh"

namespace tdm {
namespace {

template <class K>
cudaError_t allow_smem(K kernel, size_t bytes) {
    if (bytes <= 48 * 1024) return cudaSuccess;
    return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
}

template <int F>
struct CapCfg {
    static constexpr int T = F / 8;
    static constexpr int B = (256 / T) >= 1 ? 256 / T : 1;
};

// fzm0 per angle (fonctions.cpp:893-899); negative when the angle is skipped.
__global__ void k_fzm0(const int2* __restrict__ posspec, int n, int N, double rayon, double* __restrict__ fzm0) {
    const int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= n) return;
    const int fxm0 = posspec[a].x - N, fym0 = posspec[a].y - N;
    const double c = rayon * rayon - fxm0 * fxm0 - fym0 * fym0;
    fzm0[a] = (round(c) >= 0) ? sqrt(c) : -1.0;
}

template <int F>
__global__ void __launch_bounds__(CapCfg<F>::B * (F / 8))
k_cap_rows(const float2* __restrict__ fields, const float* __restrict__ tuk, const float2* __restrict__ tw,
           float2* __restrict__ r1) {
    using C = CapCfg<F>;
    extern __shared__ float2 sm[];
    const int tr = threadIdx.x / C::T, j = threadIdx.x % C::T;
    const int a = blockIdx.y, y = blockIdx.x * C::B + tr;
    float2* s = sm + tr * padded_len(F);
    const float wy = tuk[y];
    const float2* src = fields + ((size_t)a * F + y) * F;
#pragma unroll
    for (int t = 0; t < 8; ++t) {
        const int x = j + t * C::T;
        s[pad_idx(x)] = c_scale(src[x], tuk[x] * wy);
    }
    __syncthreads();
    fft_smem<F, -1>(s, j, tw);
#pragma unroll
    for (int t = 0; t < 8; ++t) {
        const int k = j + t * C::T;
        r1[((size_t)a * F + y) * F + k] = s[pad_idx(k)];
    }
}

template <int F>
__global__ void __launch_bounds__(CapCfg<F>::B * (F / 8))
k_cap_cols(const float2* __restrict__ r1, const int2* __restrict__ posspec, const double* __restrict__ fzm0,
           const double* __restrict__ s_tab, const float* __restrict__ s_tabf, Params p,
           const float2* __restrict__ tw, float2* __restrict__ rec_val, int16_t* __restrict__ rec_z,
           int* __restrict__ err) {
    using C = CapCfg<F>;
    constexpr int B = C::B;
    extern __shared__ float2 sm[];
    const int tr = threadIdx.x / C::T, j = threadIdx.x % C::T;
    const int a = blockIdx.y, kx0 = blockIdx.x * B;
    for (int i = threadIdx.x; i < B * F; i += blockDim.x) {
        const int t = i % B, ky = i / B;
        sm[t * padded_len(F) + pad_idx(ky)] = r1[((size_t)a * F + ky) * F + kx0 + t];
    }
    __syncthreads();
    fft_smem<F, -1>(sm + tr * padded_len(F), j, tw);
    const int2 ps = posspec[a];
    const double fz = fzm0[a];
    const float fzf = (float)fz;
    const int N = p.N;
    for (int i = threadIdx.x; i < B * F; i += blockDim.x) {
        const int t = i % B, ky = i / B, kx = kx0 + t;
        const size_t o = ((size_t)a * F + ky) * F + kx;
        const int fdx = ((kx + ps.x) & (F - 1)) - N, fdy = ((ky + ps.y) & (F - 1)) - N;
        int z = -1;
        if (fz >= 0.0 && fdx * fdx + fdy * fdy < p.disc_thr) {
            const int ti = (fdy + N) * F + fdx + N;
            const float sf = s_tabf[ti];
            const float d = sf - fzf;
            const float fr = d - floorf(d);
            // round(sqrt(fdz^2) - fzm0) in FP64 (fonctions.cpp:921); the FP32
            // value decides unless it lies within 1e-3 of a rounding boundary.
            const float koz = (fabsf(fr - 0.5f) > 1e-3f) ? floorf(d + 0.5f) : (float)round(s_tab[ti] - fz);
            z = (int)koz + p.D / 2;
            if (z < p.zmin || z >= p.zmin + p.band) {
                atomicOr(err, 1);
                z = -1;
            } else {
                float2 v = sm[t * padded_len(F) + pad_idx(ky)];
                const float sg = ((kx + ky) & 1) ? -p.dx2 : p.dx2;
                const float Bc = p.cap_scale * (sf * (float)p.inv_rayon) * sg;  // (k0/pi)(-2pi) sdz dx^2 (+-1)
                rec_val[o] = make_float2(-Bc * v.y, Bc * v.x);
            }
        }
        rec_z[o] = (int16_t)z;
    }
}

// ---------------------------------------------------------------- gather + z inverse FFT
constexpr int kGX = 16, kGY = 8, kGC = kGX * kGY;  // columns per CTA

template <int D>
__global__ void __launch_bounds__(kGC)
k_gather(const float2* __restrict__ rec_val, const int16_t* __restrict__ rec_z, const int2* __restrict__ posspec,
         int M, Params p, double2* __restrict__ acc_all, const float2* __restrict__ tw, float2* __restrict__ vol,
         uint8_t* __restrict__ otf, uint32_t* __restrict__ cnt_out) {
    constexpr int T = D / 8, G = kGC / T;
    extern __shared__ __align__(16) unsigned char smraw[];
    float2* fbuf = reinterpret_cast<float2*>(smraw);                       // G x padded(D)
    int2* sp = reinterpret_cast<int2*>(fbuf + G * padded_len(D));          // M
    uint16_t* cnt = reinterpret_cast<uint16_t*>(sp + M);                   // band x kGC
    const int tid = threadIdx.x, tx = tid % kGX, ty = tid / kGX;
    const int X0 = blockIdx.x * kGX, Y0 = blockIdx.y * kGY;
    const int X = X0 + tx, Y = Y0 + ty;
    const int F = p.F, band = p.band, zmin = p.zmin;
    double2* acc = acc_all + (size_t)(blockIdx.y * gridDim.x + blockIdx.x) * band * kGC;
    for (int i = tid; i < M; i += kGC) sp[i] = posspec[i];
    for (int zb = 0; zb < band; ++zb) {
        acc[zb * kGC + tid] = make_double2(0.0, 0.0);
        cnt[zb * kGC + tid] = 0;
    }
    __syncthreads();
    const int h = D / 2;
    const int kx = (X - h) & (F - 1), ky = (Y - h) & (F - 1);
    const size_t koff = (size_t)ky * F + kx;
    const int bx = X - h, by = Y - h;  // fd + N = X - D/2 + posSpec
    const size_t FF = (size_t)F * F;
    for (int a = 0; a < M; ++a) {
        const int2 q = sp[a];
        const int ux = bx + q.x, uy = by + q.y;  // fd + N
        if ((unsigned)ux < (unsigned)F && (unsigned)uy < (unsigned)F) {
            const size_t idx = (size_t)a * FF + koff;
            const int z = rec_z[idx];
            if (z >= 0) {
                const float2 v = rec_val[idx];
                const int e = (z - zmin) * kGC + tid;
                double2 t = acc[e];
                t.x += (double)v.x;
                t.y += (double)v.y;
                acc[e] = t;
                cnt[e] += 1;
            }
        }
    }
    __syncthreads();
    // OTF mask (Re != 0 after normalisation, main.cpp:262-267) and hit counts
    if (otf || cnt_out) {
        for (int Z = 0; Z < D; ++Z) {
            const int zb = Z - zmin;
            const bool in = zb >= 0 && zb < band;
            const size_t o = ((size_t)Z * D + Y) * D + X;
            if (otf) otf[o] = (in && acc[zb * kGC + tid].x != 0.0) ? 1 : 0;
            if (cnt_out) cnt_out[o] = in ? cnt[zb * kGC + tid] : 0u;
        }
    }
    // normalise, modulate, inverse FFT along z, G columns at a time
    const int tr = tid / T, j = tid % T;
    for (int c0 = 0; c0 < kGC; c0 += G) {
        for (int i = tid; i < G * D; i += kGC) {
            const int g = i % G, Z = i / G, col = c0 + g;
            const int Xc = X0 + col % kGX, Yc = Y0 + col / kGX;
            float2 v = make_float2(0.0f, 0.0f);
            const int zb = Z - zmin;
            if (zb >= 0 && zb < band) {
                const double2 t = acc[zb * kGC + col];
                const unsigned n = cnt[zb * kGC + col];
                const double dn = n ? (double)n : 1.0;
                v = make_float2((float)(t.x / dn), (float)(t.y / dn));
                if ((Xc + Yc + Z) & 1) v = make_float2(-v.x, -v.y);
            }
            fbuf[g * padded_len(D) + pad_idx(Z)] = v;
        }
        __syncthreads();
        fft_smem<D, +1>(fbuf + tr * padded_len(D), j, tw);
        for (int i = tid; i < G * D; i += kGC) {
            const int g = i / D, Z = i % D, col = c0 + g;
            const int Xc = X0 + col % kGX, Yc = Y0 + col / kGX;
            vol[((size_t)Yc * D + Xc) * D + Z] = fbuf[g * padded_len(D) + pad_idx(Z)];
        }
        __syncthreads();
    }
}

template <int D>
struct PassCfg {
    static constexpr int T = D / 8;
    static constexpr int B = (1024 / T) < 16 ? (1024 / T) : 16;
};

// inverse FFT along y, in place, for B consecutive z at fixed x
template <int D>
__global__ void __launch_bounds__(PassCfg<D>::B * (D / 8))
k_ypass(float2* __restrict__ vol, const float2* __restrict__ tw) {
    using C = PassCfg<D>;
    constexpr int B = C::B;
    extern __shared__ float2 sm[];
    const int tr = threadIdx.x / C::T, j = threadIdx.x % C::T;
    const int z0 = blockIdx.x * B, X = blockIdx.y;
    for (int i = threadIdx.x; i < B * D; i += blockDim.x) {
        const int t = i % B, Y = i / B;
        sm[t * padded_len(D) + pad_idx(Y)] = vol[((size_t)Y * D + X) * D + z0 + t];
    }
    __syncthreads();
    fft_smem<D, +1>(sm + tr * padded_len(D), j, tw);
    for (int i = threadIdx.x; i < B * D; i += blockDim.x) {
        const int t = i % B, Y = i / B;
        vol[((size_t)Y * D + X) * D + z0 + t] = sm[t * padded_len(D) + pad_idx(Y)];
    }
}

// inverse FFT along x for B consecutive z at fixed y, scaled and sign-modulated,
// written as the index (real) and absorption (imaginary) volumes, x fastest.
template <int D>
__global__ void __launch_bounds__(PassCfg<D>::B * (D / 8))
k_xpass(const float2* __restrict__ vol, const float2* __restrict__ tw, float scale, float* __restrict__ re,
        float* __restrict__ im) {
    using C = PassCfg<D>;
    constexpr int B = C::B;
    extern __shared__ float2 sm[];
    const int tr = threadIdx.x / C::T, j = threadIdx.x % C::T;
    const int z0 = blockIdx.x * B, Y = blockIdx.y;
    for (int i = threadIdx.x; i < B * D; i += blockDim.x) {
        const int t = i % B, X = i / B;
        sm[t * padded_len(D) + pad_idx(X)] = vol[((size_t)Y * D + X) * D + z0 + t];
    }
    __syncthreads();
    fft_smem<D, +1>(sm + tr * padded_len(D), j, tw);
    const int par = (3 * (D / 2)) & 1;
    for (int i = threadIdx.x; i < B * D; i += blockDim.x) {
        const int t = i / D, X = i % D, Z = z0 + t;
        const float2 v = sm[t * padded_len(D) + pad_idx(X)];
        const float s = ((X + Y + Z + par) & 1) ? -scale : scale;
        const size_t o = ((size_t)Z * D + Y) * D + X;
        if (re) re[o] = v.x * s;
        if (im) im[o] = v.y * s;
    }
}

template <int F>
int cap_impl(tdm_ctx* c, int n) {
    using C = CapCfg<F>;
    Buffers& b = c->b;
    const size_t sm = (size_t)C::B * padded_len(F) * sizeof(float2);
    if (allow_smem(k_cap_rows<F>, sm) || allow_smem(k_cap_cols<F>, sm)) return TDM_ECUDA;
    {
        Launch l(c, K_FZM0);
        k_fzm0<<<(n + 255) / 256, 256, 0, c->stream>>>(b.posspec, n, c->p.N, c->p.rayon, b.fzm0);
    }
    const size_t FF = (size_t)F * F;
    for (int g0 = 0; g0 < n; g0 += c->chunk) {
        const int m = n - g0 < c->chunk ? n - g0 : c->chunk;
        {
            Launch l(c, K_CAP_ROWS);
            k_cap_rows<F><<<dim3(F / C::B, m), C::B * C::T, sm, c->stream>>>(b.fields + g0 * FF, b.tuk_f, b.tw, b.r1);
        }
        {
            Launch l(c, K_CAP_COLS);
            k_cap_cols<F><<<dim3(F / C::B, m), C::B * C::T, sm, c->stream>>>(
                b.r1, b.posspec + g0, b.fzm0 + g0, b.s_tab, b.s_tabf, c->p, b.tw, b.rec_val + g0 * FF,
                b.rec_z + g0 * FF, b.err);
        }
    }
    return cudaGetLastError() == cudaSuccess ? TDM_OK : TDM_ECUDA;
}

template <int D>
int volume_impl(tdm_ctx* c, int n, float* re, float* im, uint8_t* otf, uint32_t* cnt) {
    using P = PassCfg<D>;
    Buffers& b = c->b;
    const Params& p = c->p;
    constexpr int T = D / 8, G = kGC / T;
    const size_t sm_g = (size_t)G * padded_len(D) * sizeof(float2) + (size_t)n * sizeof(int2) +
                        (size_t)p.band * kGC * sizeof(uint16_t);
    const size_t sm_p = (size_t)P::B * padded_len(D) * sizeof(float2);
    if (sm_g > 227 * 1024) return TDM_EUNSUPPORTED;
    if (allow_smem(k_gather<D>, sm_g) || allow_smem(k_ypass<D>, sm_p) || allow_smem(k_xpass<D>, sm_p))
        return TDM_ECUDA;
    cudaEventRecord(c->ev_stage[4], c->stream);
    {
        Launch l(c, K_GATHER);
        k_gather<D><<<dim3(D / kGX, D / kGY), kGC, sm_g, c->stream>>>(b.rec_val, b.rec_z, b.posspec, n, p, b.acc,
                                                                      b.tw, b.vol, otf, cnt);
    }
    cudaEventRecord(c->ev_stage[5], c->stream);
    {
        Launch l(c, K_YPASS);
        k_ypass<D><<<dim3(D / P::B, D), P::B * P::T, sm_p, c->stream>>>(b.vol, b.tw);
    }
    {
        Launch l(c, K_XPASS);
        k_xpass<D><<<dim3(D / P::B, D), P::B * P::T, sm_p, c->stream>>>(b.vol, b.tw, p.out_scale, re, im);
    }
    cudaEventRecord(c->ev_stage[6], c->stream);
    return cudaGetLastError() == cudaSuccess ? TDM_OK : TDM_ECUDA;
}

}  // namespace

int launch_cap(tdm_ctx* c, int n) {
    switch (c->p.F) {
        case 64: return cap_impl<64>(c, n);
        case 128: return cap_impl<128>(c, n);
        case 256: return cap_impl<256>(c, n);
        case 512: return cap_impl<512>(c, n);
        default: return TDM_EUNSUPPORTED;
    }
}

int launch_volume(tdm_ctx* c, int n, float* re, float* im, uint8_t* otf, uint32_t* cnt) {
    switch (c->p.D) {
        case 128: return volume_impl<128>(c, n, re, im, otf, cnt);
        case 256: return volume_impl<256>(c, n, re, im, otf, cnt);
        case 512: return volume_impl<512>(c, n, re, im, otf, cnt);
        case 1024: return volume_impl<1024>(c, n, re, im, otf, cnt);
        default: return TDM_EUNSUPPORTED;
    }
}

int launch_fzm0(tdm_ctx* c, int n) {
    {
        Launch l(c, K_FZM0);
        k_fzm0<<<(n + 255) / 256, 256, 0, c->stream>>>(c->b.posspec, n, c->p.N, c->p.rayon, c->b.fzm0);
    }
    return cudaGetLastError() == cudaSuccess ? TDM_OK : TDM_ECUDA;
}

}  // namespace tdm
