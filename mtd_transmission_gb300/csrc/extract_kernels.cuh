// Off-axis extraction kernels (holo2TF_UBorn, pretraitement_hors_axe_CPU/fonctions.cpp:279-304),
// shared by the context entry points (k_extract.cu) and the allocation-free
// entry point (tdm_noalloc.cu).  See k_extract.cu for the algorithm.
#pragma once

#include "tdm_internal.cuh"
#include "fft_warp.cuh"

namespace tdm {
namespace extract {

// Both passes run on the warp-resident FFT (fft_warp.cuh) in CTAs of 8
// warps.  The row pass packs two real rows into one complex transform and
// keeps the crop's kx band, written column-major (inter[a][c][y]) through a
// shared-memory tile so that each column's 2P rows leave as one contiguous
// segment; the column pass then reads whole columns contiguously and writes
// the crop rows through a second tile (and, on request, the crop's partial
// specular-peak winners, one record per CTA).
template <int H>
struct ExtractCfg {
    using W = WarpFFT<H>;
    static constexpr int NT = 256;         // threads per CTA
    static constexpr int P = 8 * W::G;     // row pairs per CTA (rows pass)
    static constexpr int C = 8 * W::G;     // columns per CTA (cols pass)
    static size_t smem_rows(int F) { return ((size_t)P * W::STRIDE + (size_t)F * (2 * P + 1)) * sizeof(float2); }
    static size_t smem_cols(int F) { return ((size_t)C * W::STRIDE + (size_t)F * (C + 1)) * sizeof(float2); }
    static dim3 grid_rows(int m) { return dim3(H / (2 * P), m); }
    static dim3 grid_cols(int F, int m) { return dim3(F / C, m); }
};

template <int H>
__global__ void __launch_bounds__(ExtractCfg<H>::NT)
k_extract_rows(const void* __restrict__ holos, int bits, const float* __restrict__ tuk,
               const float2* __restrict__ tw, float2* __restrict__ inter, int F, int x0) {
    using Cf = ExtractCfg<H>;
    using W = typename Cf::W;
    constexpr int T = W::T, E = W::E, P = Cf::P, TP = 2 * P + 1;
    extern __shared__ float2 sm[];
    float2* tile = sm + P * W::STRIDE;  // F x TP: [c][row in CTA]
    const int tr = threadIdx.x / T, j = threadIdx.x % T;
    const int a = blockIdx.y;
    const int ya = 2 * (blockIdx.x * P + tr), yb = ya + 1;
    float2* s = sm + tr * W::STRIDE;
    const float wa = tuk[ya], wb = tuk[yb];
    const float sx = (j & 1) ? -1.0f : 1.0f;  // (-1)^x for x = j + T n1, T even; ya even, yb odd
    const size_t base = (size_t)a * H * H;
    float2 x[E];
    if (bits == 16) {
        const uint16_t* ra = static_cast<const uint16_t*>(holos) + base + (size_t)ya * H;
#pragma unroll
        for (int n1 = 0; n1 < E; ++n1) {
            const int xx = j + n1 * T;
            const float w = sx * __ldg(&tuk[xx]);
            x[n1] = make_float2((float)ra[xx] * (w * wa), -(float)ra[H + xx] * (w * wb));
        }
    } else {
        const uint8_t* ra = static_cast<const uint8_t*>(holos) + base + (size_t)ya * H;
#pragma unroll
        for (int n1 = 0; n1 < E; ++n1) {
            const int xx = j + n1 * T;
            const float w = sx * __ldg(&tuk[xx]);
            x[n1] = make_float2((float)ra[xx] * (w * wa), -(float)ra[H + xx] * (w * wb));
        }
    }
    fft_warp_regs<H, -1>(x, s, j, tw);
    __syncwarp();
#pragma unroll
    for (int q = 0; q < E / T; ++q) {
#pragma unroll
        for (int k2 = 0; k2 < T; ++k2) s[warp_out_pos<H>(j, q, k2)] = x[q * T + k2];
    }
    __syncwarp();
    // separate the two real rows on the kx band: Xa = (Z(k) + conj Z(-k))/2, Xb = (Z(k) - conj Z(-k))/(2i)
    for (int c = j; c < F; c += T) {
        const int k = x0 + c, km = (H - k) & (H - 1);
        const float2 z = s[W::pad(k)], zm = s[W::pad(km)];
        tile[c * TP + 2 * tr] = make_float2(0.5f * (z.x + zm.x), 0.5f * (z.y - zm.y));
        tile[c * TP + 2 * tr + 1] = make_float2(0.5f * (z.y + zm.y), -0.5f * (z.x - zm.x));
    }
    __syncthreads();
    float2* dst = inter + (size_t)a * F * H + 2 * blockIdx.x * P;
    for (int i = threadIdx.x; i < F * 2 * P; i += Cf::NT) {
        const int c = i / (2 * P), r = i % (2 * P);
        dst[(size_t)c * H + r] = tile[c * TP + r];
    }
}

template <int H>
__global__ void __launch_bounds__(ExtractCfg<H>::NT)
k_extract_cols(const float2* __restrict__ inter, const float2* __restrict__ tw, float2* __restrict__ spectra,
               int F, int x0, int y0, float2* __restrict__ argpart) {
    using Cf = ExtractCfg<H>;
    using W = typename Cf::W;
    constexpr int T = W::T, E = W::E, C = Cf::C, TC = C + 1;
    extern __shared__ float2 sm[];
    float2* tile = sm + C * W::STRIDE;  // F x TC: [crop row][column in CTA]
    const int tr = threadIdx.x / T, j = threadIdx.x % T;
    const int a = blockIdx.y, c0 = blockIdx.x * C, c = c0 + tr;
    float2* s = sm + tr * W::STRIDE;
    const float2* src = inter + ((size_t)a * F + c) * H;
    float2 x[E];
#pragma unroll
    for (int n1 = 0; n1 < E; ++n1) x[n1] = src[j + n1 * T];
    fft_warp_regs<H, -1>(x, s, j, tw);
    __syncwarp();
#pragma unroll
    for (int q = 0; q < E / T; ++q) {
#pragma unroll
        for (int k2 = 0; k2 < T; ++k2) s[warp_out_pos<H>(j, q, k2)] = x[q * T + k2];
    }
    __syncwarp();
    const float inv = 1.0f / ((float)H * (float)H);
    const int kx = x0 + c;
    for (int r = j; r < F; r += T) {
        const int ky = y0 + r;
        const float sg = ((kx + ky) & 1) ? -inv : inv;
        tile[r * TC + tr] = c_scale(s[W::pad(ky)], sg);
    }
    __syncthreads();
    float2* dst = spectra + (size_t)a * F * F + c0;
    float best = -1.0f;
    int bi = 0x7fffffff;
    for (int i = threadIdx.x; i < F * C; i += Cf::NT) {
        const int r = i / C, t = i % C;
        const float2 z = tile[r * TC + t];
        dst[(size_t)r * F + t] = z;
        if (argpart) argmax_take(best, bi, z, r * F + c0 + t);
    }
    if (argpart) {  // this CTA's partial winner of the specular search (gridDim.x records per angle)
        argmax_block(best, bi);
        if (threadIdx.x == 0) argpart[(size_t)a * gridDim.x + blockIdx.x] = make_float2(best, __int_as_float(bi));
    }
}

}  // namespace extract
}  // namespace tdm
