// Off-axis extraction kernels (holo2TF_UBorn, pretraitement_hors_axe_CPU/fonctions.cpp:279-304),
// shared by the context entry points (k_extract.cu) and the allocation-free
// entry point (tdm_noalloc.cu).  See k_extract.cu for the algorithm.
#pragma once

#include "tdm_internal.cuh"

namespace tdm {
namespace extract {

template <int H>
struct ExtractCfg {
    static constexpr int T = H / 8;                        // threads per transform
    static constexpr int PAIRS = H >= 2048 ? 2 : 4;        // row pairs per CTA (rows pass)
    static constexpr int COLS = (1024 / T) < 16 ? (1024 / T) : 16;  // columns per CTA (cols pass)
};

template <int H>
__global__ void __launch_bounds__(ExtractCfg<H>::PAIRS * (H / 8))
k_extract_rows(const void* __restrict__ holos, int bits, const float* __restrict__ tuk,
               const float2* __restrict__ tw, float2* __restrict__ inter, int F, int x0) {
    using C = ExtractCfg<H>;
    extern __shared__ float2 sm[];
    const int pr = threadIdx.x / C::T, j = threadIdx.x % C::T;
    const int a = blockIdx.y;
    const int ya = 2 * (blockIdx.x * C::PAIRS + pr), yb = ya + 1;
    float2* s = sm + pr * tstride(H);
    const size_t base = (size_t)a * H * H;
    const float wa = tuk[ya], wb = tuk[yb];
#pragma unroll
    for (int t = 0; t < 8; ++t) {
        const int x = j + t * C::T;
        float ha, hb;
        if (bits == 16) {
            const uint16_t* h = static_cast<const uint16_t*>(holos) + base;
            ha = (float)h[(size_t)ya * H + x];
            hb = (float)h[(size_t)yb * H + x];
        } else {
            const uint8_t* h = static_cast<const uint8_t*>(holos) + base;
            ha = (float)h[(size_t)ya * H + x];
            hb = (float)h[(size_t)yb * H + x];
        }
        const float w = (x & 1) ? -tuk[x] : tuk[x];   // (-1)^x w(x); ya even, yb odd
        s[pad_idx(x)] = make_float2(ha * (w * wa), -hb * (w * wb));
    }
    __syncthreads();
    fft_smem<H, -1>(s, j, tw);
    // separate the two real rows on the kx band: Xa = (Z(k) + conj Z(-k))/2, Xb = (Z(k) - conj Z(-k))/(2i)
    for (int c = j; c < F; c += C::T) {
        const int k = x0 + c, km = (H - k) & (H - 1);
        const float2 z = s[pad_idx(k)], zm = s[pad_idx(km)];
        const float2 xa = make_float2(0.5f * (z.x + zm.x), 0.5f * (z.y - zm.y));
        const float2 xb = make_float2(0.5f * (z.y + zm.y), -0.5f * (z.x - zm.x));
        inter[((size_t)a * H + ya) * F + c] = xa;
        inter[((size_t)a * H + yb) * F + c] = xb;
    }
}

template <int H>
__global__ void __launch_bounds__(ExtractCfg<H>::COLS * (H / 8))
k_extract_cols(const float2* __restrict__ inter, const float2* __restrict__ tw, float2* __restrict__ spectra,
               int F, int x0, int y0) {
    using C = ExtractCfg<H>;
    extern __shared__ float2 sm[];
    constexpr int B = C::COLS;
    const int a = blockIdx.y;
    constexpr int NT = B * C::T;
    const int c0 = blockIdx.x * B;
    const int tr = threadIdx.x / C::T, j = threadIdx.x % C::T;
#pragma unroll
    for (int r = 0; r < B * H / NT; ++r) {
        const int i = threadIdx.x + r * NT, t = i % B, y = i / B;
        sm[t * tstride(H) + pad_idx(y)] = inter[((size_t)a * H + y) * F + c0 + t];
    }
    __syncthreads();
    fft_smem<H, -1>(sm + tr * tstride(H), j, tw);
    const float inv = 1.0f / ((float)H * (float)H);
    for (int i = threadIdx.x; i < B * F; i += blockDim.x) {
        const int t = i % B, r = i / B;
        const int ky = y0 + r, kx = x0 + c0 + t;
        const float sg = ((kx + ky) & 1) ? -inv : inv;
        spectra[((size_t)a * F + r) * F + c0 + t] = c_scale(sm[t * tstride(H) + pad_idx(ky)], sg);
    }
}

}  // namespace extract
}  // namespace tdm
