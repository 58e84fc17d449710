// Off-axis extraction (holo2TF_UBorn, pretraitement_hors_axe_CPU/fonctions.cpp:279-304).
//
// The reference multiplies the hologram by a Tukey window, fftshifts it, takes
// the 2D FFT divided by H^2, fftshifts the spectrum and copies out the
// F x F crop at (CIRCLE_CX-N, CIRCLE_CY-N).  For even H both fftshifts are
// sign modulations:
//     crop[ky][kx] = (-1)^(kx+ky) / H^2 * FFT2((-1)^(x+y) w(x) w(y) h)[ky][kx]
// with (kx, ky) in the crop window.  The row pass packs two real rows into one
// complex FFT and keeps only the crop's kx band; the column pass transforms
// only those F columns and keeps only the crop's ky rows.
#include "tdm_internal.cuh"

namespace tdm {
namespace {

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
    float2* s = sm + pr * padded_len(H);
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
    const int c0 = blockIdx.x * B;
    const int tr = threadIdx.x / C::T, j = threadIdx.x % C::T;
    for (int i = threadIdx.x; i < B * H; i += blockDim.x) {
        const int t = i % B, y = i / B;
        sm[t * padded_len(H) + pad_idx(y)] = inter[((size_t)a * H + y) * F + c0 + t];
    }
    __syncthreads();
    fft_smem<H, -1>(sm + tr * padded_len(H), j, tw);
    const float inv = 1.0f / ((float)H * (float)H);
    for (int i = threadIdx.x; i < B * F; i += blockDim.x) {
        const int t = i % B, r = i / B;
        const int ky = y0 + r, kx = x0 + c0 + t;
        const float sg = ((kx + ky) & 1) ? -inv : inv;
        spectra[((size_t)a * F + r) * F + c0 + t] = c_scale(sm[t * padded_len(H) + pad_idx(ky)], sg);
    }
}

template <class K>
cudaError_t allow_smem(K kernel, size_t bytes) {
    if (bytes <= 48 * 1024) return cudaSuccess;
    return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
}

template <int H>
int extract_impl(tdm_ctx* c, const void* holos, int bits, int n, int a0) {
    using C = ExtractCfg<H>;
    const Params& p = c->p;
    const size_t sm_rows = (size_t)C::PAIRS * padded_len(H) * sizeof(float2);
    const size_t sm_cols = (size_t)C::COLS * padded_len(H) * sizeof(float2);
    if (allow_smem(k_extract_rows<H>, sm_rows) != cudaSuccess) return TDM_ECUDA;
    if (allow_smem(k_extract_cols<H>, sm_cols) != cudaSuccess) return TDM_ECUDA;
    const size_t bytes_per = (size_t)H * H * (bits == 16 ? 2 : 1);
    for (int h0 = 0; h0 < n; h0 += c->holo_chunk) {
        const int m = n - h0 < c->holo_chunk ? n - h0 : c->holo_chunk;
        const char* src = static_cast<const char*>(holos) + (size_t)h0 * bytes_per;
        {
            Launch l(c, K_EXTRACT_ROWS);
            k_extract_rows<H><<<dim3(H / 2 / C::PAIRS, m), C::PAIRS * C::T, sm_rows, c->stream>>>(
                src, bits, c->b.tuk_h, c->b.tw, c->b.inter, p.F, p.x0);
        }
        {
            Launch l(c, K_EXTRACT_COLS);
            k_extract_cols<H><<<dim3(p.F / C::COLS, m), C::COLS * C::T, sm_cols, c->stream>>>(
                c->b.inter, c->b.tw, c->b.spectra + (size_t)(a0 + h0) * p.F * p.F, p.F, p.x0, p.y0);
        }
    }
    return cudaGetLastError() == cudaSuccess ? TDM_OK : TDM_ECUDA;
}

}  // namespace

int launch_extract(tdm_ctx* c, const void* holos, int bits, int n, int a0) {
    switch (c->p.H) {
        case 256: return extract_impl<256>(c, holos, bits, n, a0);
        case 512: return extract_impl<512>(c, holos, bits, n, a0);
        case 1024: return extract_impl<1024>(c, holos, bits, n, a0);
        case 2048: return extract_impl<2048>(c, holos, bits, n, a0);
        default: return TDM_EUNSUPPORTED;
    }
}

}  // namespace tdm
