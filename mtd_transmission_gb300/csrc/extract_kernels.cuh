// Off-axis extraction kernels (holo2TF_UBorn, pretraitement_hors_axe_CPU/fonctions.cpp:279-304),
// shared by the context entry points (k_extract.cu) and the allocation-free
// entry point (tdm_noalloc.cu).  See k_extract.cu for the algorithm.
#pragma once

#include "tdm_internal.cuh"
#include "fft_warp.cuh"
#include "bulk_copy.cuh"

namespace tdm {
namespace extract {

// Both passes run on the warp-resident FFT (fft_warp.cuh) in CTAs of 8
// warps.  The row pass packs two real rows into one complex transform and
// keeps the crop's kx band, written column-major (inter[a][c][y]): the two
// rows' values of one column are one 16-byte word, and the CTA's row pairs
// fill one segment of each column, stored whole from a shared-memory tile
// (16-byte pieces of distinct lines, one per lane, would cost the L1 a
// wavefront each and L2 a partial-sector write).  The column pass
// then reads whole columns contiguously and writes the crop rows through a
// shared-memory tile (and, on request, the crop's partial specular-peak
// winners, one record per warp).
template <int H>
struct ExtractCfg {
    using W = WarpFFT<H>;
    static constexpr int NT = 256;         // threads per CTA
    static constexpr int P = 8 * W::G;     // row pairs per CTA (rows pass)
    static constexpr int C = 8 * W::G;     // columns per CTA (cols pass)
    // row-pass CTAs per SM that the registers are capped for (shared memory
    // would allow 3 up to H = 1024, but capping to 80 registers for them
    // spills and measured slower than 2)
    static constexpr int ROWS_CTAS = H >= 2048 ? 1 : 2;
    // band columns per round of the row pass's output tile (CB x (P + 1)
    // 16-byte words, about 18 KB; the odd stride keeps both its column-wise
    // fill and its row-wise drain free of bank conflicts)
    static constexpr int CB = 1024 / P;
    static size_t smem_rows(int) {
        return (size_t)P * W::STRIDE * sizeof(float2) + (size_t)CB * (P + 1) * sizeof(float4);
    }
    static size_t smem_cols(int F) { return ((size_t)C * W::STRIDE + (size_t)F * (C + 1)) * sizeof(float2); }
    static dim3 grid_rows(int m) { return dim3(H / (2 * P), m); }
    static dim3 grid_cols(int F, int m) { return dim3((F + C - 1) / C, m); }
};

// Lanes' elements n1 whose pixels x = j + T n1 can fall in the hologram
// window's tapers: the first and the last win_edge of the E.  The window
// (Tukey, alpha 0.05) is exactly 1 on the others; window_edge_ok checks that
// on the host before a launch.
template <int H>
constexpr int win_edge() { return H >= 2048 ? 2 : 1; }
inline bool window_edge_ok(int H, int2 flat, int edge) {
    const int T = H / warp_fft_e(H);
    return flat.x <= T * edge && flat.y >= H - T * edge - 1;
}

// Row pass.  win[x] = ((-1)^x w(x), -2^23 (-1)^x w(x)) is the hologram window
// with the sign modulation of the first fftshift (hologram_window): a pixel p
// is read as the float m = 2^23 + p (its bits OR 0x4B000000) and fma(m, ws,
// cs) is p (-1)^x w(x) rounded once, with no integer-to-float conversion.  On
// the window's flat middle (-1)^x = (-1)^j, so the lane's own (+-1, -+2^23)
// stands for the table there.  The rows' factors (-1)^y w(y) are applied when
// the two packed rows are separated.  ref_inv (may be null) is the H x H
// reciprocal of the reference amplitude, applied to every pixel
// (main.cpp:147).  BULK: each warp's 2G rows (its G row pairs, consecutive in
// memory) are staged in shared memory by one bulk copy and read from there;
// requires a 16-byte aligned stack.  Otherwise the lanes load the pixels
// directly.  A bulk copy that does not complete within wait_polls polls sets
// bit 1 of *err (the call then fails); the warp then waits for its copy again,
// up to the full bound kMbarPolls, so that no copy is left in flight into the
// shared memory of a finished CTA.
template <int H, bool BULK>
__global__ void __launch_bounds__(ExtractCfg<H>::NT, ExtractCfg<H>::ROWS_CTAS)
k_extract_rows(const void* __restrict__ holos, int bits, const float2* __restrict__ win,
               const float* __restrict__ ref_inv, const float2* __restrict__ tw, float2* __restrict__ inter, int F,
               int x0, int* __restrict__ err, uint32_t wait_polls) {
    using Cf = ExtractCfg<H>;
    using W = typename Cf::W;
    constexpr int T = W::T, E = W::E, P = Cf::P, K = win_edge<H>();
    extern __shared__ __align__(16) float2 sm[];
    const int tr = threadIdx.x / T, j = threadIdx.x % T;
    const int a = blockIdx.y;
    const int ya = 2 * (blockIdx.x * P + tr), yb = ya + 1;
    float2* s = sm + tr * W::STRIDE;
    const float ha = 0.5f * __ldg(&win[ya]).x, hb = 0.5f * __ldg(&win[yb]).x;  // (-1)^y w(y) / 2
    const float2 flat = (j & 1) ? make_float2(-1.0f, 8388608.0f) : make_float2(1.0f, -8388608.0f);
    const size_t bpp = bits == 16 ? 2 : 1;
    float2 x[E];
    // windowed pixels of rows ya (real part) and yb (imaginary part)
    auto put = [&](int n1, uint32_t pa, uint32_t pb) {
        const float2 wc = (n1 < K || n1 >= E - K) ? __ldg(&win[j + n1 * T]) : flat;
        x[n1] = make_float2(fmaf(__uint_as_float(0x4B000000u | pa), wc.x, wc.y),
                            fmaf(__uint_as_float(0x4B000000u | pb), wc.x, wc.y));
    };
    auto load = [&](const char* row) {
        if (bits == 16) {
            const uint16_t* ra = reinterpret_cast<const uint16_t*>(row);
#pragma unroll
            for (int n1 = 0; n1 < E; ++n1) put(n1, ra[j + n1 * T], ra[H + j + n1 * T]);
        } else {
            const uint8_t* ra = reinterpret_cast<const uint8_t*>(row);
#pragma unroll
            for (int n1 = 0; n1 < E; ++n1) put(n1, ra[j + n1 * T], ra[H + j + n1 * T]);
        }
        if (ref_inv) {  // pixel / reference amplitude (it scales each product)
            const float* qa = ref_inv + (size_t)ya * H;
#pragma unroll
            for (int n1 = 0; n1 < E; ++n1) {
                const int xx = j + n1 * T;
                x[n1] = make_float2(x[n1].x * __ldg(&qa[xx]), x[n1].y * __ldg(&qa[H + xx]));
            }
        }
    };
    if constexpr (BULK) {
        __shared__ uint64_t bar[Cf::NT / 32];
        const int w = threadIdx.x >> 5;
        static_assert(2 * W::G * H * 2 + 8 <= W::STRIDE * 8, "staged rows fit the first array");
        // the warp's rows land at the first 16-byte boundary of its first
        // transform's array (8 (H + E + 1) bytes, so 2G H bpp + 8 fit), which
        // the transforms overwrite only after all lanes have read their pixels
        // (the first exchange follows a __syncwarp); the pointer is formed by
        // arithmetic on sm (no integer round trip), so the reads stay
        // shared-memory loads
        float2* const first = sm + (w * W::G) * W::STRIDE;
        char* stage = reinterpret_cast<char*>(first) + ((16u - (smem_addr(first) & 15u)) & 15u);
        if ((threadIdx.x & 31) == 0) {
            const uint32_t bytes = (uint32_t)(2 * W::G * H * bpp);
            const size_t y0w = 2 * ((size_t)blockIdx.x * P + w * W::G);
            mbar_init(&bar[w]);
            mbar_expect_tx(&bar[w], bytes);
            bulk_g2s(stage, static_cast<const char*>(holos) + ((size_t)a * H * H + y0w * H) * bpp, bytes, &bar[w]);
        }
        __syncwarp();
        if (!mbar_wait(&bar[w], 0, wait_polls)) {
            if ((threadIdx.x & 31) == 0) atomicOr(err, 2);
            mbar_wait(&bar[w], 0);
        }
        load(stage + (size_t)(tr - w * W::G) * 2 * H * bpp);
    } else {
        load(static_cast<const char*>(holos) + ((size_t)a * H * H + (size_t)ya * H) * bpp);
    }
    fft_warp_regs<H, -1>(x, s, j, tw);
    __syncwarp();
#pragma unroll
    for (int q = 0; q < E / T; ++q) {
#pragma unroll
        for (int k2 = 0; k2 < T; ++k2) s[warp_out_pos<H>(j, q, k2)] = x[q * T + k2];
    }
    __syncwarp();
    // separate the two real rows on the kx band: Xa = (Z(k) + conj Z(-k))/2, Xb = (Z(k) - conj Z(-k))/(2i),
    // times the rows' window factors;
    // rows ya (even) and yb = ya + 1 of column c are adjacent in inter (one
    // 16-byte word), and the CTA's P row pairs are one 16P-byte segment of
    // each column.  The words go through the tile, CB columns at a time, so
    // that each column segment is written by consecutive lanes (whole lines)
    // rather than as 16-byte pieces of distinct lines.
    float4* tile = reinterpret_cast<float4*>(sm + P * W::STRIDE);
    float4* dst = reinterpret_cast<float4*>(inter + (size_t)a * F * H + 2 * blockIdx.x * P);
    for (int cb = 0; cb < F; cb += Cf::CB) {
        const int nc = min(Cf::CB, F - cb);
        for (int c = j; c < nc; c += T) {
            const int k = x0 + cb + c, km = (H - k) & (H - 1);
            const float2 z = s[W::pad(k)], zm = s[W::pad(km)];
            tile[c * (P + 1) + tr] = make_float4(ha * (z.x + zm.x), ha * (z.y - zm.y), hb * (z.y + zm.y),
                                                 -hb * (z.x - zm.x));
        }
        __syncthreads();
        for (int i = threadIdx.x; i < nc * P; i += Cf::NT) {
            const int c = i / P, p = i % P;
            dst[(size_t)(cb + c) * (H / 2) + p] = tile[c * (P + 1) + p];
        }
        if (cb + Cf::CB < F) __syncthreads();  // the tile is refilled
    }
}

template <int H>
__global__ void __launch_bounds__(ExtractCfg<H>::NT)
k_extract_cols(const float2* __restrict__ inter, const float2* __restrict__ tw, float2* __restrict__ spectra,
               int F, int x0, int y0, float4* __restrict__ argpart) {
    using Cf = ExtractCfg<H>;
    using W = typename Cf::W;
    constexpr int T = W::T, E = W::E, C = Cf::C, TC = C + 1;
    extern __shared__ __align__(16) float2 sm[];
    float2* tile = sm + C * W::STRIDE;  // F x TC: [crop row][column in CTA]
    const int tr = threadIdx.x / T, j = threadIdx.x % T;
    const int a = blockIdx.y, c0 = blockIdx.x * C, c = c0 + tr;
    const bool valid = c < F;  // the crop width need not be a multiple of C
    float2* s = sm + tr * W::STRIDE;
    const float2* src = inter + ((size_t)a * F + c) * H;
    float2 x[E];
#pragma unroll
    for (int n1 = 0; n1 < E; ++n1) x[n1] = valid ? src[j + n1 * T] : make_float2(0.f, 0.f);
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
    float best = -1.0f, second = -1.0f;
    int bi = 0x7fffffff;
    for (int r = j; r < F; r += T) {
        const int ky = y0 + r;
        const float sg = ((kx + ky) & 1) ? -inv : inv;
        const float2 z = c_scale(s[W::pad(ky)], sg);
        tile[r * TC + tr] = z;
        if (argpart && valid) argmax_take(best, bi, second, z, r * F + c);
    }
    if (argpart) {  // this warp's partial winner of the specular search (8 records per CTA)
        argmax_warp(best, bi, second);
        if ((threadIdx.x & 31) == 0)
            argpart[((size_t)a * gridDim.x + blockIdx.x) * 8 + (threadIdx.x >> 5)] = argmax_record(best, bi, second);
    }
    __syncthreads();
    float2* dst = spectra + (size_t)a * F * F + c0;
    for (int i = threadIdx.x; i < F * C; i += Cf::NT) {
        const int r = i / C, t = i % C;
        if (c0 + t < F) dst[(size_t)r * F + t] = tile[r * TC + t];
    }
}

}  // namespace extract
}  // namespace tdm
