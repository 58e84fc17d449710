// Off-axis extraction (holo2TF_UBorn, pretraitement_hors_axe_CPU/fonctions.cpp:279-304).
//
// The reference multiplies the hologram by a Tukey window, fftshifts it, takes
// the 2D FFT divided by H^2, fftshifts the spectrum and copies out the
// F x F crop at (CIRCLE_CX-N, CIRCLE_CY-N).  For even H both fftshifts are
// sign modulations:
//     crop[ky][kx] = (-1)^(kx+ky) / H^2 * FFT2((-1)^(x+y) w(x) w(y) h)[ky][kx]
// with (kx, ky) in the crop window.  The row pass packs two real rows into one
// complex FFT and keeps only the crop's kx band; the column pass transforms
// only those F columns and keeps only the crop's ky rows.  Kernels in
// extract_kernels.cuh.
#include "extract_kernels.cuh"

namespace tdm {
namespace {

using namespace extract;

template <class K>
cudaError_t allow_smem(K kernel, size_t bytes) {
    return max_dynamic_smem(reinterpret_cast<const void*>(kernel), bytes);
}

template <int H>
int extract_impl(tdm_ctx* c, const void* holos, int bits, int n, int a0, bool argmax) {
    using C = ExtractCfg<H>;
    const Params& p = c->p;
    const size_t sm_rows = C::smem_rows(p.F), sm_cols = C::smem_cols(p.F);
    if (!window_edge_ok(H, c->tuk_h_flat, win_edge<H>())) return TDM_EUNSUPPORTED;
    if (allow_smem(k_extract_rows<H, true>, sm_rows) != cudaSuccess) return TDM_ECUDA;
    if (allow_smem(k_extract_rows<H, false>, sm_rows) != cudaSuccess) return TDM_ECUDA;
    if (allow_smem(k_extract_cols<H>, sm_cols) != cudaSuccess) return TDM_ECUDA;
    // bulk staging of the rows needs a 16-byte aligned stack (rows are multiples of 16 bytes)
    const bool bulk = (reinterpret_cast<uintptr_t>(holos) & 15) == 0;
    auto rows = bulk ? k_extract_rows<H, true> : k_extract_rows<H, false>;
    const size_t bytes_per = (size_t)H * H * (bits == 16 ? 2 : 1);
    for (int h0 = 0; h0 < n; h0 += c->holo_chunk) {
        const int m = n - h0 < c->holo_chunk ? n - h0 : c->holo_chunk;
        const char* src = static_cast<const char*>(holos) + (size_t)h0 * bytes_per;
        {
            Launch l(c, K_EXTRACT_ROWS);
            rows<<<C::grid_rows(m), C::NT, sm_rows, c->stream>>>(src, bits, c->b.win_h,
                                                                c->use_ref ? c->b.ref_inv : nullptr, c->b.tw,
                                                                c->b.inter, p.F, p.x0, c->b.err, c->wait_polls);
        }
        {
            Launch l(c, K_EXTRACT_COLS);
            k_extract_cols<H><<<C::grid_cols(p.F, m), C::NT, sm_cols, c->stream>>>(
                c->b.inter, c->b.tw, c->b.spectra + (size_t)(a0 + h0) * p.F * p.F, p.F, p.x0, p.y0,
                argmax ? c->b.argpart : nullptr);
        }
    }
    if (cudaGetLastError() != cudaSuccess) return TDM_ECUDA;
    return argmax ? (int)C::grid_cols(p.F, 1).x * (C::NT / 32) : TDM_OK;
}

}  // namespace

int launch_extract(tdm_ctx* c, const void* holos, int bits, int n, int a0, bool argmax) {
    if (argmax && (n > c->holo_chunk || n > c->chunk)) return TDM_EINVAL;  // partials of one chunk only
    switch (c->p.H) {
        case 256: return extract_impl<256>(c, holos, bits, n, a0, argmax);
        case 512: return extract_impl<512>(c, holos, bits, n, a0, argmax);
        case 1024: return extract_impl<1024>(c, holos, bits, n, a0, argmax);
        case 2048: return extract_impl<2048>(c, holos, bits, n, a0, argmax);
        default: return TDM_EUNSUPPORTED;
    }
}

}  // namespace tdm
