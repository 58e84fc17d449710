// Specular-peak search of coordSpec (pretraitement_hors_axe_CPU/fonctions.cpp:88-101):
// |z|^2 at index 0, |z| elsewhere, the first maximum in row-major order wins.
// Partial winners are (value, index bits) float2 records; merging keeps the
// larger value and, on ties, the smaller index, so any slicing of the
// spectrum gives the reference's answer.
#pragma once

#include <cuda_runtime.h>

namespace tdm {

constexpr int kArgSlices = 32;     // slices per spectrum of the standalone partial pass
constexpr int kArgPartsMax = 512;  // partial records per angle, any producer

__device__ __forceinline__ void argmax_merge(float& best, int& bi, float ob, int oi) {
    if (ob > best || (ob == best && oi < bi)) {
        best = ob;
        bi = oi;
    }
}

// Candidate spectrum value z at row-major index i.
__device__ __forceinline__ void argmax_take(float& best, int& bi, float2 z, int i) {
    const float sq = z.x * z.x + z.y * z.y;
    argmax_merge(best, bi, (i == 0) ? sq : sqrtf(sq), i);
}

__device__ __forceinline__ void argmax_warp(float& best, int& bi) {
#pragma unroll
    for (int off = 16; off > 0; off >>= 1)
        argmax_merge(best, bi, __shfl_xor_sync(0xffffffffu, best, off), __shfl_xor_sync(0xffffffffu, bi, off));
}

// Winner over the CTA (blockDim.x a multiple of 32, at most 1024); the
// result is valid in thread 0.  Contains __syncthreads().
__device__ __forceinline__ void argmax_block(float& best, int& bi) {
    __shared__ float sb[32];
    __shared__ int si[32];
    argmax_warp(best, bi);
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31, nw = blockDim.x >> 5;
    if (l == 0) {
        sb[w] = best;
        si[w] = bi;
    }
    __syncthreads();
    if (w == 0) {
        best = l < nw ? sb[l] : -1.0f;
        bi = l < nw ? si[l] : 0x7fffffff;
        argmax_warp(best, bi);
    }
}

// Winner over the nparts partial records of one angle, computed by every
// warp that calls it (all lanes get the result).
__device__ __forceinline__ int argmax_final(const float2* __restrict__ part, int nparts) {
    float best = -1.0f;
    int bi = 0x7fffffff;
    for (int i = threadIdx.x & 31; i < nparts; i += 32) {
        const float2 q = part[i];
        argmax_merge(best, bi, q.x, __float_as_int(q.y));
    }
    argmax_warp(best, bi);
    return bi == 0x7fffffff ? 0 : bi;  // all NaN: the reference keeps index 0
}

}  // namespace tdm
