// Specular-peak search of coordSpec (pretraitement_hors_axe_CPU/fonctions.cpp:88-101):
// |z|^2 at index 0, |z| elsewhere, the first maximum in row-major order wins.
//
// The values are compared in FP32 first.  Partial winners are float4 records
// (value, index bits, runner-up value, 0): merging keeps the larger value
// and, on ties, the smaller index, and carries the largest value that lost,
// so any slicing of the spectrum gives the FP32 answer and the best losing
// value.  The reference compares in FP64.  Where the runner-up lies within
// kArgGuard (relative) of the winner, FP32 rounding may have swapped or tied
// two bins that FP64 separates, so the search is repeated over the bins
// within the guard with the reference's FP64 values (argmax_exact): the same
// rule as the FP64 fallback of the cap-plane decision.  Outside the guard the
// FP32 order is the FP64 order (the FP32 magnitude is within 2 ulp of the
// exact one; the guard is 30 ulp).
#pragma once

#include <cuda_runtime.h>

namespace tdm {

constexpr int kArgSlices = 32;     // slices per spectrum of the standalone partial pass
constexpr int kArgPartsMax = 512;  // partial records (float4) per angle, any producer
constexpr float kArgGuard = 4e-6f; // relative distance below the winner that is re-decided in FP64

__device__ __forceinline__ void argmax_merge(float& best, int& bi, float& second, float ob, int oi, float os) {
    if (ob > best || (ob == best && oi < bi)) {
        second = fmaxf(best, fmaxf(second, os));
        best = ob;
        bi = oi;
    } else {
        second = fmaxf(second, fmaxf(ob, os));
    }
}

// FP32 candidate value of spectrum value z at row-major index i.
__device__ __forceinline__ float argmax_value(float2 z, int i) {
    const float sq = z.x * z.x + z.y * z.y;
    return i == 0 ? sq : sqrtf(sq);
}

// The reference's FP64 value: pow(re,2)+pow(im,2) at index 0, abs(z) elsewhere.
// For FP32 inputs the squares are exact in FP64; the square root of their
// rounded sum is the correctly rounded |z| whenever that sum is exact.
__device__ __forceinline__ double argmax_value64(float2 z, int i) {
    const double x = z.x, y = z.y;
    const double sq = x * x + y * y;
    return i == 0 ? sq : sqrt(sq);
}

__device__ __forceinline__ void argmax_take(float& best, int& bi, float& second, float2 z, int i) {
    argmax_merge(best, bi, second, argmax_value(z, i), i, -1.0f);
}

__device__ __forceinline__ void argmax_warp(float& best, int& bi, float& second) {
#pragma unroll
    for (int off = 16; off > 0; off >>= 1)
        argmax_merge(best, bi, second, __shfl_xor_sync(0xffffffffu, best, off),
                     __shfl_xor_sync(0xffffffffu, bi, off), __shfl_xor_sync(0xffffffffu, second, off));
}

// Winner over the CTA (blockDim.x a multiple of 32, at most 1024); the
// result is valid in thread 0.  Contains __syncthreads().
__device__ __forceinline__ void argmax_block(float& best, int& bi, float& second) {
    __shared__ float sb[32], ss[32];
    __shared__ int si[32];
    argmax_warp(best, bi, second);
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31, nw = blockDim.x >> 5;
    if (l == 0) {
        sb[w] = best;
        si[w] = bi;
        ss[w] = second;
    }
    __syncthreads();
    if (w == 0) {
        best = l < nw ? sb[l] : -1.0f;
        bi = l < nw ? si[l] : 0x7fffffff;
        second = l < nw ? ss[l] : -1.0f;
        argmax_warp(best, bi, second);
    }
}

__device__ __forceinline__ float4 argmax_record(float best, int bi, float second) {
    return make_float4(best, __int_as_float(bi), second, 0.0f);
}

// FP64 decision over the bins whose FP32 value is at least thr (the bins
// within the guard of the FP32 winner), by the whole CTA (blockDim.x a
// multiple of 32); every thread gets the result.  Contains __syncthreads().
static __device__ __noinline__ int argmax_exact(const float2* __restrict__ spec, int n, float thr) {
    __shared__ double sb[32];
    __shared__ int si[32];
    __shared__ int s_res;
    double best = -1.0;
    int bi = 0x7fffffff;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const float2 z = spec[i];
        if (!(argmax_value(z, i) >= thr)) continue;
        const double v = argmax_value64(z, i);
        if (v > best || (v == best && i < bi)) {
            best = v;
            bi = i;
        }
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        const double ob = __shfl_xor_sync(0xffffffffu, best, off);
        const int oi = __shfl_xor_sync(0xffffffffu, bi, off);
        if (ob > best || (ob == best && oi < bi)) {
            best = ob;
            bi = oi;
        }
    }
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31, nw = blockDim.x >> 5;
    if (l == 0) {
        sb[w] = best;
        si[w] = bi;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int k = 1; k < nw; ++k)
            if (sb[k] > best || (sb[k] == best && si[k] < bi)) {
                best = sb[k];
                bi = si[k];
            }
        s_res = bi == 0x7fffffff ? 0 : bi;
    }
    __syncthreads();
    return s_res;
}

// Winner over the nparts partial records of one angle whose spectrum (n
// bins) is spec, computed by the whole CTA (every thread gets the result).
// Contains __syncthreads() when the FP32 decision is within the guard.
__device__ __forceinline__ int argmax_final(const float4* __restrict__ part, int nparts,
                                            const float2* __restrict__ spec, int n) {
    float best = -1.0f, second = -1.0f;
    int bi = 0x7fffffff;
    for (int i = threadIdx.x & 31; i < nparts; i += 32) {
        const float4 q = part[i];
        argmax_merge(best, bi, second, q.x, __float_as_int(q.y), q.z);
    }
    argmax_warp(best, bi, second);
    if (bi == 0x7fffffff) return 0;  // all NaN: the reference keeps index 0
    const float thr = best * (1.0f - kArgGuard);
    if (second >= thr) return argmax_exact(spec, n, thr);  // uniform: every warp merged the same records
    return bi;
}

}  // namespace tdm
