// Mean of an angle's wrapped phase for the Volkov unwrap, from per-CTA sums
// left by the field column pass (k_fields.cu, k_generic.cu): the solve for
// the phasor's gradient returns the unwrapped phase less its mean.
#pragma once

#include "tdm_internal.cuh"

namespace tdm {

// The CTA's sum of the per-thread values v into *out: a shuffle tree per
// warp, then the warps' sums in FP64 in warp order, so the result does not
// depend on timing.  Every thread of the CTA calls it.
template <int NT>
__device__ __forceinline__ void phase_sum_cta(float v, double* out) {
    __shared__ float red[NT / 32];
#pragma unroll
    for (int off = 16; off; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int k = 0; k < NT / 32; ++k) t += red[k];
        *out = t;
    }
}

// The mean of an F x F wrapped phase from its nps sums (psum: the angle's first sum).
__device__ __forceinline__ float phase_mean(const double* __restrict__ psum, int nps, int F) {
    double t = 0.0;
    for (int k = 0; k < nps; ++k) t += psum[k];
    return (float)(t / ((double)F * (double)F));
}

}  // namespace tdm
