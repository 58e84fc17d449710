// Ewald-cap geometry of retroPropag_Born (Reconstruction/src/fonctions.cpp:875-935),
// shared by the cap passes for every field size and by the forward
// operator's sampling.
#pragma once

#include "tdm_internal.cuh"

namespace tdm {

// v mod F for v in [0, 2F) (a bin plus a specular coordinate).
__device__ __forceinline__ int wrap_f(int v, int F) { return v >= F ? v - F : v; }

// fzm0 of an angle (fonctions.cpp:893-899); negative when the angle is skipped.
__device__ __forceinline__ double cap_fzm0(const Params& p, int2 ps) {
    const int fxm0 = ps.x - p.N, fym0 = ps.y - p.N;
    const double c = p.rayon * p.rayon - fxm0 * fxm0 - fym0 * fym0;
    return (round(c) >= 0) ? sqrt(c) : -1.0;
}

// Plane z of the cap cell of FFT bin (kx, ky) of an angle with specular
// position ps and height fz (fonctions.cpp:903-921), or -1 outside the NA
// disc or for a skipped angle; *sf is sqrt(r^2 - fd^2) in float for the
// cell's weight.  A plane outside the cap band sets *err and gives -1.
// fzf = (float)fz, converted once by the caller: FP64 instructions run at a
// small fraction of the FP32 rate on this GPU, so the per-bin path is FP32
// and FP64 is used only in the rare rounding-boundary branch.
// The plane of cap pixel fd = (fdx, fdy) (|fd|^2 below the disc threshold)
// for an angle of height fz (fzf = (float)fz); fz_of() gives fz in FP64, and
// is called only near a rounding boundary.  -1 (and *err set) when the plane
// lies outside the cap band.
template <class FzOf>
__device__ __forceinline__ int cap_plane_fd(const Params& p, int fdx, int fdy, float fzf, FzOf&& fz_of,
                                            const double* __restrict__ s_tab, const float* __restrict__ s_tabf,
                                            float* sf, int* __restrict__ err) {
    const int F = p.F, N = p.N;
    const int ti = (fdy + N) * F + fdx + N;
    // sqrt(r^2 - fd^2) in float: computed from the exact integer when r^2 < 2^24 (equal to the table)
    *sf = p.r2i ? __fsqrt_rn((float)(p.r2i - fdx * fdx - fdy * fdy)) : s_tabf[ti];
    const float d = *sf - fzf;
    const float fr = d - floorf(d);
    // round(sqrt(fdz^2) - fzm0) in FP64 (fonctions.cpp:921); the FP32 value
    // decides unless it lies within 1e-3 of a rounding boundary.
    float koz;
    if (fabsf(fr - 0.5f) > 1e-3f) {
        koz = floorf(d + 0.5f);
    } else {
        koz = (float)round(s_tab[ti] - fz_of());
    }
    const int z = (int)koz + p.D / 2;
    if (z < p.zmin || z >= p.zmin + p.band) {
        if (err) atomicOr(err, 1);
        return -1;
    }
    return z;
}

__device__ __forceinline__ int cap_plane(const Params& p, int2 ps, double fz, float fzf, int kx, int ky,
                                         const double* __restrict__ s_tab, const float* __restrict__ s_tabf,
                                         float* sf, int* __restrict__ err) {
    const int F = p.F, N = p.N;
    const int fdx = wrap_f(kx + ps.x, F) - N, fdy = wrap_f(ky + ps.y, F) - N;
    if (!(fzf >= 0.0f) || fdx * fdx + fdy * fdy >= p.disc_thr) return -1;  // fz is sqrt(c) >= 0 or -1
    return cap_plane_fd(p, fdx, fdy, fzf, [&] { return fz; }, s_tab, s_tabf, sf, err);
}

// Cap-cell weight (k0/pi)(-2pi) sdz dx^2 (-1)^(kx+ky) of retroPropag_Born
// (fonctions.cpp:902,927) with the recentring sign of the per-field spectrum.
// ir = (float)p.inv_rayon, converted once by the caller.
__device__ __forceinline__ float cap_weight(const Params& p, float sf, float ir, int kx, int ky) {
    const float sg = ((kx + ky) & 1) ? -p.dx2 : p.dx2;
    return p.cap_scale * (sf * ir) * sg;
}

// Voxel column of FFT bin kx of an angle with specular coordinate q (x or y):
// D/2 + fd + N - q, the inverse of the gather's bin (X - D/2) mod F.
__device__ __forceinline__ int cap_col(const Params& p, int k, int q) {
    return p.D / 2 + wrap_f(k + q, p.F) - q;
}

}  // namespace tdm
