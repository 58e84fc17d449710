// Field formation from the unwrapped phase, the amplitude and the two
// degree-4 aberration fits (aberCorr2 / ampliCorr2,
// pretraitement_hors_axe_CPU/Correction_aberration.cpp:166-217, and the
// Born/Rytov formation of pretraitement_hors_axe_CPU/main.cpp:289-316).
// Shared by the field stage (k_form) and the cap row pass that forms the
// field on the fly (k_cap_rows_form), with the same operation order.
#pragma once

#include "tdm_internal.cuh"

namespace tdm {

// The fits at image row y reduced to polynomials in u: c[px] = sum_py b_k v^py
// (monomial coefficients bf[0..kNC) for the phase, bf[kNC..2 kNC) for the
// amplitude, in scaled coordinates u, v in [-1, 1]).
struct FormRow {
    float cp[5], ca[5];
};

__device__ __forceinline__ float form_scaled(int i, int F) {
    const float h = 0.5f * (float)(F - 1);
    return ((float)i - h) / h;
}

__device__ __forceinline__ FormRow form_row(const float* bf, int y, int F) {
    const float v = form_scaled(y, F);
    FormRow r;
    int k = 0;
#pragma unroll
    for (int px = 0; px <= 4; ++px) {
        float pp = 0.0f, pa = 0.0f, vp = 1.0f;
#pragma unroll
        for (int py = 0; px + py <= 4; ++py) {
            pp = fmaf(bf[k], vp, pp);
            pa = fmaf(bf[kNC + k], vp, pa);
            vp *= v;
            ++k;
        }
        r.cp[px] = pp;
        r.ca[px] = pa;
    }
    return r;
}

// Corrected phase and amplitude at column x of the row, then the Born
// (A e^{i phi} - 1) or Rytov (log A + i phi) field.
__device__ __forceinline__ float2 form_value(const FormRow& r, int x, int F, float unwrapped, float amp, int born) {
    const float u = form_scaled(x, F);
    float sp = 0.0f, sa = 0.0f, up = 1.0f;
#pragma unroll
    for (int px = 0; px <= 4; ++px) {
        sp = fmaf(r.cp[px], up, sp);
        sa = fmaf(r.ca[px], up, sa);
        up *= u;
    }
    const float pf = unwrapped - sp;
    float af = amp / (sa + 0.00000001f);
    if (af > 10.0f) af = 1.0f;
    if (af < -10.0f) af = 1.0f;
    const float m = fabsf(af);  // sqrt(A^2)
    if (born) {
        float sn, cs;
        sincosf(pf, &sn, &cs);
        return make_float2(m * cs - 1.0f, m * sn);
    }
    return make_float2(logf(m), pf);
}

}  // namespace tdm
