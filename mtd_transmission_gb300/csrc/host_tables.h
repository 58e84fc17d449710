// Host-side tables shared by the entry points.
#pragma once

#include <cmath>
#include <cstdint>
#include <vector>

#include "fft_core.cuh"

namespace tdm {

// Twiddle table uploaded to the device: exp(-2 pi i k / kTwN) for k < kTwN,
// then, for each warp-FFT size N = 64 .. 2048 at offset twr_offset(N), the
// factors exp(-2 pi i j k1 / N) laid out [k1][j] for k1 < E(N), j < T(N),
// so that the T lanes of a transform read consecutive entries.  Computed in
// long double and rounded once to float.
inline std::vector<float2> twiddle_table() {
    const long double two_pi = 2.0L * 3.14159265358979323846264338327950288L;
    std::vector<float2> tw(kTwTotal);
    for (int k = 0; k < kTwN; ++k) {
        const long double a = -two_pi * k / kTwN;
        tw[k] = make_float2((float)std::cos(a), (float)std::sin(a));
    }
    for (int n = 64; n <= 2048; n *= 2) {
        const int e = warp_fft_e(n), t = n / e;
        for (int k1 = 0; k1 < e; ++k1)
            for (int j = 0; j < t; ++j) {
                const long double a = -two_pi * (long double)((j * k1) % n) / n;
                tw[twr_offset(n) + k1 * t + j] = make_float2((float)std::cos(a), (float)std::sin(a));
            }
    }
    return tw;
}

// Tukey window factor, same float arithmetic as tukey2D
// (pretraitement_hors_axe_CPU/FFT_fonctions.cpp:61-87): the 2D window is the
// product of this factor along x and along y.
inline std::vector<double> tukey_factor(int n, float alpha) {
    std::vector<double> t(n, 0.0);
    const int b1 = (int)std::round(alpha * (n - 1) / 2);
    const int b2 = (int)std::round((n - 1) * (1 - alpha / 2));
    for (int i = 0; i < b1 + 1 && i < n; ++i) {
        const float arg = 2 * i / (alpha * (n - 1)) - 1;
        t[i] = 0.5 * (1 + std::cos(3.1415 * arg));
    }
    for (int i = b1 + 1; i < b2 + 1 && i < n; ++i) t[i] = 1;
    for (int i = b2 + 1; i < n; ++i) {
        const float arg = 2 * i / (alpha * (n - 1)) - 2 / alpha + 1;
        t[i] = 0.5 * (1 + std::cos(3.1415 * arg));
    }
    return t;
}

// Row-pass table of the hologram window (Tukey, alpha 0.05, main.cpp:105):
// ((-1)^x w(x), -2^23 (-1)^x w(x)) for x in [0, H).  (-1)^x is the first
// fftshift; the second member lets a kernel turn a pixel read as 2^23 + p into
// p (-1)^x w(x) with one FMA.
inline std::vector<float2> hologram_window(int H) {
    const std::vector<double> t = tukey_factor(H, 0.05f);
    std::vector<float2> w(H);
    for (int x = 0; x < H; ++x) {
        const float ws = (x & 1) ? -(float)t[x] : (float)t[x];
        w[x] = make_float2(ws, -8388608.0f * ws);
    }
    return w;
}

// The C library's rand() as the reference's build draws it: glibc's random()
// with its default state, the additive feedback generator r[0] = 1,
// r[i] = 16807 r[i-1] mod (2^31 - 1) (0 < i < 31), r[i] = r[i-31]
// (31 <= i < 34), r[i] = r[i-3] + r[i-31] mod 2^32 (i >= 34), whose k-th
// output is r[k + 344] >> 1.
class CRand {
    uint32_t ring_[34];
    int pos_ = 0;  // ring slot of r[i-34], i the next index

public:
    CRand() {
        int64_t r[34];
        r[0] = 1;
        for (int i = 1; i < 31; ++i) r[i] = (16807 * r[i - 1]) % 2147483647;
        for (int i = 31; i < 34; ++i) r[i] = r[i - 31];
        for (int i = 0; i < 34; ++i) ring_[i] = (uint32_t)r[i];
        for (int i = 34; i < 344; ++i) step();
    }
    uint32_t step() {
        const uint32_t v = ring_[(pos_ + 31) % 34] + ring_[(pos_ + 3) % 34];
        ring_[pos_] = v;
        pos_ = pos_ + 1 == 34 ? 0 : pos_ + 1;
        return v;
    }
    int next() { return (int)(step() >> 1); }
};

// Herraez unwrapping's border reliabilities (VOLKOV 0).  initialisePIXELs
// (pretraitement_hors_axe_CPU/deroulement_herraez.cpp:348) draws one rand()
// per pixel, row by row, F^2 per angle in the order tomo_pretraitement
// unwraps them; calculate_reliability then overwrites the interior's.  Per
// angle, the draws of the border pixels: row 0, then columns 0 and F - 1 of
// rows 1 .. F - 2, then row F - 1 (4F - 4 values).
inline std::vector<int> crand_border_table(int F, int angles) {
    std::vector<int> t((size_t)angles * (4 * F - 4));
    CRand g;
    size_t o = 0;
    for (int a = 0; a < angles; ++a)
        for (int i = 0; i < F; ++i)
            for (int j = 0; j < F; ++j) {
                const int v = g.next();
                if (i == 0 || i == F - 1 || j == 0 || j == F - 1) t[o++] = v;
            }
    return t;
}

// Indices [x, y] where tukey_factor(n, alpha) is exactly 1 (its flat middle,
// same bounds as above): kernels skip the table there.
inline int2 tukey_flat(int n, float alpha) {
    const int b1 = (int)std::round(alpha * (n - 1) / 2);
    const int b2 = (int)std::round((n - 1) * (1 - alpha / 2));
    return make_int2(b1 + 1, b2 < n - 1 ? b2 : n - 1);
}

}  // namespace tdm
