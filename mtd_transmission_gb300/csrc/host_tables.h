// Host-side tables shared by the entry points.
#pragma once

#include <cmath>
#include <vector>

namespace tdm {

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

}  // namespace tdm
