// FP64 CPU oracle for the tomographic diffractive microscopy hot path.
//
// TEST INFRASTRUCTURE ONLY.  tests/, the smoke check and the CPU-baseline leg
// of bench.py call it to produce reference values.
// Nothing in the product (mtd_transmission_gb300/) links, loads or calls it.
//
// PARITY PINNED ON THE REFERENCE'S OWN CODE.  The reference's programs
// cannot be built as they stand (FFTW3, OpenCV4, libtiff and HDF5 are absent)
// and it ships no tests, golden vectors or fixtures for this path.  This
// oracle is a line-by-line FP64 restatement of the reference's functions;
// every function below cites the reference file:line it follows.  The
// reference's own source files for the path are compiled, against stand-in
// headers, into oracle/_ref/ (oracle/ref/build_ref.py), and
// tests/test_oracle_pinned.py compares this restatement with them on the
// same inputs (window and counts bit for bit, positions exactly, values at
// FP64 round-off).  Its FFT replaces FFTW3 (DFT with FFTW's sign and scaling
// conventions: FORWARD = exp(-2*pi*i*jk/n), BACKWARD = exp(+2*pi*i*jk/n),
// both unnormalised) and is cross-checked against numpy.fft in the tests.  The
// least-squares solve replaces OpenCV's cv::solve(DECOMP_NORMAL): normal
// equations A^T A, A^T b followed by Gaussian elimination with partial
// pivoting (OpenCV is not available to the pin; checked against numpy).
//
// Undefined behaviour in the reference is given a pinned oracle policy:
//  * Volkov DC term (deroulement_volkov4.cpp:189 reads tampon[nbPix], one past
//    the end): the zero-frequency term is set to 0.
//  * compuBackgr2 (Correction_aberration.cpp:157) sums 16 terms of a
//    15-coefficient polynomial: the oracle sums the 15 in-bounds terms.
//  * coupeCplx / retroPropag_Born have no bounds checks: out-of-range crops or
//    voxels are reported as errors instead of being written.
//
// Paths are relative to the reference project root.

#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

using cd = std::complex<double>;

namespace {

// ---------------------------------------------------------------------------
// FFT (FFTW conventions).  Radix-2 iterative Cooley-Tukey for power-of-two
// sizes; other sizes (the reference's own configuration has NXMAX 125: 250-
// and 500-point transforms) by a recursive mixed-radix decomposition
// (decimation in time, n = p m: p transforms of m points on the stride-p
// subsequences combined by p-point DFTs with twiddles W_n^(q k)).
// ---------------------------------------------------------------------------
struct Plan {
    int n = 0, logn = 0;
    std::vector<cd> tw;     // exp(-2 pi i k / n), k < n/2 (power of two); k < n (other sizes)
    std::vector<int> rev;
    std::vector<int> radices;  // other sizes: the factors, small first
};

std::mutex g_plan_mu;
std::map<int, std::unique_ptr<Plan>> g_plans;

const Plan& get_plan(int n) {
    std::lock_guard<std::mutex> lk(g_plan_mu);
    auto it = g_plans.find(n);
    if (it != g_plans.end()) return *it->second;
    auto p = std::make_unique<Plan>();
    p->n = n;
    if (n & (n - 1)) {
        int m = n;
        for (int r : {4, 2, 3, 5, 7})
            while (m % r == 0) {
                p->radices.push_back(r);
                m /= r;
            }
        for (int r = 11; m > 1; r += 2)
            while (m % r == 0) {
                p->radices.push_back(r);
                m /= r;
            }
        p->tw.resize(n);
        for (int k = 0; k < n; ++k) {
            long double a = -2.0L * 3.14159265358979323846264338327950288L * (long double)k / (long double)n;
            p->tw[k] = cd((double)std::cos(a), (double)std::sin(a));
        }
        const Plan& ref = *p;
        g_plans[n] = std::move(p);
        return ref;
    }
    int lg = 0;
    while ((1 << lg) < n) ++lg;
    p->logn = lg;
    p->tw.resize(std::max(1, n / 2));
    for (int k = 0; k < n / 2; ++k) {
        long double a = -2.0L * 3.14159265358979323846264338327950288L * (long double)k / (long double)n;
        p->tw[k] = cd((double)std::cos(a), (double)std::sin(a));
    }
    p->rev.resize(n);
    for (int i = 0; i < n; ++i) {
        int r = 0;
        for (int b = 0; b < lg; ++b) if (i & (1 << b)) r |= 1 << (lg - 1 - b);
        p->rev[i] = r;
    }
    const Plan& ref = *p;
    g_plans[n] = std::move(p);
    return ref;
}

bool is_pow2(long n) { return n > 0 && (n & (n - 1)) == 0; }

double omp_wall() {
#ifdef _OPENMP
    return omp_get_wtime();
#else
    return 0.0;
#endif
}

// out[0, len) = DFT of in[0], in[stride], ... (len points) with the plan's
// radices from index fi on; len divides p.n.
void fft_mixed(const cd* in, cd* out, int len, long stride, size_t fi, const Plan& p, int sign) {
    if (len == 1) {
        out[0] = in[0];
        return;
    }
    const int r = p.radices[fi], m = len / r, step = p.n / len;  // W_len^e = tw[e step]
    for (int q = 0; q < r; ++q) fft_mixed(in + q * stride, out + q * m, m, stride * r, fi + 1, p, sign);
    auto w = [&](long e) {
        const cd v = p.tw[(size_t)(e % len) * step];
        return sign > 0 ? std::conj(v) : v;
    };
    cd t[16];
    std::vector<cd> tv;
    cd* tt = t;
    if (r > 16) {
        tv.resize(r);
        tt = tv.data();
    }
    for (int k = 0; k < m; ++k) {
        for (int q = 0; q < r; ++q) tt[q] = out[q * m + k] * w((long)q * k);
        for (int j = 0; j < r; ++j) {
            cd acc = 0;
            for (int q = 0; q < r; ++q) acc += tt[q] * w((long)q * j * m);  // W_r^(q j)
            out[k + j * m] = acc;
        }
    }
}

// In-place 1D DFT. sign = -1: FFTW_FORWARD, +1: FFTW_BACKWARD. Unnormalised.
void fft1d(cd* x, const Plan& p, int sign) {
    const int n = p.n;
    if (!p.radices.empty()) {
        std::vector<cd> a(x, x + n);
        fft_mixed(a.data(), x, n, 1, 0, p, sign);
        return;
    }
    for (int i = 0; i < n; ++i) {
        int j = p.rev[i];
        if (i < j) std::swap(x[i], x[j]);
    }
    for (int len = 2; len <= n; len <<= 1) {
        const int half = len >> 1, step = n / len;
        for (int i = 0; i < n; i += len) {
            for (int k = 0; k < half; ++k) {
                cd w = p.tw[k * step];
                if (sign > 0) w = std::conj(w);
                cd u = x[i + k], v = x[i + k + half] * w;
                x[i + k] = u + v;
                x[i + k + half] = u - v;
            }
        }
    }
}

// 2D DFT of a dim x dim row-major array (FFTW fftw_plan_dft_2d(dim, dim)).
void fft2d(cd* a, int dim, int sign) {
    const Plan& p = get_plan(dim);
#pragma omp parallel for schedule(static)
    for (int y = 0; y < dim; ++y) fft1d(a + (size_t)y * dim, p, sign);
#pragma omp parallel
    {
        std::vector<cd> col(dim);
#pragma omp for schedule(static)
        for (int x = 0; x < dim; ++x) {
            for (int y = 0; y < dim; ++y) col[y] = a[(size_t)y * dim + x];
            fft1d(col.data(), p, sign);
            for (int y = 0; y < dim; ++y) a[(size_t)y * dim + x] = col[y];
        }
    }
}

// 3D DFT of a dim^3 array (FFTW fftw_plan_dft_3d(dim, dim, dim)).
void fft3d(cd* a, int dim, int sign) {
    const Plan& p = get_plan(dim);
    const size_t d = dim, d2 = d * d;
#pragma omp parallel for schedule(static)
    for (long r = 0; r < (long)d2; ++r) fft1d(a + (size_t)r * d, p, sign);
#pragma omp parallel
    {
        std::vector<cd> line(dim);
#pragma omp for schedule(static)
        for (long zx = 0; zx < (long)d2; ++zx) {
            size_t z = zx / d, x = zx % d;
            cd* base = a + z * d2 + x;
            for (size_t y = 0; y < d; ++y) line[y] = base[y * d];
            fft1d(line.data(), p, sign);
            for (size_t y = 0; y < d; ++y) base[y * d] = line[y];
        }
#pragma omp for schedule(static)
        for (long yx = 0; yx < (long)d2; ++yx) {
            cd* base = a + yx;
            for (size_t z = 0; z < d; ++z) line[z] = base[z * d2];
            fft1d(line.data(), p, sign);
            for (size_t z = 0; z < d; ++z) base[z * d2] = line[z];
        }
    }
}

// ---------------------------------------------------------------------------
// Reference helpers
// ---------------------------------------------------------------------------

// tukey2D: pretraitement_hors_axe_CPU/FFT_fonctions.cpp:61-87 and
// Reconstruction/src/FFT_fonctions.cpp:224-248 (identical).  The float alpha
// makes the index bounds and the cosine arguments single-precision
// expressions; 3.1415 is the reference's own constant.
std::vector<double> tukey2D(int dimx, int dimy, float alpha) {
    int N = dimx;
    std::vector<double> tuk2D((size_t)dimx * dimy);
    std::vector<double> tuk1Dx((size_t)dimx * dimy);
    int borne1 = (int)std::round(alpha * (N - 1) / 2);
    int borne2 = (int)std::round((N - 1) * (1 - alpha / 2));
    for (int cpt = 0; cpt < borne1 + 1; cpt++) {
        float arg = 2 * cpt / (alpha * (N - 1)) - 1;
        tuk1Dx[cpt] = 0.5 * (1 + std::cos(3.1415 * arg));
    }
    for (int cpt = borne1 + 1; cpt < borne2 + 1; cpt++) tuk1Dx[cpt] = 1;
    for (int cpt = borne2 + 1; cpt < N; cpt++) {
        float arg = 2 * cpt / (alpha * (N - 1)) - 2 / alpha + 1;
        tuk1Dx[cpt] = 0.5 * (1 + std::cos(3.1415 * arg));
    }
    for (int cpt = 0; cpt < N * N; cpt++) {
        int cptx = cpt % N, cpty = cpt / N;
        tuk2D[cpt] = tuk1Dx[cptx] * tuk1Dx[cpty];
    }
    return tuk2D;
}

// fftshift2D: pretraitement_hors_axe_CPU/FFT_fonctions.cpp:89-114 (complex) and
// :237-264 (double): result[(y+d/2)%d][(x+d/2)%d] = in[y][x] for even d.
template <class T>
std::vector<T> fftshift2D(const std::vector<T>& in, int dim) {
    std::vector<T> out(in.size());
    int dec = dim / 2;
    for (int yi = 0; yi < dec; yi++)
        for (int xi = 0; xi < dec; xi++) {
            size_t pixel = (size_t)yi * dim + xi;
            size_t pixel_shift = (size_t)(yi + dec) * dim + xi + dec;
            out[pixel_shift] = in[pixel];
            out[pixel] = in[pixel_shift];
            out[(size_t)(yi + dec) * dim + xi] = in[pixel + dec];
            out[pixel + dec] = in[(size_t)(yi + dec) * dim + xi];
        }
    return out;
}

// decal2DCplxGen2: pretraitement_hors_axe_CPU/fonctions.cpp:64-85 and
// decal2DCplxGen: Reconstruction/src/fonctions.cpp:1268-1309 (same mapping):
// circular shift, result[(y+dy) mod d][(x+dx) mod d] = in[y][x].
void decal2D(const cd* in, cd* out, int dim, int dx, int dy) {
    dy = dy % dim;
    dx = dx % dim;
    if (dx < 0) dx += dim;
    if (dy < 0) dy += dim;
    for (int y = 0; y < dim; ++y) {
        int yo = (y + dy) % dim;
        for (int x = 0; x < dim; ++x) out[(size_t)yo * dim + (x + dx) % dim] = in[(size_t)y * dim + x];
    }
}

// init_kvect_shift: pretraitement_hors_axe_CPU/FFT_fonctions.cpp:7-17.
// kvect = (i - round(n/2))/n, then fftshift2D: kappa(k) = k/n for k < n/2,
// (k-n)/n otherwise (the Nyquist bin holds -1/2).
double kvect1(int k, int n) {
    int i = (k + n / 2) % n;  // fftshift source index
    return ((double)i - std::round((double)(n / 2))) / (double)n;
}

// Symetrise_mirror: src/deroulement_volkov4.cpp:221-244.
std::vector<double> symetrise_mirror(const std::vector<double>& img, int dim) {
    std::vector<double> s((size_t)4 * dim * dim);
    for (int x = 0; x < dim; x++)
        for (int y = 0; y < dim; y++) {
            double v = img[(size_t)x + (size_t)y * dim];
            s[(size_t)(dim - 1 - x) + (size_t)(dim - 1 - y) * (2 * dim)] = v;
            s[(size_t)(dim + x) + (size_t)(dim - y - 1) * (2 * dim)] = v;
            s[(size_t)(dim - x - 1) + (size_t)(dim + y) * (2 * dim)] = v;
            s[(size_t)(dim + x) + (size_t)(dim + y) * (2 * dim)] = v;
        }
    return s;
}

// TF2Dcplx (pretraitement, FFT_fonctions.cpp:366-400): forward FFT / nbPix.
std::vector<cd> tf2d_norm(std::vector<cd> a, int dim) {
    fft2d(a.data(), dim, -1);
    const double n = (double)a.size();
    for (auto& v : a) v = cd(v.real() / n, v.imag() / n);
    return a;
}
// TF2Dcplx_INV (FFT_fonctions.cpp:420-438): backward FFT, unnormalised.
std::vector<cd> tf2d_inv(std::vector<cd> a, int dim) {
    fft2d(a.data(), dim, +1);
    return a;
}

// gradient_fft4 (src/deroulement_volkov4.cpp:98-159): FFT/n, multiply by
// 2*pi*kappa*i, two unnormalised inverse FFTs.
void gradient_fft4(const std::vector<cd>& in, int dim, std::vector<cd>& gx, std::vector<cd>& gy) {
    std::vector<cd> spectre = tf2d_norm(in, dim);
    std::vector<cd> tx(spectre.size()), ty(spectre.size());
    const cd I(0, 1);
    for (int y = 0; y < dim; ++y)
        for (int x = 0; x < dim; ++x) {
            size_t c = (size_t)y * dim + x;
            tx[c] = 2 * M_PI * kvect1(x, dim) * spectre[c] * I;
            ty[c] = 2 * M_PI * kvect1(y, dim) * spectre[c] * I;
        }
    gx = tf2d_inv(tx, dim);
    gy = tf2d_inv(ty, dim);
}

// integ_grad4 (src/deroulement_volkov4.cpp:162-191).  DC policy: 0.
std::vector<cd> integ_grad4(const std::vector<double>& gx, const std::vector<double>& gy, int dim) {
    std::vector<cd> a(gx.begin(), gx.end()), b(gy.begin(), gy.end());
    std::vector<cd> TFx = tf2d_norm(a, dim), TFy = tf2d_norm(b, dim);
    std::vector<cd> tampon(TFx.size());
    const cd I(0, 1);
    for (int y = 0; y < dim; ++y)
        for (int x = 0; x < dim; ++x) {
            size_t c = (size_t)y * dim + x;
            double kx = kvect1(x, dim), ky = kvect1(y, dim);
            double k2 = kx * kx + ky * ky;
            tampon[c] = -I * (TFx[c] * kx + TFy[c] * ky) / (2 * M_PI * k2);
        }
    tampon[0] = cd(0, 0);
    return tf2d_inv(tampon, dim);
}

// deroul_volkov4_total_sym_paire (src/deroulement_volkov4.cpp:14-92).
std::vector<double> volkov_unwrap(const std::vector<double>& phase, int dim) {
    const int L = 2 * dim;
    std::vector<double> sym = symetrise_mirror(phase, dim);
    std::vector<cd> symc(sym.begin(), sym.end());
    std::vector<cd> gxe, gye, gxz, gyz;
    gradient_fft4(symc, L, gxe, gye);
    std::vector<cd> Z(sym.size());
    for (size_t c = 0; c < sym.size(); ++c) Z[c] = cd(std::cos(sym[c]), std::sin(sym[c]));
    gradient_fft4(Z, L, gxz, gyz);
    const cd I(0, 1);
    std::vector<double> gix(sym.size()), giy(sym.size());
    for (size_t c = 0; c < sym.size(); ++c) {
        cd ax = -I * (gxz[c] / Z[c]);
        cd ay = -I * (gyz[c] / Z[c]);
        gix[c] = (ax.real() - gxe[c].real()) / (2 * M_PI);
        giy[c] = (ay.real() - gye[c].real()) / (2 * M_PI);
    }
    std::vector<cd> dint = integ_grad4(gix, giy, L);
    std::vector<double> out((size_t)dim * dim);
    for (int x = 0; x < dim; x++)
        for (int y = 0; y < dim; y++) {
            double intm = dint[(size_t)(dim + x) + (size_t)(dim + y) * L].real();  // cut_quad4 :263-276
            out[(size_t)x + (size_t)y * dim] = phase[(size_t)x + (size_t)y * dim] + 2 * M_PI * intm;
        }
    return out;
}

// ---------------------------------------------------------------------------
// Aberration correction: pretraitement_hors_axe_CPU/Correction_aberration.cpp
// ---------------------------------------------------------------------------
struct Aber {
    int dim = 0;
    std::vector<uint8_t> mask;   // marked mask (220 = sample point)
    std::vector<double> polyUs;  // NbPtOk x 15, row-major
    std::vector<double> poly;    // dim*dim x 15
    int nbPt = 0;
    std::vector<double> AtA;     // 15 x 15
};
constexpr int kDeg = 4, kNC = 15;

// countM (:86-106): every 5th row/column pixel with value > 45 becomes 220.
int countM(std::vector<uint8_t>& m, int dim) {
    int n = 0;
    for (int i = 0; i < dim; i += 5)
        for (int j = 0; j < dim; j += 5) {
            uint8_t& v = m[(size_t)j * dim + i];  // mask.at<uchar>(j,i): row j, column i
            if (v > 45) { v = 220; ++n; }
        }
    return n;
}

void mono(double x, double y, double* row) {  // CalcPolyUs_xy / CalcPoly_xy (:108-149)
    int k = 0;
    for (int px = 0; px <= kDeg; px++)
        for (int py = 0; px + py <= kDeg; py++) row[k++] = std::pow(x, px) * std::pow(y, py);
}

bool aber_init(Aber& A, const uint8_t* mask_in, int dim) {
    A.dim = dim;
    A.mask.assign((size_t)dim * dim, 255);  // init_mask_aber (:43-70): unit mask when absent
    if (mask_in) std::memcpy(A.mask.data(), mask_in, (size_t)dim * dim);
    A.nbPt = countM(A.mask, dim);
    if (A.nbPt <= 9) return false;  // CalcPolyUs_xy / compuCoefPoly2 need > 9 points
    A.polyUs.assign((size_t)A.nbPt * kNC, 0);
    int r = 0;
    for (int y = 0; y < dim; y++)
        for (int x = 0; x < dim; x++)
            if (A.mask[(size_t)y * dim + x] == 220) {
                if (r < A.nbPt) mono(x, y, &A.polyUs[(size_t)r * kNC]);
                ++r;
            }
    if (r != A.nbPt) return false;  // pre-marked 220 values elsewhere: reference UB
    A.poly.assign((size_t)dim * dim * kNC, 0);
    for (int y = 0; y < dim; y++)
        for (int x = 0; x < dim; x++) mono(x, y, &A.poly[((size_t)y * dim + x) * kNC]);
    A.AtA.assign(kNC * kNC, 0);
    for (int i = 0; i < kNC; ++i)
        for (int j = 0; j < kNC; ++j) {
            double s = 0;
            for (int p = 0; p < A.nbPt; ++p) s += A.polyUs[(size_t)p * kNC + i] * A.polyUs[(size_t)p * kNC + j];
            A.AtA[i * kNC + j] = s;
        }
    return true;
}

// Gaussian elimination with partial pivoting (cv::solve DECOMP_NORMAL -> LU).
void lu_solve(std::vector<double> M, std::vector<double> b, double* x) {
    const int n = kNC;
    for (int i = 0; i < n; ++i) {
        int piv = i;
        for (int j = i + 1; j < n; ++j) if (std::fabs(M[j * n + i]) > std::fabs(M[piv * n + i])) piv = j;
        if (piv != i) {
            for (int k = 0; k < n; ++k) std::swap(M[i * n + k], M[piv * n + k]);
            std::swap(b[i], b[piv]);
        }
        for (int j = i + 1; j < n; ++j) {
            double f = M[j * n + i] / M[i * n + i];
            for (int k = i; k < n; ++k) M[j * n + k] -= f * M[i * n + k];
            b[j] -= f * b[i];
        }
    }
    for (int i = n - 1; i >= 0; --i) {
        double s = b[i];
        for (int k = i + 1; k < n; ++k) s -= M[i * n + k] * x[k];
        x[i] = s / M[i * n + i];
    }
}

// compuCoefPoly2 (:186-217) + compuBackgr2 (:151-164, 15 in-bounds terms).
std::vector<double> aber_surface(const Aber& A, const std::vector<double>& img) {
    const int dim = A.dim;
    std::vector<double> b(A.nbPt);
    int u = 0;
    for (int y = 0; y < dim; y++)
        for (int x = 0; x < dim; x++)
            if (A.mask[(size_t)y * dim + x] == 220) b[u++] = img[(size_t)y * dim + x];
    std::vector<double> Atb(kNC, 0);
    for (int i = 0; i < kNC; ++i) {
        double s = 0;
        for (int p = 0; p < A.nbPt; ++p) s += A.polyUs[(size_t)p * kNC + i] * b[p];
        Atb[i] = s;
    }
    double coef[kNC];
    lu_solve(A.AtA, Atb, coef);
    std::vector<double> surf((size_t)dim * dim);
    for (size_t c = 0; c < surf.size(); ++c) {
        double s = 0;
        for (int k = 0; k < kNC; ++k) s += coef[k] * A.poly[c * kNC + k];
        surf[c] = s;
    }
    return surf;
}

// ---------------------------------------------------------------------------
// Herraez unwrapping (pretraitement_hors_axe_CPU/deroulement_herraez.cpp)
// ---------------------------------------------------------------------------
// The C library's rand() as the reference's build draws it: glibc's random()
// with its default TYPE_3 state, i.e. the additive feedback generator
//   r[0] = 1, r[i] = 16807 r[i-1] mod (2^31 - 1) (0 < i < 31),
//   r[i] = r[i-31] (31 <= i < 34), r[i] = r[i-3] + r[i-31] mod 2^32 (i >= 34),
// whose k-th output is r[k + 344] >> 1.
struct CRand {
    uint32_t ring[34];
    int pos = 0;  // index of r[i-34] in the ring, i the next index
    CRand() {
        int64_t r[34];
        r[0] = 1;
        for (int i = 1; i < 31; ++i) r[i] = (16807 * r[i - 1]) % 2147483647;
        for (int i = 31; i < 34; ++i) r[i] = r[i - 31];
        for (int i = 0; i < 34; ++i) ring[i] = (uint32_t)r[i];
        for (int i = 34; i < 344; ++i) step();
    }
    uint32_t step() {  // r[i] = r[i-3] + r[i-31]
        const uint32_t v = ring[(pos + 31) % 34] + ring[(pos + 3) % 34];
        ring[pos] = v;
        pos = (pos + 1) % 34;
        return v;
    }
    int next() { return (int)(step() >> 1); }
};

// Float constants and helpers of the file (:9-10, :357-380).
constexpr float kHzPi = 3.141592654f, kHzTwoPi = 6.283185307f;
float hz_wrap(float v) { return v > kHzPi ? v - kHzTwoPi : (v < -kHzPi ? v + kHzTwoPi : v); }
int hz_find_wrap(float l, float r) {
    const float d = l - r;
    return d > kHzPi ? -1 : (d < -kHzPi ? 1 : 0);
}

// sort (:163-180) and Mix (:113-159): a merge sort on edge indices that
// halves with size/2, so the last index of an odd-sized run is left where it
// is; stable merges, ties taken from the first run.
void hz_sort(const std::vector<float>& key, int* idx, int size, std::vector<int>& tmp) {
    if (size == 2) {
        if (key[idx[0]] > key[idx[1]]) std::swap(idx[0], idx[1]);
    } else if (size > 2) {
        const int h = size / 2;
        hz_sort(key, idx, h, tmp);
        hz_sort(key, idx + h, h, tmp);
        int a = 0, b = 0, o = 0;
        while (a < h && b < h) tmp[o++] = key[idx[a]] <= key[idx[h + b]] ? idx[a++] : idx[h + b++];
        while (a < h) tmp[o++] = idx[a++];
        while (b < h) tmp[o++] = idx[h + b++];
        std::copy(tmp.begin(), tmp.begin() + 2 * h, idx);
    }
}

// phaseUnwrapping_Mat (:32-74) on a W x W wrapped phase, as the angle of
// index `angle` in tomo_pretraitement's loop: every earlier angle drew W^2
// rand() values (initialisePIXELs, :348).  Writes the unwrapped phase and
// each pixel's number of 2 pi.
void herraez(const double* phase, int W, int angle, double* out, int32_t* inc_out) {
    const int n = W * W;
    CRand g;
    for (long long i = 0; i < (long long)angle * n; ++i) g.step();
    std::vector<float> value(n), rel(n);
    for (int p = 0; p < n; ++p) {  // initialisePIXELs (:333-355): 9999999 + rand() in int, wrapping past INT_MAX
        value[p] = (float)phase[p];
        rel[p] = (float)(int32_t)(9999999u + (uint32_t)g.next());
    }
    for (int i = 1; i < W - 1; ++i)  // calculate_reliability (:385-413), in float
        for (int j = 1; j < W - 1; ++j) {
            const int p = i * W + j;
            auto d2 = [&](int o) { return hz_wrap((float)(phase[p - o] - phase[p])) - hz_wrap((float)(phase[p] - phase[p + o])); };
            const float H = d2(1), V = d2(W), D1 = d2(W + 1), D2 = d2(W - 1);
            rel[p] = H * H + V * V + D1 * D1 + D2 * D2;
        }
    // horizentalEDGEs (:415-437) then verticalEDGEs (:439-459)
    const int ne = W * (W - 1) * 2;
    std::vector<int> p1(ne), p2(ne), einc(ne);
    std::vector<float> key(ne);
    int e = 0;
    for (int i = 0; i < W; ++i)
        for (int j = 0; j < W - 1; ++j, ++e) p1[e] = i * W + j, p2[e] = i * W + j + 1;
    for (int i = 0; i < W - 1; ++i)
        for (int j = 0; j < W; ++j, ++e) p1[e] = i * W + j, p2[e] = (i + 1) * W + j;
    for (e = 0; e < ne; ++e) {
        key[e] = rel[p1[e]] + rel[p2[e]];
        einc[e] = hz_find_wrap(value[p1[e]], value[p2[e]]);
    }
    std::vector<int> idx(ne), tmp(ne);  // quick_sort (:193-213)
    for (e = 0; e < ne; ++e) idx[e] = e;
    hz_sort(key, idx.data(), ne, tmp);
    // gatherPIXELs (:461-561): groups as linked lists from their head
    std::vector<int> head(n), last(n), next(n, -1), count(n, 1), inc(n, 0);
    for (int p = 0; p < n; ++p) head[p] = last[p] = p;
    for (int k = 0; k < ne; ++k) {
        const int q = idx[k], P1 = p1[q], P2 = p2[q], ei = einc[q];
        if (head[P2] == head[P1]) continue;
        if (next[P2] < 0 && head[P2] == P2) {  // PIXEL 2 alone: it joins PIXEL 1's group
            const int h1 = head[P1];
            next[last[h1]] = P2;
            last[h1] = P2;
            ++count[h1];
            head[P2] = h1;
            inc[P2] = inc[P1] - ei;
        } else if (next[P1] < 0 && head[P1] == P1) {  // PIXEL 1 alone: it joins PIXEL 2's group
            const int h2 = head[P2];
            next[last[h2]] = P1;
            last[h2] = P1;
            ++count[h2];
            head[P1] = h2;
            inc[P1] = inc[P2] + ei;
        } else {
            int g1 = head[P1], g2 = head[P2];
            if (count[g1] > count[g2]) {  // group 2 into group 1
                next[last[g1]] = g2;
                last[g1] = last[g2];
                count[g1] += count[g2];
                const int d = inc[P1] - ei - inc[P2];
                for (int r = g2; r >= 0; r = next[r]) head[r] = g1, inc[r] += d;
            } else {  // group 1 into group 2
                next[last[g2]] = g1;
                last[g2] = last[g1];
                count[g2] += count[g1];
                const int d = inc[P2] + ei - inc[P1];
                for (int r = g1; r >= 0; r = next[r]) head[r] = g2, inc[r] += d;
            }
        }
    }
    for (int p = 0; p < n; ++p) {  // unwrapImage (:564-575), returnImage (:580-594)
        const float v = value[p] + kHzTwoPi * (float)inc[p];
        out[p] = v;
        if (inc_out) inc_out[p] = inc[p];
    }
}

}  // namespace

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------
extern "C" {

typedef struct {
    double n0, na, lambda0, f_tube, f_obj, tpcam, rf;  // as returned by extract_val (float-rounded)
    double coef_na_obj_limit;
    int ccd_roix, nxmax, circle_cx, circle_cy, dim_final;
    int born, c_aber, deroul, volkov;
} orc_cfg;

typedef struct {
    double rayon, tp_holo, tp_uborn, tp_tomo, delta_f;
} orc_derived;

// manip (pretraitement_hors_axe_CPU/manip.cpp:32-104,
// Reconstruction/src/manip.cpp:52-94).
void orc_derive(const orc_cfg* c, orc_derived* d) {
    double G = c->f_tube / c->f_obj;
    double Gt = G / c->rf;
    d->tp_holo = c->tpcam / Gt;
    d->tp_uborn = d->tp_holo * c->ccd_roix / (double)(2 * (size_t)c->nxmax);
    d->delta_f = 1 / (d->tp_uborn * 2 * (double)c->nxmax);
    d->tp_tomo = d->tp_uborn * (double)(2 * (size_t)c->nxmax) / (double)c->dim_final;
    d->rayon = std::round((double)(size_t)c->nxmax * c->n0 / c->na);
}

// phaseUnwrapping_Mat (pretraitement_hors_axe_CPU/deroulement_herraez.cpp:32-74)
// for the angle of index `angle` of the stack (rand() draws of the earlier
// angles skipped); inc_out (may be null) receives each pixel's 2 pi count.
void orc_herraez(const double* phase, int F, int angle, double* out, int32_t* inc_out) {
    herraez(phase, F, angle, out, inc_out);
}

// The first n outputs of the C library's rand() generator (glibc, default
// seed) after `skip` draws, as the oracle restates it.
void orc_crand(long long skip, int n, int32_t* out) {
    CRand g;
    for (long long i = 0; i < skip; ++i) g.step();
    for (int i = 0; i < n; ++i) out[i] = g.next();
}

void orc_tukey2d(int n, float alpha, double* out) {
    std::vector<double> t = tukey2D(n, n, alpha);
    std::memcpy(out, t.data(), t.size() * sizeof(double));
}

// Plain DFTs for cross-checks (FFTW sign conventions, unnormalised).
int orc_fft2d(double* data, int dim, int sign) {
    if (dim < 1) return -1;
    fft2d(reinterpret_cast<cd*>(data), dim, sign);
    return 0;
}
int orc_fft3d(double* data, int dim, int sign) {
    if (dim < 1) return -1;
    fft3d(reinterpret_cast<cd*>(data), dim, sign);
    return 0;
}

// holo2TF_UBorn (pretraitement_hors_axe_CPU/fonctions.cpp:279-304) with the
// crop at coinHA = (CIRCLE_CX-NXMAX, CIRCLE_CY-NXMAX) (main.cpp:116),
// coupeCplx (fonctions.cpp:104-124).  holo: H*H samples as double.
// out: F*F complex (interleaved re, im).  Returns 0, or -1 on a crop outside
// the hologram spectrum (reference UB).
int orc_extract(const double* holo, int H, int nxmax, int cx, int cy, const double* tukey, double* out) {
    if (H & 1) return -2;
    const int F = 2 * nxmax;
    const int x0 = cx - nxmax, y0 = cy - nxmax;
    if (x0 < 0 || y0 < 0 || x0 + F > H || y0 + F > H) return -1;
    std::vector<double> h((size_t)H * H);
    for (size_t p = 0; p < h.size(); ++p) h[p] = holo[p] * tukey[p];
    std::vector<double> hs = fftshift2D(h, H);
    std::vector<cd> tf(hs.begin(), hs.end());
    fft2d(tf.data(), H, -1);
    const double nb = (double)tf.size();
    for (auto& v : tf) v = cd(v.real() / nb, v.imag() / nb);  // TF2Dcplx_vec :316-330
    std::vector<cd> tc = fftshift2D(tf, H);
    cd* o = reinterpret_cast<cd*>(out);
    for (int yd = 0; yd < F; ++yd)
        for (int xd = 0; xd < F; ++xd) o[(size_t)yd * F + xd] = tc[(size_t)(x0 + xd) + (size_t)(y0 + yd) * H];
    return 0;
}

// coordSpec (pretraitement_hors_axe_CPU/fonctions.cpp:88-101): element 0 is
// compared by |z|^2, the others by |z|; the first strictly greater wins.
int orc_coord_spec(const double* spec, int F) {
    const cd* s = reinterpret_cast<const cd*>(spec);
    const size_t n = (size_t)F * F;
    std::vector<double> mod(n);
    int cpt_max = 0;
    mod[0] = std::pow(s[0].real(), 2) + std::pow(s[0].imag(), 2);
    for (size_t c = 1; c < n; ++c) {
        mod[c] = std::abs(s[c]);
        if (mod[c] > mod[cpt_max]) cpt_max = (int)c;
    }
    return cpt_max;
}

// calc_Uborn2 (fonctions.cpp:348-374): shift by -posSpec, unnormalised
// backward FFT, shift by (F/2, F/2).
void orc_calc_uborn2(const double* spec, int F, int px, int py, double* field) {
    const cd* s = reinterpret_cast<const cd*>(spec);
    std::vector<cd> a((size_t)F * F), b;
    decal2D(s, a.data(), F, -px, -py);
    b = tf2d_inv(a, F);
    decal2D(b.data(), reinterpret_cast<cd*>(field), F, F / 2, F / 2);
}

// deroul_volkov4_total_sym_paire on a F*F wrapped phase.
void orc_volkov(const double* phase, int F, double* out) {
    std::vector<double> p(phase, phase + (size_t)F * F);
    std::vector<double> u = volkov_unwrap(p, F);
    std::memcpy(out, u.data(), u.size() * sizeof(double));
}

// Aberration fit surface of img (F*F) over the marked mask (NULL = unit mask).
// Returns the number of sample points, or -1 when the fit is undefined.
int orc_aber_surface(const uint8_t* mask, int F, const double* img, double* surf_out) {
    Aber A;
    if (!aber_init(A, mask, F)) return -1;
    std::vector<double> im(img, img + (size_t)F * F);
    std::vector<double> s = aber_surface(A, im);
    std::memcpy(surf_out, s.data(), s.size() * sizeof(double));
    return A.nbPt;
}

// Second loop of tomo_pretraitement (pretraitement_hors_axe_CPU/main.cpp:230-342)
// over M cropped spectra (M*F*F complex).  Writes the saved fields
// (UBornFinal, M*F*F complex) and tabPosSpec (x values then y values).
// Optional per-angle intermediates (may be NULL): wrapped phase, unwrapped
// phase, amplitude, corrected phase, corrected amplitude (M*F*F doubles each).
// Returns 0 or -1 (aberration fit undefined).  VOLKOV 0 unwraps with Herraez's
// method, the stack's angle a drawing its border reliabilities as the
// reference's loop would for its a-th angle (main.cpp:262-266).
int orc_fields(const double* spectra, int M, int nxmax, const orc_cfg* cfg, const uint8_t* mask,
               double* fields_out, double* posspec_out, double* dbg_phase, double* dbg_unwrap,
               double* dbg_amp, double* dbg_phase_corr, double* dbg_amp_corr) {
    const int F = 2 * nxmax;
    const size_t P = (size_t)F * F;
    Aber A;
    if (cfg->c_aber && !aber_init(A, mask, F)) return -1;
    for (int a = 0; a < M; ++a) {
        const cd* tf = reinterpret_cast<const cd*>(spectra) + (size_t)a * P;
        int cpt_max = orc_coord_spec(reinterpret_cast<const double*>(tf), F);
        double mre = tf[cpt_max].real(), mim = tf[cpt_max].imag();
        double mmod = std::sqrt(mim * mim + mre * mre);
        int kxmi = cpt_max % F, kymi = cpt_max / F;
        posspec_out[a] = (double)kxmi;
        posspec_out[a + M] = (double)kymi;
        cd* fo = reinterpret_cast<cd*>(fields_out) + (size_t)a * P;
        std::vector<cd> ub(P);
        if (cfg->c_aber) {
            orc_calc_uborn2(reinterpret_cast<const double*>(tf), F, kxmi, kymi, reinterpret_cast<double*>(ub.data()));
            std::vector<double> ph(P), unw;
            for (size_t c = 0; c < P; ++c) ph[c] = std::atan2(ub[c].imag(), ub[c].real());
            if (cfg->deroul && cfg->volkov) {
                unw = volkov_unwrap(ph, F);
            } else if (cfg->deroul) {
                unw.resize(P);
                herraez(ph.data(), F, a, unw.data(), nullptr);
            } else {
                unw = ph;
            }
            std::vector<double> sph = aber_surface(A, unw);
            std::vector<double> amp(P);
            for (size_t c = 0; c < P; ++c) amp[c] = std::abs(ub[c]);
            std::vector<double> samp = aber_surface(A, amp);
            for (size_t c = 0; c < P; ++c) {
                double pf = unw[c] - sph[c];
                double af = amp[c] / (samp[c] + 0.00000001);
                if (dbg_phase_corr) dbg_phase_corr[(size_t)a * P + c] = pf;
                if (dbg_amp_corr) dbg_amp_corr[(size_t)a * P + c] = af;
                if (af > 10) af = 1;
                if (af < -10) af = 1;
                if (cfg->born)
                    fo[c] = cd(std::sqrt(af * af) * std::cos(pf) - 1, std::sqrt(af * af) * std::sin(pf));
                else
                    fo[c] = cd(std::log(std::sqrt(af * af)), pf);
            }
            if (dbg_phase) std::memcpy(dbg_phase + (size_t)a * P, ph.data(), P * sizeof(double));
            if (dbg_unwrap) std::memcpy(dbg_unwrap + (size_t)a * P, unw.data(), P * sizeof(double));
            if (dbg_amp) std::memcpy(dbg_amp + (size_t)a * P, amp.data(), P * sizeof(double));
        } else {
            std::vector<cd> nrm(P);
            for (size_t c = 0; c < P; ++c)
                nrm[c] = cd((tf[c].real() * mre + tf[c].imag() * mim) / mmod,
                            (tf[c].imag() * mre - tf[c].real() * mim) / mmod);
            orc_calc_uborn2(reinterpret_cast<const double*>(nrm.data()), F, kxmi, kymi, reinterpret_cast<double*>(fo));
        }
    }
    return 0;
}

// tomo_reconstruction (Reconstruction/main.cpp:172-352) on M fields.
//  fields: M*F*F complex (UBornFinal), posspec: 2M doubles (x then y).
//  indice_out: D^3 complex, index = (-1/(2 n0 kv^2)) * PotObj (main.cpp:345-352).
//  sup_redon_out (D^3 doubles), otf_out (D^3 doubles, OTF3D mask) and
//  spectrum_out (D^3 complex, normalised TF3D_PotObj before the shift) may be NULL.
// Returns 0, or -1 when a cap voxel falls outside the volume (reference UB).
int orc_reconstruction(const double* fields, const double* posspec, int M, const orc_cfg* cfg,
                       double* indice_out, double* sup_redon_out, double* otf_out, double* spectrum_out,
                       double* seconds_out) {
    const double t_begin = omp_wall();
    orc_derived dv;
    orc_derive(cfg, &dv);
    const int N = cfg->nxmax, F = 2 * N, D = cfg->dim_final;
    const size_t P = (size_t)F * F, NT = (size_t)D * D * D;
    if ((F & 1) || (D & 1)) return -2;  // even sizes (the shifts are half-size rolls)
    std::vector<double> tuk = tukey2D(F, F, 0.1f);
    std::vector<cd> tf3d(NT);
    std::vector<double> sup(NT, 0.0);
    const int dec = (int)std::round(D / 2);
    // retroPropag_Born constants (Reconstruction/src/fonctions.cpp:884-902);
    // that file defines PI as 3.14159 (:2)
    const double PI_REF = 3.14159;
    float n0f = (float)cfg->n0;
    float kv = (float)(2 * PI_REF / cfg->lambda0);
    float k0 = kv * n0f;
    const double rayon = dv.rayon;
    const double cteNorm = -2 * PI_REF;
    const double r2 = rayon * rayon;
    const double norm_altitude = 1.0 / rayon;
    const int dimVolX = (int)std::round((double)D), dimPlanFinal = (int)std::round((double)D * D);
    const cd cteUb2Pot(0, k0 / PI_REF);
    const double dx = dv.tp_uborn;
    const double coefnorm = std::pow(dx, 2);
    int bad = 0;
    std::vector<cd> u2(P), ud(P), tfi(P), tfc(P);
    for (int a = 0; a < M; ++a) {
        int px = (int)posspec[a], py = (int)posspec[M + a];  // main.cpp:205
        const cd* fa = reinterpret_cast<const cd*>(fields) + (size_t)a * P;
        for (size_t c = 0; c < P; ++c) u2[c] = cd(fa[c].real() * tuk[c], fa[c].imag() * tuk[c]);
        decal2D(u2.data(), ud.data(), F, N, N);
        tfi = ud;
        fft2d(tfi.data(), F, -1);
        for (auto& v : tfi) v = cd(v.real() * coefnorm, v.imag() * coefnorm);  // TF2Dcplx (FFT_fonctions.cpp:333-349)
        decal2D(tfi.data(), tfc.data(), F, px, py);
        // retroPropag_Born (Reconstruction/src/fonctions.cpp:875-935)
        int fxm0 = px - N, fym0 = py - N;
        double fzm0_carre = rayon * rayon - fxm0 * fxm0 - fym0 * fym0;
        if (std::round(fzm0_carre) >= 0) {
            double fzm0 = std::sqrt(fzm0_carre);
            int NMAX_CARRE = N * N;
            for (int fdy = -N; fdy < N; fdy++) {
                int fdy_carre = fdy * fdy;
                for (int fdx = -N; fdx < N; fdx++) {
                    int cpt = (fdy + N) * 2 * N + fdx + N;
                    if (fdx * fdx + fdy_carre < cfg->coef_na_obj_limit * NMAX_CARRE) {
                        double fdz_carre = r2 - fdx * fdx - fdy_carre;
                        double koz = std::round(std::sqrt(fdz_carre) - fzm0);
                        double sdz = std::sqrt(rayon * rayon - fdx * fdx - fdy * fdy) * norm_altitude;
                        double altitude = (koz + dec) * dimPlanFinal;
                        double idx = (-fxm0 + fdx + dec) + (-fym0 + fdy + dec) * dimVolX + std::round(altitude);
                        long cptPot = (long)idx;
                        int ix = -fxm0 + fdx + dec, iy = -fym0 + fdy + dec;
                        int iz = (int)(koz + dec);
                        if (ix < 0 || ix >= D || iy < 0 || iy >= D || iz < 0 || iz >= D) { ++bad; continue; }
                        tf3d[cptPot] += cteUb2Pot * cteNorm * sdz * tfc[cpt];
                        sup[cptPot] += 1;
                    }
                }
            }
        }
    }
    if (bad) return -1;
    const double t_loop = omp_wall();
    // main.cpp:243-270
    for (size_t c = 0; c < NT; ++c) {
        if (sup_redon_out) sup_redon_out[c] = sup[c];
        if (sup[c] == 0) sup[c] = 1;
        tf3d[c] = tf3d[c] / sup[c];
        if (otf_out) otf_out[c] = (tf3d[c].real() != 0) ? 1.0 : 0.0;
    }
    if (spectrum_out) std::memcpy(spectrum_out, tf3d.data(), NT * sizeof(cd));
    // fftshift3D (Reconstruction/src/FFT_fonctions.cpp:78-151), TF3Dcplx_INV
    // (:394-412) x delta_f^3, fftshift3D, index constant (main.cpp:346-352).
    std::vector<cd> sh(NT);
    const size_t d = D, h = D / 2;
    auto shift3 = [&](const std::vector<cd>& in, std::vector<cd>& out) {
#pragma omp parallel for schedule(static)
        for (long z = 0; z < (long)d; ++z)
            for (size_t y = 0; y < d; ++y)
                for (size_t x = 0; x < d; ++x)
                    out[((z + h) % d) * d * d + ((y + h) % d) * d + (x + h) % d] = in[z * d * d + y * d + x];
    };
    shift3(tf3d, sh);
    std::vector<cd>().swap(tf3d);
    fft3d(sh.data(), D, +1);
    const double cn = std::pow(dv.delta_f, 3);
    for (auto& v : sh) v = cd(v.real() * cn, v.imag() * cn);
    std::vector<cd> po(NT);
    shift3(sh, po);
    std::vector<cd>().swap(sh);
    double k_v = 2 * M_PI / cfg->lambda0;
    cd cte(-1 / (2 * cfg->n0 * k_v * k_v), 0);
    cd* io = reinterpret_cast<cd*>(indice_out);
    for (size_t c = 0; c < NT; ++c) io[c] = cte * po[c];
    if (seconds_out) {
        seconds_out[0] = t_loop - t_begin;  // per-angle preparation and cap mapping
        seconds_out[1] = omp_wall() - t_loop;  // normalisation, shifts, 3D FFT, index
    }
    return 0;
}

int orc_set_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
    return omp_get_max_threads();
#else
    (void)n;
    return 1;
#endif
}

}  // extern "C"
