// Implementation of the FFTW3 subset declared in shim/fftw3.h, for the
// oracle's reference build (test infrastructure only): the reference's own
// sources call these functions and get unnormalised discrete Fourier
// transforms with FFTW's conventions (sign -1 forward, row-major arrays with
// the last dimension contiguous, r2c keeping n1/2 + 1 columns).
//
// The transform is a recursive mixed-radix Cooley-Tukey decomposition
// (decimation in time: an n = p m point transform is p transforms of m points
// on the stride-p subsequences, combined by p-point DFTs with twiddles
// W_n^(q k)), for any length; twiddles are computed in long double.
#include <cmath>
#include <complex>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "shim/fftw3.h"

namespace {

using cd = std::complex<double>;

struct Fft1d {
    int n = 0, sign = -1;
    std::vector<int> radices;
    std::vector<cd> w;  // w[j] = exp(sign 2 pi i j / n)
    Fft1d(int n_, int sign_) : n(n_), sign(sign_) {
        int m = n;
        for (int p : {4, 2, 3, 5, 7})
            while (m % p == 0 && m > 1) {
                radices.push_back(p);
                m /= p;
            }
        for (int p = 11; m > 1; p += 2)
            while (m % p == 0) {
                radices.push_back(p);
                m /= p;
            }
        w.resize(n);
        const long double two_pi = 6.283185307179586476925286766559L;
        for (int j = 0; j < n; ++j) {
            const long double a = two_pi * (long double)j / (long double)n;
            w[j] = cd((double)cosl(a), (double)(sign * sinl(a)));
        }
    }
    // out[0, len) = DFT of in[0], in[stride], ... (len points), radices from index fi on
    void rec(const cd* in, cd* out, int len, long stride, size_t fi) const {
        if (len == 1) {
            out[0] = in[0];
            return;
        }
        const int p = radices[fi], m = len / p;
        for (int q = 0; q < p; ++q) rec(in + q * stride, out + q * m, m, stride * p, fi + 1);
        const int step = n / len;  // W_len^e = w[e * step]
        std::vector<cd> t(p);
        for (int k = 0; k < m; ++k) {
            for (int q = 0; q < p; ++q) t[q] = out[q * m + k] * w[(size_t)((long)q * k % len) * step];
            for (int r = 0; r < p; ++r) {
                cd s = 0;
                for (int q = 0; q < p; ++q) s += t[q] * w[(size_t)((long)q * r * m % len) * step];  // W_p^(q r)
                out[k + r * m] = s;
            }
        }
    }
    void run(cd* x, long stride, std::vector<cd>& a, std::vector<cd>& b) const {
        a.resize(n);
        b.resize(n);
        for (int i = 0; i < n; ++i) a[i] = x[i * stride];
        rec(a.data(), b.data(), n, 1, 0);
        for (int i = 0; i < n; ++i) x[i * stride] = b[i];
    }
};

}  // namespace

struct tdm_ref_fftw_plan_s {
    int rank = 0;
    int dims[3] = {1, 1, 1};
    int sign = -1;
    bool r2c = false;
    fftw_complex* in = nullptr;
    fftw_complex* out = nullptr;
    double* rin = nullptr;
};

static fftw_plan make(int rank, const int* d, fftw_complex* in, fftw_complex* out, int sign) {
    auto* p = new tdm_ref_fftw_plan_s;
    p->rank = rank;
    for (int i = 0; i < rank; ++i) p->dims[i] = d[i];
    p->in = in;
    p->out = out;
    p->sign = sign;
    return p;
}

// Unnormalised DFT of the row-major array x over all its dimensions.
static void transform(cd* x, int rank, const int* dims, int sign) {
    size_t total = 1;
    for (int i = 0; i < rank; ++i) total *= (size_t)dims[i];
    std::vector<cd> a, b;
    for (int ax = 0; ax < rank; ++ax) {
        const int n = dims[ax];
        if (n == 1) continue;
        long stride = 1;
        for (int i = ax + 1; i < rank; ++i) stride *= dims[i];
        const Fft1d f(n, sign);
        const size_t outer = total / ((size_t)n * stride);
        for (size_t o = 0; o < outer; ++o)
            for (long s = 0; s < stride; ++s) f.run(x + o * n * stride + s, stride, a, b);
    }
}

extern "C" {

void* fftw_malloc(size_t n) { return std::malloc(n ? n : 1); }
void fftw_free(void* p) { std::free(p); }
fftw_complex* fftw_alloc_complex(size_t n) { return (fftw_complex*)fftw_malloc(n * sizeof(fftw_complex)); }
double* fftw_alloc_real(size_t n) { return (double*)fftw_malloc(n * sizeof(double)); }
int fftw_init_threads(void) { return 1; }
void fftw_plan_with_nthreads(int) {}
void fftw_cleanup_threads(void) {}
void fftw_cleanup(void) {}

fftw_plan fftw_plan_dft_1d(int n, fftw_complex* in, fftw_complex* out, int sign, unsigned) {
    const int d[1] = {n};
    return make(1, d, in, out, sign);
}
fftw_plan fftw_plan_dft_2d(int n0, int n1, fftw_complex* in, fftw_complex* out, int sign, unsigned) {
    const int d[2] = {n0, n1};
    return make(2, d, in, out, sign);
}
fftw_plan fftw_plan_dft_3d(int n0, int n1, int n2, fftw_complex* in, fftw_complex* out, int sign, unsigned) {
    const int d[3] = {n0, n1, n2};
    return make(3, d, in, out, sign);
}
fftw_plan fftw_plan_dft_r2c_2d(int n0, int n1, double* in, fftw_complex* out, unsigned) {
    const int d[2] = {n0, n1};
    fftw_plan p = make(2, d, nullptr, out, -1);
    p->r2c = true;
    p->rin = in;
    return p;
}

void fftw_execute_dft(const fftw_plan p, fftw_complex* in, fftw_complex* out) {
    size_t total = 1;
    for (int i = 0; i < p->rank; ++i) total *= (size_t)p->dims[i];
    std::vector<cd> x(total);
    std::memcpy((void*)x.data(), in, total * sizeof(cd));
    transform(x.data(), p->rank, p->dims, p->sign);
    std::memcpy(out, x.data(), total * sizeof(cd));
}

void fftw_execute(const fftw_plan p) {
    if (!p->r2c) {
        fftw_execute_dft(p, p->in, p->out);
        return;
    }
    const int n0 = p->dims[0], n1 = p->dims[1], h = n1 / 2 + 1;
    std::vector<cd> x((size_t)n0 * n1);
    for (size_t i = 0; i < x.size(); ++i) x[i] = cd(p->rin[i], 0.0);
    transform(x.data(), 2, p->dims, -1);
    for (int r = 0; r < n0; ++r)
        std::memcpy(p->out + (size_t)r * h, x.data() + (size_t)r * n1, (size_t)h * sizeof(cd));
}

void fftw_destroy_plan(fftw_plan p) { delete p; }
int fftw_export_wisdom_to_filename(const char*) { return 1; }
int fftw_import_wisdom_from_filename(const char*) { return 0; }
int fftw_import_wisdom_from_file(void*) { return 0; }

}  // extern "C"
