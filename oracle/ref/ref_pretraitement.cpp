// Driver of the reference's own preprocessing functions (test infrastructure
// only): compiled with Tomo_prog/pretraitement_hors_axe_CPU/{fonctions.cpp,
// FFT_fonctions.cpp, src/deroulement_volkov4.cpp, src/FFTW_init.cpp,
// src/vecteur.cpp, deroulement_herraez.cpp} into
// oracle/_ref/libref_pretraitement.so.  Each entry point
// sets up its arguments as tomo_pretraitement's main does
// (pretraitement_hors_axe_CPU/main.cpp, lines cited) and calls the
// reference function; nothing here recomputes what the reference computes.
#include <malloc.h>

#include <complex>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "FFTW_init.h"
#include "FFT_fonctions.h"
#include "deroulement_herraez.h"
#include "deroulement_volkov4.h"
#include "fonctions.h"

using cd = std::complex<double>;

namespace {
// integ_grad4 (src/deroulement_volkov4.cpp:189) reads one element past the
// end of its spectrum for the zero frequency.  Large blocks are mapped
// pages, and the bytes after such a block are zero, so that read returns 0
// here: a piston of 2 pi Re(tampon[1])/2 on the unwrapped phase.
struct MapLargeBlocks {
    MapLargeBlocks() { mallopt(M_MMAP_THRESHOLD, 64 * 1024); }
} map_large_blocks;
}  // namespace

extern "C" {

// tukey2D (FFT_fonctions.cpp:61-87), main.cpp:105 with alpha 0.05.
void ref_pre_tukey2d(int n, float alpha, double* out) {
    const std::vector<double> t = tukey2D(n, n, alpha);
    std::memcpy(out, t.data(), t.size() * sizeof(double));
}

// holo2TF_UBorn (fonctions.cpp:279-304) as main.cpp:100-105,116,150 call it.
void ref_pre_extract(const double* holo, int H, int nxmax, int cx, int cy, double* out) {
    const size_t n = (size_t)H * H;
    fftw_complex* in_holo = (fftw_complex*)fftw_malloc(sizeof(fftw_complex) * n);
    fftw_complex* out_holo = (fftw_complex*)fftw_malloc(sizeof(fftw_complex) * n);
    fftw_plan p = fftw_plan_dft_2d(H, H, in_holo, out_holo, FFTW_FORWARD, FFTW_MEASURE);
    const std::vector<double> tukey = tukey2D(H, H, 0.05);
    const Var2D dimROI = {H, H}, dim2DHA = {2 * nxmax, 2 * nxmax}, coinHA = {cx - nxmax, cy - nxmax};
    std::vector<cd> tot((size_t)4 * nxmax * nxmax);
    std::vector<double> holo1(holo, holo + n);
    holo2TF_UBorn(holo1, tot, dimROI, dim2DHA, coinHA, 0, tukey, in_holo, out_holo, p);
    std::memcpy(out, tot.data(), tot.size() * sizeof(cd));
    fftw_destroy_plan(p);
    fftw_free(in_holo);
    fftw_free(out_holo);
}

// coordSpec (fonctions.cpp:88-101), main.cpp:235.
int ref_pre_coord_spec(const double* spec, int F) {
    const std::vector<cd> s(reinterpret_cast<const cd*>(spec), reinterpret_cast<const cd*>(spec) + (size_t)F * F);
    std::vector<double> mod((size_t)F * F);
    return coordSpec(s, mod, Var2D{F / 2, F / 2});
}

// calc_Uborn2 (fonctions.cpp:348-374) with the c2c plans of main.cpp:186, and
// calcPhase_mpi_pi_atan2 (fonctions.cpp:39-43), main.cpp:258-263.
void ref_pre_field(const double* spec, int F, int px, int py, double* field, double* phase) {
    const std::vector<cd> s(reinterpret_cast<const cd*>(spec), reinterpret_cast<const cd*>(spec) + (size_t)F * F);
    FFTW_init param_c2c(s, 1);
    std::vector<cd> ub((size_t)F * F);
    calc_Uborn2(s, ub, Var2D{F, F}, Var2D{px, py}, param_c2c);
    std::memcpy(field, ub.data(), ub.size() * sizeof(cd));
    if (phase) {
        std::vector<double> ph((size_t)F * F);
        calcPhase_mpi_pi_atan2(ub, ph);
        std::memcpy(phase, ph.data(), ph.size() * sizeof(double));
    }
}

// deroul_volkov4_total_sym_paire (src/deroulement_volkov4.cpp:14-92) with the
// plans and wave vectors of main.cpp:190-191,224-226.
void ref_pre_volkov(const double* phase, int F, double* out) {
    std::vector<double> ph(phase, phase + (size_t)F * F), un((size_t)F * F);
    std::vector<double> sym((size_t)4 * F * F);
    FFTW_init param_c2c_double(sym, 1);
    std::vector<vecteur> kv = init_kvect_shift(Var2D{2 * F, 2 * F});
    deroul_volkov4_total_sym_paire(ph, un, kv, param_c2c_double);
    std::memcpy(out, un.data(), un.size() * sizeof(double));
}

// phaseUnwrapping_Mat (deroulement_herraez.cpp:32-74) as main.cpp:263 calls
// it for the angle of index `angle` in tomo_pretraitement's loop: every
// earlier angle drew F^2 rand() values in initialisePIXELs (:348), so the C
// library's generator is reset (srand(1) is its initial state) and advanced
// by angle F^2 draws first.
void ref_pre_herraez(const double* phase, int F, int angle, double* out) {
    srand(1);
    for (long long i = 0; i < (long long)angle * F * F; ++i) rand();
    const std::vector<double> ph(phase, phase + (size_t)F * F);
    phaseUnwrapping_Mat(Var2D{F, F}, ph, out);
}

}  // extern "C"
