// Driver of the reference's own reconstruction functions (test
// infrastructure only): compiled with Tomo_prog/Reconstruction/src/{fonctions.cpp,
// FFT_fonctions.cpp, FFT_encaps.cpp, manip.cpp, Point2D.cpp, Point3D.cpp}
// into oracle/_ref/libref_reconstruction.so.  The parameters come from the
// reference's manip class reading a configuration tree under `home` (its
// $HOME/.config/gui_tomo.conf, recon.txt, config_manip.txt and
// parametres.raw); ref_rec_volume then runs the sequence of
// tomo_reconstruction's main (Reconstruction/main.cpp:107-352, lines cited)
// on fields and specular positions given in memory instead of read from the
// raw files.
#include <cstdlib>
#include <cstring>
#include <complex>
#include <string>
#include <vector>

#include "FFT_encaps.h"
#include "FFT_fonctions.h"
#include "fonctions.h"
#include "manip.h"

using cd = std::complex<double>;

namespace {
manip load(const char* home) {
    setenv("HOME", home, 1);
    return manip("gui_tomo.conf", "", false);
}
}  // namespace

extern "C" {

// The manip constructor's parameters (Reconstruction/src/manip.cpp:10-94):
// rayon, tailleTheoPixelHolo, tailleTheoPixelUborn, Delta_fUborn,
// tailleTheoPixelTomo, n0, lambda0, NA, coef_NA_obj_limit, dim_final, NXMAX.
int ref_rec_manip(const char* home, double* out) {
    const manip m = load(home);
    const double v[11] = {m.rayon, m.tailleTheoPixelHolo, m.tailleTheoPixelUborn, m.Delta_fUborn,
                          m.tailleTheoPixelTomo, m.n0, m.lambda0, m.NA_obj, m.coef_NA_obj_limit,
                          (double)m.dim_final, (double)m.NXMAX};
    std::memcpy(out, v, sizeof(v));
    return 0;
}

// main.cpp:107-352 on n fields (F x F complex each) and specular positions
// (n x values then n y values, as tab_posSpec.raw): indice receives the
// complex index volume (Re = indice.tif, Im = absorption.tif), counts the hit
// counts (sup_redon before its zeros are replaced), otf the OTF mask.
int ref_rec_volume(const char* home, const double* fields, const double* tab_pos_spec, int n, double* indice,
                   double* counts, double* otf) {
    manip m1 = load(home);
    const int NXMAX = (int)m1.NXMAX;
    const Var2D NMAX = {NXMAX, NXMAX}, dim2DHA = {2 * NXMAX, 2 * NXMAX};
    const Point2D dim2DUBorn(2 * NXMAX, 2 * NXMAX, 2 * NXMAX);
    FFT_encaps tf2D(dim2DUBorn);                                                   // main.cpp:131
    const int dim_final = (int)m1.dim_final;                                       // :134
    const Var3D decal3DTF = {(int)round(dim_final / 2), (int)round(dim_final / 2), (int)round(dim_final / 2)};
    const int NbPixU_Born = dim2DHA.x * dim2DHA.y;
    const size_t N_tab = (size_t)dim_final * dim_final * dim_final;
    std::vector<cd> UBornFinal2D(NbPixU_Born), UBorn2DFinalDecal(NbPixU_Born), TF_UBorn_normC(NbPixU_Born),
        TF_UBorn_normI(NbPixU_Born);
    std::vector<cd> TF3D_PotObj(N_tab);
    std::vector<double> sup_redon(N_tab);
    const std::vector<double> mask_tukey2D = tukey2D(dim2DHA.x, dim2DHA.y, 0.1f);  // :184-185
    const cd* f = reinterpret_cast<const cd*>(fields);
    for (int a = 0; a < n; ++a) {                                                  // :200-224
        const Var2D posSpec = {(int)tab_pos_spec[a], (int)tab_pos_spec[n + a]};
        for (int cpt = 0; cpt < NbPixU_Born; ++cpt) {
            UBornFinal2D[cpt].real(f[cpt + (size_t)a * NbPixU_Born].real() * mask_tukey2D[cpt]);
            UBornFinal2D[cpt].imag(f[cpt + (size_t)a * NbPixU_Born].imag() * mask_tukey2D[cpt]);
        }
        decal2DCplxGen(UBornFinal2D, UBorn2DFinalDecal, dim2DHA, NMAX);
        TF2Dcplx(UBorn2DFinalDecal, TF_UBorn_normI, tf2D, m1.tailleTheoPixelUborn);
        const Var2D recal = {posSpec.x, posSpec.y};
        decal2DCplxGen(TF_UBorn_normI, TF_UBorn_normC, dim2DHA, recal);
        retroPropag_Born(TF3D_PotObj, TF_UBorn_normC, sup_redon, dim_final, posSpec, decal3DTF, NMAX, m1.rayon, m1);
    }
    if (counts) std::memcpy(counts, sup_redon.data(), N_tab * sizeof(double));
    for (size_t cpt = 0; cpt < N_tab; ++cpt) {                                     // :243-249
        if (sup_redon[cpt] == 0) sup_redon[cpt] = 1;
        TF3D_PotObj[cpt] = TF3D_PotObj[cpt] / sup_redon[cpt];
    }
    if (otf)                                                                       // :262-267
        for (size_t c = 0; c < N_tab; ++c) otf[c] = TF3D_PotObj[c].real() != 0 ? 1.0 : 0.0;
    std::vector<cd> shifted(N_tab);
    fftshift3D(TF3D_PotObj, shifted);                                              // :282
    std::vector<cd>().swap(TF3D_PotObj);
    std::vector<cd> PotObj_shift(N_tab);
    Point3D dim3D(dim_final, dim_final, dim_final, dim_final);
    FFT_encaps tf3D_out(dim3D, 1, 0);                                              // :318
    TF3Dcplx_INV(tf3D_out.in, tf3D_out.out, shifted, PotObj_shift, tf3D_out.p_backward_OUT, m1.Delta_fUborn);
    std::vector<cd>().swap(shifted);
    std::vector<cd> PotObj3D(N_tab);
    fftshift3D(PotObj_shift, PotObj3D);                                            // :332
    const double k_v = 2 * M_PI / m1.lambda0;  // :341-347 (PI is M_PI, :28)
    const cd ctePot2Ind(-1 / (2 * m1.n0 * k_v * k_v), 0);
    cd* out = reinterpret_cast<cd*>(indice);
    for (size_t cpt = 0; cpt < N_tab; ++cpt) out[cpt] = ctePot2Ind * PotObj3D[cpt];
    return 0;
}

}  // extern "C"
