// tomo_reconstruction on GB300: Ewald-cap mapping and 3D inverse FFT of the
// fields written by tomo_pretraitement, with the file contract of
// Tomo_prog/Reconstruction/main.cpp:
//   inputs  CHEMIN_RESULT/parametres.raw, tab_posSpec.raw, UBornfinal_{Re,Im}*.raw,
//           CHEMIN_CONFIG/recon.txt and config_manip.txt
//   outputs indice.tif, absorption.tif, OTF3D.tif (EXPORT_OTF), centre_reconstruction.tif,
//           slice.tiff
// -polar -etat S: configuration and results in CHEMIN_RACINE/demosaic/<S>UBorn/,
// the volume as indice_cplx_hdf5.hdf instead of the two TIFF volumes
// (Reconstruction/src/manip.cpp:18-30, main.cpp:358-367).
#include "app_common.h"

int main(int argc, char** argv) {
    const app::Args A = app::parse_args(argc, argv);
    if (A.help) {
        app::print_help("tomo_reconstruction");
        return 0;
    }
    app::Paths P;
    if (!app::read_paths_recon(A, P)) {
        std::fprintf(stderr, "cannot read $HOME/.config/%s\n", A.gui.c_str());
        return 1;
    }
    const std::string recon = P.config + "/recon.txt", manip = P.config + "/config_manip.txt";
    tdm_geom g;
    if (tdm_read_geom(recon.c_str(), manip.c_str(), &g) != TDM_OK) {
        std::fprintf(stderr, "cannot read %s or %s\n", recon.c_str(), manip.c_str());
        return 1;
    }
    // parametres.raw: NXMAX, NbAngle, rayon, dimROI, tailleTheoPixelHolo (Reconstruction/src/manip.cpp:42-45)
    std::vector<double> param;
    if (!app::read_f64(P.result + "parametres.raw", param, 5)) return 1;
    g.nxmax = (int)param[0];
    g.ccd_roix = (int)param[3];
    g.circle_cx = g.circle_cy = g.ccd_roix / 2;  // the crop is not used by the reconstruction
    const long tsz = app::file_size(P.result + "tab_posSpec.raw");
    if (tsz < 16) {
        std::fprintf(stderr, "Impossible d'ouvrir le fichier %stab_posSpec.raw\n", P.result.c_str());
        return 1;
    }
    const int M = (int)(tsz / 16);  // main.cpp:105-107
    const int F = 2 * g.nxmax, D = g.dim_final;
    std::vector<double> tab;
    if (!app::read_f64(P.result + "tab_posSpec.raw", tab, 2 * (size_t)M)) return 1;
    std::vector<int32_t> pos(2 * (size_t)M);
    std::vector<float> centres((size_t)F * F, 0.0f);
    for (int a = 0; a < M; ++a) {
        pos[a] = (int32_t)tab[a];  // (int) cast, main.cpp:205
        pos[M + a] = (int32_t)tab[M + a];
        const long cpt = std::lround(tab[M + a]) * F + std::lround(tab[a]);
        if (cpt >= 0 && cpt < (long)F * F) centres[cpt] = (float)a;
    }
    const std::string dim = std::to_string(F) + "x" + std::to_string(F) + "x" + std::to_string(M);
    std::vector<double> re, im;
    if (!app::read_f64(P.result + "UBornfinal_Im" + dim + ".raw", im, (size_t)M * F * F) ||
        !app::read_f64(P.result + "UBornfinal_Re" + dim + ".raw", re, (size_t)M * F * F))
        return 1;
    std::vector<float> fields((size_t)M * F * F * 2);
    for (size_t i = 0; i < re.size(); ++i) {
        fields[2 * i] = (float)re[i];
        fields[2 * i + 1] = (float)im[i];
    }
    double export_otf = 1;
    tdm_extract_val(recon.c_str(), "EXPORT_OTF", 1, &export_otf);
    tdm_ctx* c = nullptr;
    if (app::check(tdm_create(&g, M, &c), c, "tdm_create")) return 1;
    tdm_derived dv;
    tdm_get_derived(c, &dv);
    tdm_write_tiff_f32((P.result + "centre_reconstruction.tif").c_str(), centres.data(), F, F, 1, 1.0, 1);
    const size_t NT = (size_t)D * D * D;
    std::vector<float> vre(NT), vim(NT);
    std::vector<uint8_t> otf(export_otf != 0 ? NT : 0);
    if (app::check(tdm_reconstruct(c, fields.data(), pos.data(), M, vre.data(), vim.data(),
                                   export_otf != 0 ? otf.data() : nullptr, nullptr),
                   c, "tdm_reconstruct"))
        return 1;
    tdm_destroy(c);
    if (export_otf != 0) {
        std::vector<float> of(NT);
        for (size_t i = 0; i < NT; ++i) of[i] = otf[i];
        tdm_write_tiff_f32((P.result + "OTF3D.tif").c_str(), of.data(), D, D, D, dv.tp_tomo, 4);
    }
    if (A.polar) {
        if (tdm_write_hdf5_complex((P.result + "/indice_cplx_hdf5.hdf").c_str(), vre.data(), vim.data(), D, D, D) !=
            TDM_OK) {
            std::fprintf(stderr, "cannot write %s/indice_cplx_hdf5.hdf\n", P.result.c_str());
            return 1;
        }
    } else if (tdm_write_tiff_f32((P.result + "indice.tif").c_str(), vre.data(), D, D, D, dv.tp_tomo, 4) != TDM_OK ||
               tdm_write_tiff_f32((P.result + "absorption.tif").c_str(), vim.data(), D, D, D, dv.tp_tomo, 4) !=
                   TDM_OK) {
        std::fprintf(stderr, "cannot write the volumes in %s\n", P.result.c_str());
        return 1;
    }
    if (D > 236) {  // extractSliceZ(indice, "x", 236) (main.cpp:375-376)
        std::vector<float> sl((size_t)D * D);
        for (int z = 0; z < D; ++z)
            for (int y = 0; y < D; ++y) sl[(size_t)z * D + y] = vre[236 + (size_t)y * D + (size_t)z * D * D];
        tdm_write_tiff_f32((P.result + "slice.tiff").c_str(), sl.data(), D, D, 1, dv.tp_tomo, 1);
    }
    std::printf("#######-- Reconstruction terminee --#######\nResultats dans %s\n", P.result.c_str());
    return 0;
}
