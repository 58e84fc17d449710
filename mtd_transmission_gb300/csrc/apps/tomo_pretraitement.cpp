// tomo_pretraitement on GB300: off-axis extraction and field formation for a
// stack of holograms, with the file contract of
// Tomo_prog/pretraitement_hors_axe_CPU/main.cpp:
//   inputs  CHEMIN_ACQUIS/i%03d.pgm (missing files are skipped), Image_mask.pgm,
//           CHEMIN_CONFIG/recon.txt and config_manip.txt
//   outputs CHEMIN_RESULT/UBornfinal_{Re,Im}{2N}x{2N}x{M}.raw (FP64, angle-major),
//           parametres.raw, tab_posSpec.raw, centres.tif, SAV_param_manip.txt
// -polar -etat S: one state of the polarisation set-up, acquisitions in
// CHEMIN_RACINE/demosaic<S>, results in <that>/UBorn/ (main.cpp:63-80).
#include "app_common.h"

int main(int argc, char** argv) {
    const app::Args A = app::parse_args(argc, argv);
    if (A.help) {
        app::print_help("tomo_pretraitement");
        return 0;
    }
    app::Paths P;
    if (!app::read_paths(A, P)) {
        std::fprintf(stderr, "cannot read $HOME/.config/%s\n", A.gui.c_str());
        return 1;
    }
    const std::string recon = P.config + "/recon.txt", manip = P.config + "/config_manip.txt";
    tdm_geom g;
    if (tdm_read_geom(recon.c_str(), manip.c_str(), &g) != TDM_OK) {
        std::fprintf(stderr, "cannot read %s or %s\n", recon.c_str(), manip.c_str());
        return 1;
    }
    double nb_holo = 0, premier = 0;
    tdm_extract_val(manip.c_str(), "NB_HOLO", 0, &nb_holo);
    tdm_extract_val(recon.c_str(), "PREMIER_ANGLE", 0, &premier);
    const int nb_angle = (int)nb_holo - (int)premier;  // manip.cpp:67-69
    const int H = g.ccd_roix, F = 2 * g.nxmax;
    std::vector<uint16_t> holos;
    const int ok = app::read_stack(P.acquis, H, nb_angle, holos);
    if (ok <= 0) {
        std::fprintf(stderr, "no hologram read from %s\n", P.acquis.c_str());
        return 1;
    }
    tdm_ctx* c = nullptr;
    if (app::check(tdm_create(&g, ok, &c), c, "tdm_create")) return 1;
    if (app::check(app::load_mask(c, P.mask, F), c, "tdm_set_mask")) return 1;
    std::vector<float> fields((size_t)ok * F * F * 2);
    std::vector<int32_t> pos(2 * (size_t)ok);
    if (app::check(tdm_extract(c, holos.data(), 16, ok, nullptr), c, "tdm_extract")) return 1;
    if (app::check(tdm_fields(c, nullptr, ok, fields.data(), pos.data()), c, "tdm_fields")) return 1;
    tdm_derived dv;
    tdm_get_derived(c, &dv);
    tdm_destroy(c);
    // outputs (main.cpp:325-358)
    const std::string dim = std::to_string(F) + "x" + std::to_string(F) + "x" + std::to_string(ok);
    std::vector<double> plane((size_t)ok * F * F);
    for (int part = 0; part < 2; ++part) {
        for (size_t i = 0; i < plane.size(); ++i) plane[i] = fields[2 * i + part];
        const std::string f = P.result + (part ? "UBornfinal_Im" : "UBornfinal_Re") + dim + ".raw";
        std::remove(f.c_str());
        if (!app::write_f64(f, plane.data(), plane.size())) {
            std::fprintf(stderr, "Erreur d'ouverture du fichier %s\n", f.c_str());
            return 1;
        }
    }
    const double param[5] = {(double)g.nxmax, (double)ok, dv.rayon, (double)H, dv.tp_holo};
    std::vector<double> tab(2 * (size_t)ok);
    std::vector<float> centre((size_t)F * F, 0.0f);
    for (int a = 0; a < ok; ++a) {
        tab[a] = pos[a];
        tab[ok + a] = pos[ok + a];
        centre[(size_t)pos[a] * F + pos[ok + a]] = (float)a;  // centre[kxmi*2N+kymi] (main.cpp:252)
    }
    if (!app::write_f64(P.result + "parametres.raw", param, 5) ||
        !app::write_f64(P.result + "tab_posSpec.raw", tab.data(), tab.size()))
        return 1;
    tdm_write_tiff_f32((P.result + "centres.tif").c_str(), centre.data(), F, F, 1, g.na / g.nxmax, 1);
    FILE* fp = std::fopen((P.result + "SAV_param_manip.txt").c_str(), "w");
    if (fp) {
        std::fprintf(fp, "Fichiers d'acquisition : %s\n", P.acquis.c_str());
        std::fprintf(fp, "Tp Holo %g m\nNXMAX %d\nrayon Ewald %g pixels\nNbAngleOk %d\nNA %g\n", dv.tp_holo, g.nxmax,
                     dv.rayon, ok, g.na);
        std::fclose(fp);
    }
    std::printf("Fin pretraitement: %d hologrammes\nResults in %s\n", ok, P.result.c_str());
    return 0;
}
