// tomo_pipeline: tomo_pretraitement followed by tomo_reconstruction in one
// pass, the fields staying in GPU memory.  Same inputs as tomo_pretraitement
// and the outputs of tomo_reconstruction in CHEMIN_RESULT; --save-fields also
// writes the UBornfinal_*.raw, parametres.raw and tab_posSpec.raw files.
#include "app_common.h"

int main(int argc, char** argv) {
    bool save_fields = false;
    for (int i = 1; i < argc; ++i)
        if (std::string(argv[i]) == "--save-fields") save_fields = true;
    if (int r = app::parse_args(argc, argv, "tomo_pipeline")) return r == 1 ? 0 : r;
    app::Paths P;
    if (!app::read_paths(P)) {
        std::fprintf(stderr, "cannot read $HOME/.config/gui_tomo.conf\n");
        return 1;
    }
    const std::string recon = P.config + "/recon.txt", manip = P.config + "/config_manip.txt";
    tdm_geom g;
    if (tdm_read_geom(recon.c_str(), manip.c_str(), &g) != TDM_OK) {
        std::fprintf(stderr, "cannot read %s or %s\n", recon.c_str(), manip.c_str());
        return 1;
    }
    double nb_holo = 0, premier = 0, export_otf = 1;
    tdm_extract_val(manip.c_str(), "NB_HOLO", 0, &nb_holo);
    tdm_extract_val(recon.c_str(), "PREMIER_ANGLE", 0, &premier);
    tdm_extract_val(recon.c_str(), "EXPORT_OTF", 1, &export_otf);
    const int H = g.ccd_roix, F = 2 * g.nxmax, D = g.dim_final;
    std::vector<uint16_t> holos;
    const int M = app::read_stack(P.acquis, H, (int)nb_holo - (int)premier, holos);
    if (M <= 0) {
        std::fprintf(stderr, "no hologram read from %s\n", P.acquis.c_str());
        return 1;
    }
    tdm_ctx* c = nullptr;
    if (app::check(tdm_create(&g, M, &c), c, "tdm_create")) return 1;
    if (app::check(app::load_mask(c, P.acquis + "Image_mask.pgm", F), c, "tdm_set_mask")) return 1;
    tdm_derived dv;
    tdm_get_derived(c, &dv);
    const size_t NT = (size_t)D * D * D;
    std::vector<float> vre(NT), vim(NT);
    std::vector<uint8_t> otf(export_otf != 0 ? NT : 0);
    std::vector<int32_t> pos(2 * (size_t)M);
    if (app::check(tdm_pipeline(c, holos.data(), 16, M, vre.data(), vim.data(),
                                export_otf != 0 ? otf.data() : nullptr, nullptr, pos.data()),
                   c, "tdm_pipeline"))
        return 1;
    if (save_fields) {
        std::vector<float> fields((size_t)M * F * F * 2);
        if (app::check(tdm_fields(c, nullptr, M, fields.data(), nullptr), c, "tdm_fields")) return 1;
        const std::string dim = std::to_string(F) + "x" + std::to_string(F) + "x" + std::to_string(M);
        std::vector<double> plane((size_t)M * F * F);
        for (int part = 0; part < 2; ++part) {
            for (size_t i = 0; i < plane.size(); ++i) plane[i] = fields[2 * i + part];
            app::write_f64(P.result + (part ? "UBornfinal_Im" : "UBornfinal_Re") + dim + ".raw", plane.data(),
                           plane.size());
        }
        const double param[5] = {(double)g.nxmax, (double)M, dv.rayon, (double)H, dv.tp_holo};
        std::vector<double> tab(pos.begin(), pos.end());
        app::write_f64(P.result + "parametres.raw", param, 5);
        app::write_f64(P.result + "tab_posSpec.raw", tab.data(), tab.size());
    }
    tdm_destroy(c);
    if (export_otf != 0) {
        std::vector<float> of(NT);
        for (size_t i = 0; i < NT; ++i) of[i] = otf[i];
        tdm_write_tiff_f32((P.result + "OTF3D.tif").c_str(), of.data(), D, D, D, dv.tp_tomo, 4);
    }
    if (tdm_write_tiff_f32((P.result + "indice.tif").c_str(), vre.data(), D, D, D, dv.tp_tomo, 4) != TDM_OK ||
        tdm_write_tiff_f32((P.result + "absorption.tif").c_str(), vim.data(), D, D, D, dv.tp_tomo, 4) != TDM_OK) {
        std::fprintf(stderr, "cannot write the volumes in %s\n", P.result.c_str());
        return 1;
    }
    std::printf("tomo_pipeline: %d holograms -> %d^3 volume in %s\n", M, D, P.result.c_str());
    return 0;
}
