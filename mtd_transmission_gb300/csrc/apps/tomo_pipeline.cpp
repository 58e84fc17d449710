// tomo_pipeline: tomo_pretraitement followed by tomo_reconstruction in one
// pass, the fields staying in GPU memory.  Same inputs as tomo_pretraitement
// and the outputs of tomo_reconstruction in CHEMIN_RESULT; --save-fields also
// writes the UBornfinal_*.raw, parametres.raw and tab_posSpec.raw files.
//
// Polarisation mode: -polar -etat S processes one state (acquisitions in
// CHEMIN_RACINE/demosaic<S>, results in <that>/UBorn/, mask
// CHEMIN_RACINE/Image_mask.pgm, as tomo_pretraitement -polar -etat S reads
// them) and writes the volume as indice_cplx_hdf5.hdf, as tomo_reconstruction
// -polar does.  -polar alone processes the four states (/LC/polar0/,
// /LC/polar90/, /RC/polar0/, /RC/polar90/), whose stacks may differ in size,
// as one CUDA-graph launch (tdm_batch): one branch per state.
#include <cuda_runtime.h>

#include "app_common.h"

namespace {

struct Stack {
    std::string state;
    app::Paths P;
    std::vector<uint16_t> holos;
    int M = 0;
    tdm_ctx* c = nullptr;
};

int write_volume(const std::string& dir, bool polar, const float* re, const float* im, const uint8_t* otf, int D,
                 double tp_tomo) {
    const size_t NT = (size_t)D * D * D;
    if (otf) {
        std::vector<float> of(NT);
        for (size_t i = 0; i < NT; ++i) of[i] = otf[i];
        tdm_write_tiff_f32((dir + "OTF3D.tif").c_str(), of.data(), D, D, D, tp_tomo, 4);
    }
    const int rc = polar ? tdm_write_hdf5_complex((dir + "/indice_cplx_hdf5.hdf").c_str(), re, im, D, D, D)
                         : (tdm_write_tiff_f32((dir + "indice.tif").c_str(), re, D, D, D, tp_tomo, 4) != TDM_OK
                                ? TDM_EIO
                                : tdm_write_tiff_f32((dir + "absorption.tif").c_str(), im, D, D, D, tp_tomo, 4));
    if (rc != TDM_OK) std::fprintf(stderr, "cannot write the volume in %s\n", dir.c_str());
    return rc;
}

bool cuda_ok(cudaError_t e, const char* what) {
    if (e != cudaSuccess) std::fprintf(stderr, "%s: %s\n", what, cudaGetErrorString(e));
    return e == cudaSuccess;
}

// The four states as one CUDA-graph launch.
int four_states(const app::Args& A, const tdm_geom& g, int nb_angle, bool export_otf) {
    const int H = g.ccd_roix, F = 2 * g.nxmax, D = g.dim_final;
    const size_t NT = (size_t)D * D * D;
    std::vector<Stack> st;
    for (const std::string& s : app::polar_states()) {
        Stack k;
        k.state = s;
        app::Args a = A;
        a.etat = s;
        if (!app::read_paths(a, k.P)) return 1;
        k.M = app::read_stack(k.P.acquis, H, nb_angle, k.holos);
        if (k.M <= 0) {
            std::fprintf(stderr, "no hologram read from %s\n", k.P.acquis.c_str());
            return 1;
        }
        st.push_back(std::move(k));
    }
    const int n = (int)st.size();
    std::vector<tdm_ctx*> ctxs(n);
    std::vector<void*> dh(n);
    std::vector<float*> dre(n), dim_(n);
    std::vector<uint8_t*> dotf(n, nullptr);
    std::vector<int> bits(n, 16), cnt(n);
    for (int i = 0; i < n; ++i) {
        Stack& k = st[i];
        if (app::check(tdm_create(&g, k.M, &k.c), k.c, "tdm_create")) return 1;
        if (app::check(app::load_mask(k.c, k.P.mask, F), k.c, "tdm_set_mask")) return 1;
        ctxs[i] = k.c;
        cnt[i] = k.M;
        const size_t hb = k.holos.size() * sizeof(uint16_t);
        if (!cuda_ok(cudaMalloc(&dh[i], hb), "cudaMalloc") ||
            !cuda_ok(cudaMemcpy(dh[i], k.holos.data(), hb, cudaMemcpyHostToDevice), "cudaMemcpy") ||
            !cuda_ok(cudaMalloc(reinterpret_cast<void**>(&dre[i]), NT * sizeof(float)), "cudaMalloc") ||
            !cuda_ok(cudaMalloc(reinterpret_cast<void**>(&dim_[i]), NT * sizeof(float)), "cudaMalloc") ||
            (export_otf && !cuda_ok(cudaMalloc(reinterpret_cast<void**>(&dotf[i]), NT), "cudaMalloc")))
            return 1;
    }
    tdm_batch* b = nullptr;
    if (app::check(tdm_batch_create(n, ctxs.data(), dh.data(), bits.data(), cnt.data(), dre.data(), dim_.data(),
                                    export_otf ? dotf.data() : nullptr, &b),
                   ctxs[0], "tdm_batch_create"))
        return 1;
    if (app::check(tdm_batch_launch(b, nullptr), ctxs[0], "tdm_batch_launch") ||
        !cuda_ok(cudaDeviceSynchronize(), "batch"))
        return 1;
    tdm_batch_destroy(b);
    std::vector<float> re(NT), im(NT);
    std::vector<uint8_t> otf(export_otf ? NT : 0);
    for (int i = 0; i < n; ++i) {
        Stack& k = st[i];
        if (app::check(tdm_synchronize(k.c), k.c, "tdm_synchronize")) return 1;
        tdm_derived dv;
        tdm_get_derived(k.c, &dv);
        if (!cuda_ok(cudaMemcpy(re.data(), dre[i], NT * sizeof(float), cudaMemcpyDeviceToHost), "cudaMemcpy") ||
            !cuda_ok(cudaMemcpy(im.data(), dim_[i], NT * sizeof(float), cudaMemcpyDeviceToHost), "cudaMemcpy") ||
            (export_otf && !cuda_ok(cudaMemcpy(otf.data(), dotf[i], NT, cudaMemcpyDeviceToHost), "cudaMemcpy")))
            return 1;
        if (write_volume(k.P.result, true, re.data(), im.data(), export_otf ? otf.data() : nullptr, D, dv.tp_tomo))
            return 1;
        std::printf("tomo_pipeline: %s %d holograms -> %d^3 volume in %s\n", k.state.c_str(), k.M, D,
                    k.P.result.c_str());
        tdm_destroy(k.c);
        cudaFree(dh[i]);
        cudaFree(dre[i]);
        cudaFree(dim_[i]);
        if (dotf[i]) cudaFree(dotf[i]);
    }
    return 0;
}

}  // namespace

int main(int argc, char** argv) {
    const app::Args A = app::parse_args(argc, argv);
    if (A.help) {
        app::print_help("tomo_pipeline");
        return 0;
    }
    bool save_fields = false;
    for (const std::string& r : A.rest)
        if (r == "--save-fields") save_fields = true;
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
    double nb_holo = 0, premier = 0, export_otf = 1;
    tdm_extract_val(manip.c_str(), "NB_HOLO", 0, &nb_holo);
    tdm_extract_val(recon.c_str(), "PREMIER_ANGLE", 0, &premier);
    tdm_extract_val(recon.c_str(), "EXPORT_OTF", 1, &export_otf);
    const int nb_angle = (int)nb_holo - (int)premier;
    if (A.polar && A.etat.empty()) return four_states(A, g, nb_angle, export_otf != 0);
    const int H = g.ccd_roix, F = 2 * g.nxmax, D = g.dim_final;
    std::vector<uint16_t> holos;
    const int M = app::read_stack(P.acquis, H, nb_angle, holos);
    if (M <= 0) {
        std::fprintf(stderr, "no hologram read from %s\n", P.acquis.c_str());
        return 1;
    }
    tdm_ctx* c = nullptr;
    if (app::check(tdm_create(&g, M, &c), c, "tdm_create")) return 1;
    if (app::check(app::load_mask(c, P.mask, F), c, "tdm_set_mask")) return 1;
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
    if (write_volume(P.result, A.polar, vre.data(), vim.data(), export_otf != 0 ? otf.data() : nullptr, D,
                     dv.tp_tomo))
        return 1;
    std::printf("tomo_pipeline: %d holograms -> %d^3 volume in %s\n", M, D, P.result.c_str());
    return 0;
}
