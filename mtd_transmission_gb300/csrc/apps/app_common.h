// Shared helpers of the drop-in executables: command line, configuration
// path indirection and the raw binary files of the reference programs.
#pragma once

#include <sys/stat.h>

#include <cmath>
#include <complex>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "tdm.h"

namespace app {

struct Paths {
    std::string config, result, acquis, racine, mask;
};

// Command line of pretraitement_hors_axe_CPU/main.cpp:37-61 and
// Reconstruction/main.cpp:63-86: "-polar" (polarisation mode), "-etat S" (one
// of the four states /LC/polar0/, /LC/polar90/, /RC/polar0/, /RC/polar90/),
// "--help".  Either option selects $HOME/.config/gui_tomo_polar.conf; as in
// the reference, any other argument selects gui_tomo.conf again.
struct Args {
    bool help = false, polar = false;
    std::string etat, gui = "gui_tomo.conf";
    std::vector<std::string> rest;
};

inline Args parse_args(int argc, char** argv) {
    Args a;
    for (int i = 1; i < argc; ++i) {
        const std::string s = argv[i];
        if (s == "--help") {
            a.help = true;
        } else if (s == "-polar") {
            a.polar = true;
            a.gui = "gui_tomo_polar.conf";
        } else if (s == "-etat" && i + 1 < argc) {
            a.etat = argv[++i];
            a.gui = "gui_tomo_polar.conf";
        } else {
            a.gui = "gui_tomo.conf";
            a.rest.push_back(s);
        }
    }
    return a;
}

inline void print_help(const char* prog) {
    std::printf("%s (GB300)\n-polar : mode polar\n-etat : indiquez un des 4 etats :\n/LC/polar0/\n/LC/polar90/\n"
                "/RC/polar0/\n/RC/polar90/\n", prog);
}

inline std::string gui_key(const std::string& gui, const char* key) {
    char buf[4096];
    return tdm_extract_string(gui.c_str(), key, buf, sizeof buf) == 1 ? std::string(buf) : std::string();
}

// Paths of the preprocessing (pretraitement_hors_axe_CPU/manip.cpp:14-29,
// main.cpp:63-80): in polarisation mode the acquisitions are
// CHEMIN_RACINE/demosaic<etat>, the results <that>/UBorn/ and the mask
// CHEMIN_RACINE/Image_mask.pgm.
inline bool read_paths(const Args& a, Paths& p) {
    const char* home = std::getenv("HOME");
    if (!home) return false;
    const std::string gui = std::string(home) + "/.config/" + a.gui;
    p.config = gui_key(gui, "CHEMIN_CONFIG");
    if (p.config.empty()) return false;
    p.result = gui_key(gui, "CHEMIN_RESULT") + "/";
    p.acquis = gui_key(gui, "CHEMIN_ACQUIS") + "/";
    p.racine = gui_key(gui, "CHEMIN_RACINE") + "/";
    if (a.polar) {
        p.acquis = p.racine + "demosaic" + a.etat + "/";
        p.result = p.racine + "demosaic" + a.etat + "/UBorn/";
        p.mask = p.racine + "Image_mask.pgm";
    } else {
        p.mask = p.acquis + "Image_mask.pgm";
    }
    return true;
}

// Paths of the reconstruction (Reconstruction/src/manip.cpp:10-30): in
// polarisation mode the configuration files and the results are both in
// CHEMIN_RACINE/demosaic/<etat>UBorn/.
inline bool read_paths_recon(const Args& a, Paths& p) {
    const char* home = std::getenv("HOME");
    if (!home) return false;
    const std::string gui = std::string(home) + "/.config/" + a.gui;
    p.acquis = gui_key(gui, "CHEMIN_ACQUIS");
    if (a.polar) {
        p.racine = gui_key(gui, "CHEMIN_RACINE");
        p.config = p.racine + "/demosaic/" + a.etat + "UBorn/";
        p.result = p.config;
    } else {
        p.result = gui_key(gui, "CHEMIN_RESULT") + "/";
        p.config = gui_key(gui, "CHEMIN_CONFIG");
        if (p.config.empty()) return false;
    }
    return true;
}

// The four states of the polarisation set-up (pretraitement_hors_axe_CPU/main.cpp:42-46).
inline std::vector<std::string> polar_states() { return {"/LC/polar0/", "/LC/polar90/", "/RC/polar0/", "/RC/polar90/"}; }

inline bool file_exists(const std::string& f) {
    struct stat st;
    return stat(f.c_str(), &st) == 0;
}

inline long file_size(const std::string& f) {
    struct stat st;
    return stat(f.c_str(), &st) == 0 ? (long)st.st_size : -1;
}

// FP64 little-endian writer (SAV2 / SAVCplx with t_double, src/IO_fonctions.cpp:120-220).
inline bool write_f64(const std::string& f, const double* v, size_t n, const char* mode = "wb") {
    FILE* fp = std::fopen(f.c_str(), mode);
    if (!fp) return false;
    const bool ok = std::fwrite(v, sizeof(double), n, fp) == n;
    return std::fclose(fp) == 0 && ok;
}

// lire_bin (Reconstruction/src/fonctions.cpp:1810-1842): reads the whole file;
// a size mismatch is reported, an unreadable file is fatal.
inline bool read_f64(const std::string& f, std::vector<double>& v, size_t expect) {
    const long sz = file_size(f);
    if (sz < 0) {
        std::fprintf(stderr, "Impossible d'ouvrir le fichier %s\n", f.c_str());
        return false;
    }
    if ((size_t)sz != expect * 8)
        std::fprintf(stderr, "Taille du fichier %s incompatible avec les dimensions\n", f.c_str());
    v.assign(std::max<size_t>(expect, (size_t)sz / 8), 0.0);
    FILE* fp = std::fopen(f.c_str(), "rb");
    if (!fp) return false;
    const size_t got = std::fread(v.data(), 1, (size_t)sz, fp);
    std::fclose(fp);
    v.resize(expect);
    return got == (size_t)sz;
}

// First loop of tomo_pretraitement (pretraitement_hors_axe_CPU/main.cpp:130-165):
// i%03d.pgm for a in [0, nb_angle); missing files are skipped.  8-bit samples
// are widened to uint16.  Returns the number of holograms read, -1 on error.
inline int read_stack(const std::string& dir, int H, int nb_angle, std::vector<uint16_t>& holos) {
    int ok = 0;
    char name[64];
    std::vector<uint16_t> tmp((size_t)H * H);
    for (int a = 0; a < nb_angle; ++a) {
        std::snprintf(name, sizeof name, "i%03d.pgm", a);
        const std::string f = dir + name;
        if (!file_exists(f)) {
            std::printf("fichier %d inexistant\n", a);
            continue;
        }
        int bits = 0;
        if (tdm_read_pgm(f.c_str(), H, tmp.data(), &bits) != TDM_OK) {
            std::fprintf(stderr, "Impossible d'ouvrir %s\n", f.c_str());
            return -1;
        }
        if (bits == 8) {  // widen in place, from the end
            const uint8_t* b8 = reinterpret_cast<const uint8_t*>(tmp.data());
            for (size_t i = (size_t)H * H; i-- > 0;) tmp[i] = b8[i];
        }
        holos.insert(holos.end(), tmp.begin(), tmp.end());
        ++ok;
    }
    return ok;
}

// Image_mask.pgm (Correction_aberration.cpp:43-70): unit mask when absent.
inline int load_mask(tdm_ctx* c, const std::string& path, int F) {
    std::vector<uint8_t> mask((size_t)F * F);
    int mb = 0, mw = 0, mh = 0, mmax = 0;
    if (file_exists(path) && tdm_pgm_info(path.c_str(), &mw, &mh, &mmax) == TDM_OK && mmax < 256 && mw >= F &&
        mh >= F && tdm_read_pgm(path.c_str(), F, mask.data(), &mb) == TDM_OK)
        return tdm_set_mask(c, mask.data());
    std::printf("Masque : %s non trouve, masque unite\n", path.c_str());
    return TDM_OK;
}

inline int check(int rc, tdm_ctx* c, const char* what) {
    if (rc != TDM_OK) std::fprintf(stderr, "%s failed (%d): %s\n", what, rc, c ? tdm_last_error(c) : "");
    return rc;
}

}  // namespace app
