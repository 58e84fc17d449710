// Host-side file contracts of the reference programs: KEY value configuration
// files, PGM holograms, raw binary fields and float32 multi-page TIFF volumes.
#include <cctype>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <string>
#include <vector>

#include "../../include/tdm.h"

namespace {

// Lines of a config file without '#' comment lines (IO_fonctions.cpp:88-95).
bool read_lines(const char* path, std::vector<std::string>& lines) {
    std::ifstream f(path);
    if (!f) return false;
    std::string l;
    while (std::getline(f, l)) {
        if (!l.empty() && l[0] == '#') continue;
        lines.push_back(l);
    }
    return true;
}

// Key is the text before the first space; value is the rest of the line.
// The last matching line wins (IO_fonctions.cpp:100-112).
bool find_key(const std::vector<std::string>& lines, const char* key, std::string& value) {
    bool found = false;
    for (const std::string& l : lines) {
        if (l.empty()) continue;
        const size_t pos = l.find(' ');
        const std::string k = l.substr(0, pos);
        if (k == key) {
            value = (pos == std::string::npos) ? l : l.substr(pos + 1);
            found = true;
        }
    }
    return found;
}

void put16(std::vector<uint8_t>& b, size_t at, uint16_t v) {
    b[at] = v & 0xff;
    b[at + 1] = v >> 8;
}
void put32(std::vector<uint8_t>& b, size_t at, uint32_t v) {
    for (int i = 0; i < 4; ++i) b[at + i] = (v >> (8 * i)) & 0xff;
}
void put64(std::vector<uint8_t>& b, size_t at, uint64_t v) {
    for (int i = 0; i < 8; ++i) b[at + i] = (v >> (8 * i)) & 0xff;
}

// Rational approximation of a positive float (resolution tags).
void to_rational(double v, uint32_t& num, uint32_t& den) {
    den = 1;
    while (v * den < 1e8 && den < 100000000u && std::fabs(v * den - std::round(v * den)) > 1e-9 * v * den) den *= 10;
    const double n = std::round(v * den);
    num = n > 4294967295.0 ? 4294967295u : (uint32_t)n;
}

}  // namespace

extern "C" {

int tdm_extract_val(const char* path, const char* key, double def, double* out) {
    if (!path || !key || !out) return TDM_EINVAL;
    std::vector<std::string> lines;
    if (!read_lines(path, lines)) {
        *out = def;
        return TDM_EIO;
    }
    std::string v;
    if (!find_key(lines, key, v)) {
        *out = def;
        return 0;
    }
    *out = (double)(float)std::atof(v.c_str());  // extract_val returns float
    return 1;
}

int tdm_extract_string(const char* path, const char* key, char* out, size_t cap) {
    if (!path || !key || !out || cap == 0) return TDM_EINVAL;
    std::vector<std::string> lines;
    out[0] = 0;
    if (!read_lines(path, lines)) return TDM_EIO;
    std::string v;
    if (!find_key(lines, key, v)) return 0;
    while (!v.empty() && (v.back() == '\r' || v.back() == ' ' || v.back() == '\t')) v.pop_back();
    std::snprintf(out, cap, "%s", v.c_str());
    return 1;
}

int tdm_read_geom(const char* recon, const char* manip, tdm_geom* g) {
    if (!recon || !manip || !g) return TDM_EINVAL;
    std::vector<std::string> lr, lm;
    if (!read_lines(recon, lr) || !read_lines(manip, lm)) return TDM_EIO;
    auto val = [](const std::vector<std::string>& ls, const char* k, double def) {
        std::string v;
        if (!find_key(ls, k, v)) return def;
        return (double)(float)std::atof(v.c_str());
    };
    *g = tdm_geom{};
    g->ccd_roix = (int)val(lr, "CCD_ROIX", 0);
    g->deroul = val(lr, "DEROUL", 0) != 0;
    g->volkov = val(lr, "VOLKOV", 0) != 0;
    g->c_aber = val(lr, "C_ABER", 0) != 0;
    g->born = val(lr, "BORN", 0) != 0;
    g->dim_final = (int)val(lr, "DIM_FINAL", 0);
    g->coef_na_obj_limit = val(lr, "COEF_NA_OBJ_LIMIT", 1.0);
    g->na = val(lm, "NA", 0);
    g->n0 = val(lm, "N0", 0);
    g->lambda0 = val(lm, "LAMBDA", 0);
    g->f_tube = val(lm, "F_TUBE", 0);
    g->f_obj = val(lm, "F_OBJ", 0);
    g->tpcam = val(lm, "TPCAM", 0);
    g->rf = val(lm, "RF", 0);
    g->nxmax = (int)val(lm, "NXMAX", 0);
    g->circle_cx = (int)val(lm, "CIRCLE_CX", 0);
    g->circle_cy = (int)val(lm, "CIRCLE_CY", 0);
    return TDM_OK;
}

int tdm_pgm_info(const char* path, int* width, int* height, int* maxval) {
    FILE* f = std::fopen(path, "rb");
    if (!f) return TDM_EIO;
    char magic[3] = {0, 0, 0};
    if (std::fread(magic, 1, 2, f) != 2 || magic[0] != 'P' || (magic[1] != '5' && magic[1] != '2')) {
        std::fclose(f);
        return TDM_EIO;
    }
    int vals[3], got = 0;
    while (got < 3) {
        int ch = std::fgetc(f);
        if (ch == EOF) break;
        if (ch == '#') {
            while (ch != '\n' && ch != EOF) ch = std::fgetc(f);
            continue;
        }
        if (std::isspace(ch)) continue;
        long v = 0;
        while (ch != EOF && std::isdigit(ch)) {
            v = v * 10 + (ch - '0');
            ch = std::fgetc(f);
        }
        vals[got++] = (int)v;
    }
    std::fclose(f);
    if (got < 3 || vals[0] <= 0 || vals[1] <= 0 || vals[2] <= 0 || vals[2] > 65535) return TDM_EIO;
    if (width) *width = vals[0];
    if (height) *height = vals[1];
    if (maxval) *maxval = vals[2];
    return TDM_OK;
}

int tdm_read_pgm(const char* path, int roi, void* buf, int* bits) {
    if (!path || !buf || roi <= 0) return TDM_EINVAL;
    FILE* f = std::fopen(path, "rb");
    if (!f) return TDM_EIO;
    char magic[2];
    if (std::fread(magic, 1, 2, f) != 2 || magic[0] != 'P' || (magic[1] != '5' && magic[1] != '2')) {
        std::fclose(f);
        return TDM_EIO;
    }
    const bool ascii = magic[1] == '2';
    int vals[3], got = 0, ch = 0;
    while (got < 3) {
        ch = std::fgetc(f);
        if (ch == EOF) break;
        if (ch == '#') {
            while (ch != '\n' && ch != EOF) ch = std::fgetc(f);
            continue;
        }
        if (std::isspace(ch)) continue;
        long v = 0;
        while (ch != EOF && std::isdigit(ch)) {
            v = v * 10 + (ch - '0');
            ch = std::fgetc(f);
        }
        vals[got++] = (int)v;
    }
    // ch holds the single whitespace after maxval
    const int w = vals[0], h = vals[1], mx = vals[2];
    if (got < 3 || w < roi || h < roi || mx <= 0 || mx > 65535) {
        std::fclose(f);
        return TDM_EIO;
    }
    const int b = mx < 256 ? 8 : 16;
    if (bits) *bits = b;
    const size_t bps = b / 8;
    std::vector<uint8_t> row((size_t)w * bps);
    for (int y = 0; y < roi; ++y) {
        if (ascii) {
            for (int x = 0; x < w; ++x) {
                long v;
                if (std::fscanf(f, "%ld", &v) != 1) {
                    std::fclose(f);
                    return TDM_EIO;
                }
                if (x < roi) {
                    if (b == 8) static_cast<uint8_t*>(buf)[(size_t)y * roi + x] = (uint8_t)v;
                    else static_cast<uint16_t*>(buf)[(size_t)y * roi + x] = (uint16_t)v;
                }
            }
            continue;
        }
        if (std::fread(row.data(), 1, row.size(), f) != row.size()) {
            std::fclose(f);
            return TDM_EIO;
        }
        if (b == 8) {
            std::memcpy(static_cast<uint8_t*>(buf) + (size_t)y * roi, row.data(), roi);
        } else {
            uint16_t* o = static_cast<uint16_t*>(buf) + (size_t)y * roi;
            for (int x = 0; x < roi; ++x) o[x] = (uint16_t)((row[2 * x] << 8) | row[2 * x + 1]);  // big-endian
        }
    }
    std::fclose(f);
    return TDM_OK;
}

int tdm_write_tiff_f32(const char* path, const float* vol, int wdt, int hgt, int pages, double pixel_size,
                       int orientation) {
    if (!path || !vol || wdt <= 0 || hgt <= 0 || pages <= 0) return TDM_EINVAL;
    FILE* f = std::fopen(path, "wb");
    if (!f) return TDM_EIO;
    const uint64_t page_bytes = (uint64_t)wdt * hgt * 4;
    const bool big = page_bytes * pages + (uint64_t)pages * 512 > 0xFFFF0000ull;  // BigTIFF beyond 4 GB
    const double res = 0.01f / (float)pixel_size;  // pixels per cm (fonctions.cpp:2299)
    uint32_t rn, rd;
    to_rational(res, rn, rd);
    const int ntag = 17;
    const size_t esz = big ? 20 : 12, cntsz = big ? 8 : 2, nxtsz = big ? 8 : 4;
    const size_t ifd_size = cntsz + ntag * esz + nxtsz + 16;  // + two rationals
    std::vector<uint8_t> hdr(big ? 16 : 8, 0);
    hdr[0] = 'I';
    hdr[1] = 'I';
    if (big) {
        put16(hdr, 2, 43);
        put16(hdr, 4, 8);
        put16(hdr, 6, 0);
        put64(hdr, 8, hdr.size());
    } else {
        put16(hdr, 2, 42);
        put32(hdr, 4, (uint32_t)hdr.size());
    }
    if (std::fwrite(hdr.data(), 1, hdr.size(), f) != hdr.size()) {
        std::fclose(f);
        return TDM_EIO;
    }
    uint64_t off = hdr.size();
    for (int z = 0; z < pages; ++z) {
        const uint64_t ifd_off = off, data_off = ifd_off + ifd_size;
        const uint64_t next = (z + 1 < pages) ? data_off + page_bytes : 0;
        std::vector<uint8_t> d(ifd_size, 0);
        size_t at = 0;
        if (big) put64(d, at, ntag); else put16(d, at, ntag);
        at += cntsz;
        const uint64_t rat_off = ifd_off + cntsz + ntag * esz + nxtsz;
        auto tag = [&](uint16_t id, uint16_t type, uint64_t count, uint64_t value) {
            put16(d, at, id);
            put16(d, at + 2, type);
            if (big) {
                put64(d, at + 4, count);
                put64(d, at + 12, value);
            } else {
                put32(d, at + 4, (uint32_t)count);
                put32(d, at + 8, (uint32_t)value);
            }
            at += esz;
        };
        const uint16_t SHORT = 3, LONG = 4, RATIONAL = 5, LONG8 = 16;
        tag(254, LONG, 1, 2);                                       // NewSubfileType: page
        tag(256, LONG, 1, (uint32_t)wdt);                           // ImageWidth
        tag(257, LONG, 1, (uint32_t)hgt);                           // ImageLength
        tag(258, SHORT, 1, 32);                                     // BitsPerSample
        tag(259, SHORT, 1, 1);                                      // Compression: none
        tag(262, SHORT, 1, 1);                                      // Photometric: min-is-black
        tag(273, big ? LONG8 : LONG, 1, data_off);                  // StripOffsets
        tag(274, SHORT, 1, (uint16_t)orientation);                  // Orientation
        tag(277, SHORT, 1, 1);                                      // SamplesPerPixel
        tag(278, LONG, 1, (uint32_t)hgt);                           // RowsPerStrip
        tag(279, big ? LONG8 : LONG, 1, page_bytes);                // StripByteCounts
        tag(282, RATIONAL, 1, rat_off);                             // XResolution
        tag(283, RATIONAL, 1, rat_off + 8);                         // YResolution
        tag(284, SHORT, 1, 1);                                      // PlanarConfig: contiguous
        tag(285, SHORT, 2, (uint32_t)z | ((uint32_t)pages << 16));  // PageNumber
        tag(296, SHORT, 1, 3);                                      // ResolutionUnit: cm
        tag(339, SHORT, 1, 3);                                      // SampleFormat: IEEE float
        if (big) put64(d, at, next); else put32(d, at, (uint32_t)next);
        at += nxtsz;
        put32(d, at, rn);
        put32(d, at + 4, rd);
        put32(d, at + 8, rn);
        put32(d, at + 12, rd);
        if (std::fwrite(d.data(), 1, d.size(), f) != d.size() ||
            std::fwrite(vol + (size_t)z * wdt * hgt, 4, (size_t)wdt * hgt, f) != (size_t)wdt * hgt) {
            std::fclose(f);
            return TDM_EIO;
        }
        off = data_off + page_bytes;
    }
    return std::fclose(f) == 0 ? TDM_OK : TDM_EIO;
}

}  // extern "C"
