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

// ---------------------------------------------------------------- HDF5
// A minimal HDF5 file (format specification, superblock version 0) holding
// the polarisation mode's volume as save_complex_volume_hdf5 writes it
// (Reconstruction/src/IO_functions.cpp:52-82): group "/indice_complexe" with
// the float32 datasets "Re" and "Im" of dimensions (Nz, Ny, Nx).  Offsets and
// lengths are 8 bytes; groups are symbol tables (a version-1 B-tree of group
// nodes, one symbol table node, a local heap of names); dataset object
// headers (version 1) carry the dataspace, datatype (IEEE float32, little
// endian), fill-value (version 2, undefined) and contiguous layout (version 3)
// messages; the raw data follow the metadata.
namespace {

constexpr uint64_t kUndef = ~0ull;
constexpr int kGroupLeafK = 4, kGroupNodeK = 16;

struct H5Buf {
    std::vector<uint8_t> b;
    size_t pos() const { return b.size(); }
    void u8(uint32_t v) { b.push_back((uint8_t)v); }
    void u16(uint32_t v) { for (int i = 0; i < 2; ++i) b.push_back((uint8_t)(v >> (8 * i))); }
    void u32(uint32_t v) { for (int i = 0; i < 4; ++i) b.push_back((uint8_t)(v >> (8 * i))); }
    void u64(uint64_t v) { for (int i = 0; i < 8; ++i) b.push_back((uint8_t)(v >> (8 * i))); }
    void bytes(const char* s, size_t n) { b.insert(b.end(), s, s + n); }
    void zeros(size_t n) { b.insert(b.end(), n, 0); }
    void align8() { while (b.size() % 8) b.push_back(0); }
    void put64(size_t at, uint64_t v) { for (int i = 0; i < 8; ++i) b[at + i] = (uint8_t)(v >> (8 * i)); }
};

// Version-1 object header with the given messages (type, data); returns its address.
size_t h5_object_header(H5Buf& f, const std::vector<std::pair<int, std::vector<uint8_t>>>& msgs) {
    f.align8();
    const size_t at = f.pos();
    size_t body = 0;
    for (const auto& m : msgs) body += 8 + ((m.second.size() + 7) & ~size_t(7));
    f.u8(1);                        // version
    f.u8(0);                        // reserved
    f.u16((uint32_t)msgs.size());   // number of header messages
    f.u32(1);                       // object reference count
    f.u32((uint32_t)body);          // object header size
    f.u32(0);                       // alignment of the messages to 8 bytes
    for (const auto& m : msgs) {
        const size_t n = (m.second.size() + 7) & ~size_t(7);
        f.u16((uint32_t)m.first);
        f.u16((uint32_t)n);
        f.u8(0);                    // flags
        f.zeros(3);
        f.b.insert(f.b.end(), m.second.begin(), m.second.end());
        f.zeros(n - m.second.size());
    }
    return at;
}

// Symbol table entry (link name offset, object header address, cache type, scratch).
void h5_entry(H5Buf& f, uint64_t name_off, uint64_t ohdr, uint32_t cache, uint64_t btree = 0, uint64_t heap = 0) {
    f.u64(name_off);
    f.u64(ohdr);
    f.u32(cache);
    f.u32(0);
    f.u64(btree);
    f.u64(heap);
}

struct H5Group {
    size_t heap = 0, btree = 0, snod = 0;
    std::vector<uint64_t> name_off;  // heap offsets of the members' names, in the order given
};

// Local heap of the member names ("" at offset 0), the B-tree with one child
// and the symbol table node; member object header addresses are patched in
// later through snod_entry_at().  names must be in ascending order.
H5Group h5_group_tables(H5Buf& f, const std::vector<std::string>& names) {
    H5Group g;
    std::vector<uint8_t> data(8, 0);  // offset 0: the empty name
    for (const auto& n : names) {
        g.name_off.push_back(data.size());
        data.insert(data.end(), n.begin(), n.end());
        data.push_back(0);
        while (data.size() % 8) data.push_back(0);
    }
    f.align8();
    g.heap = f.pos();
    f.bytes("HEAP", 4);
    f.u8(0);
    f.zeros(3);
    f.u64(data.size());      // data segment size
    f.u64(1);                // free list: none (1 ends a free list; the reference HDF5 library writes it for an empty list)
    f.u64(f.pos() + 8);      // data segment address: right after this field
    f.b.insert(f.b.end(), data.begin(), data.end());
    f.align8();
    g.btree = f.pos();
    f.bytes("TREE", 4);
    f.u8(0);                 // group nodes
    f.u8(0);                 // leaf level
    f.u16(1);                // entries used
    f.u64(kUndef);           // left sibling
    f.u64(kUndef);           // right sibling
    f.u64(0);                // key 0: the empty name
    const size_t child = f.pos();
    f.u64(0);                // child 0: the symbol table node (patched below)
    f.u64(g.name_off.empty() ? 0 : g.name_off.back());  // key 1: the last name
    f.zeros((size_t)(2 * kGroupNodeK - 1) * 16);        // unused keys and children of the node
    f.align8();
    g.snod = f.pos();
    f.put64(child, g.snod);
    f.bytes("SNOD", 4);
    f.u8(1);
    f.u8(0);
    f.u16((uint32_t)names.size());
    for (size_t i = 0; i < names.size(); ++i) h5_entry(f, g.name_off[i], 0, 0);
    f.zeros((size_t)(2 * kGroupLeafK - names.size()) * 40);
    return g;
}

size_t snod_entry_at(const H5Group& g, size_t i) { return g.snod + 8 + i * 40; }

std::vector<uint8_t> h5_msg_symbol_table(uint64_t btree, uint64_t heap) {
    H5Buf m;
    m.u64(btree);
    m.u64(heap);
    return m.b;
}

}  // namespace

extern "C" int tdm_write_hdf5_complex(const char* path, const float* re, const float* im, int nx, int ny, int nz) {
    if (!path || !re || !im || nx <= 0 || ny <= 0 || nz <= 0) return TDM_EINVAL;
    const uint64_t n = (uint64_t)nx * ny * nz, bytes = n * 4;
    H5Buf f;
    // superblock (version 0), root entry patched below
    f.bytes("\x89HDF\r\n\x1a\n", 8);
    f.u8(0); f.u8(0); f.u8(0); f.u8(0);   // superblock, free space, root entry, reserved
    f.u8(0); f.u8(8); f.u8(8); f.u8(0);   // shared header version, sizeof offsets, sizeof lengths, reserved
    f.u16(kGroupLeafK);
    f.u16(kGroupNodeK);
    f.u32(0);                             // file consistency flags
    f.u64(0);                             // base address
    f.u64(kUndef);                        // free-space info
    const size_t eof_at = f.pos();
    f.u64(0);                             // end of file address (patched)
    f.u64(kUndef);                        // driver information block
    const size_t root_entry = f.pos();
    h5_entry(f, 0, 0, 1);                 // patched below
    // root group: one member, "indice_complexe"
    const H5Group root = h5_group_tables(f, {"indice_complexe"});
    const size_t root_oh = h5_object_header(f, {{0x0011, h5_msg_symbol_table(root.btree, root.heap)}});
    // the group "/indice_complexe": members "Im", "Re" (ascending)
    const H5Group grp = h5_group_tables(f, {"Im", "Re"});
    const size_t grp_oh = h5_object_header(f, {{0x0011, h5_msg_symbol_table(grp.btree, grp.heap)}});
    // the two datasets
    H5Buf space, type, fill;
    space.u8(1); space.u8(3); space.u8(0); space.u8(0); space.u32(0);  // version 1, rank 3, no max dims
    space.u64((uint64_t)nz); space.u64((uint64_t)ny); space.u64((uint64_t)nx);
    type.u8(0x11);                        // version 1, class 1 (floating point)
    type.u8(0x20); type.u8(31); type.u8(0);  // little endian, implied mantissa msb, sign at bit 31
    type.u32(4);                          // size
    type.u16(0); type.u16(32);            // bit offset, precision
    type.u8(23); type.u8(8); type.u8(0); type.u8(23);  // exponent location and size, mantissa location and size
    type.u32(127);                        // exponent bias
    fill.u8(2); fill.u8(1); fill.u8(1); fill.u8(0);  // version 2, early allocation, never written, undefined
    auto layout = [&](uint64_t addr) {
        H5Buf l;
        l.u8(3); l.u8(1);                 // version 3, contiguous
        l.u64(addr);
        l.u64(bytes);
        return l.b;
    };
    std::vector<size_t> ds_oh(2), layout_at(2);
    for (int k = 0; k < 2; ++k) {  // 0: Im, 1: Re
        ds_oh[k] = h5_object_header(f, {{0x0001, space.b}, {0x0003, type.b}, {0x0005, fill.b}, {0x0008, layout(0)}});
        // the layout message is the last one: its address field follows 4 header messages
        layout_at[k] = f.pos() - 24 + 2;
    }
    f.align8();
    const uint64_t data_im = f.pos(), data_re = data_im + bytes, eof = data_re + bytes;
    f.put64(layout_at[0], data_im);
    f.put64(layout_at[1], data_re);
    f.put64(eof_at, eof);
    // patch the entries: root entry, root member, group members
    f.put64(root_entry + 8, root_oh);
    f.put64(root_entry + 24, root.btree);
    f.put64(root_entry + 32, root.heap);
    const size_t e0 = snod_entry_at(root, 0);
    f.put64(e0 + 8, grp_oh);
    f.b[e0 + 16] = 1;                     // cache type 1: the group's B-tree and heap
    f.put64(e0 + 24, grp.btree);
    f.put64(e0 + 32, grp.heap);
    f.put64(snod_entry_at(grp, 0) + 8, ds_oh[0]);
    f.put64(snod_entry_at(grp, 1) + 8, ds_oh[1]);
    FILE* fp = std::fopen(path, "wb");
    if (!fp) return TDM_EIO;
    bool ok = std::fwrite(f.b.data(), 1, f.b.size(), fp) == f.b.size();
    ok = ok && std::fwrite(im, 4, n, fp) == n && std::fwrite(re, 4, n, fp) == n;
    return std::fclose(fp) == 0 && ok ? TDM_OK : TDM_EIO;
}
